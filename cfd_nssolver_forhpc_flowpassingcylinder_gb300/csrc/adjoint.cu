// Discrete adjoint of the FP64 projection step (reverse mode, hand-written).
//
// Forward step n (reference order, src/RUN_CPU.cpp:257-436) on the state U^n (T0 after
// the ghost fill):
//   u*  = CD(U^n) on interior faces; T1's ghost and last-face values are copies of U^n
//   b   = -(1/dt) div(u*)                       (n > 1)
//   x   = A^+ b  (p^n on the interior)          (n > 1; p^1 = initial p)
//   U~  = (1 - eta_f)(u* - dt grad p^n)          on the faces update_UandF writes
//   Cd^n = (2 / (lz dt)) sum eta_f (u* - dt dp/dx) dV   (x faces)
//   U^{n+1} = BC(U~; inlet)
// The adjoint of each piece, in reverse: BC^T (phases z, y, x: the reverse of the forward
// order), correction^T (with dCd/d and d/d eta), the Poisson solve (A is symmetric on a
// uniform grid, and the Jacobi-scaled system has the same solution, so lambda_b =
// A^+ lambda_x for both solvers), RHS^T, and CD^T, the transposed QUICK stencil with the
// upwind branches of the forward state held fixed (the scheme is piecewise linear in the
// transported field and bilinear in the face velocities).  CD^T scatters with FP64
// atomics (one per target and thread: a thread sums its contributions per target first);
// every other kernel gathers.  Divisions by the metrics are multiplications by their
// reciprocal tables (RN(1/D)) and the DFIB face factors come from their table: the
// transpose holds to an ulp per term, and the FP64 pipe is spared the division sequence.
#include <algorithm>

#include "cfdgb_internal.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace cfdgb {

#define ROWS(g) \
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < (g).ncell; row += (long long)gridDim.x * kBlock)

// ---- BC^T: transpose of the velocity part of k_bc_x/y/z --------------------------------
// A write dst = a + s * src (chains dst1 = dst2 = ... = a + s * src) has adjoint
// lam[src] += s * sum(lam[dst]); lam[dst] = 0.  Within a phase a thread owns one line.
__global__ void __launch_bounds__(kBlock) k_adj_bc_x(Geo g, BcTable t, double *lu, double *lv, double *lw,
                                                     double *linlet) {
  const int nyc = g.nyc, nzc = g.nzc, nx = g.nx;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nyc * nzc; q += gridDim.x * kBlock) {
    const int j = q / nzc + 2, k = q % nzc + 2;
    auto I = [&](int i) { return pidx(g, i, j, k); };
    // face x+ (BC_1)
    double s = lu[I(nx - 1)] + lu[I(nx - 2)] + lu[I(nx - 3)];
    lu[I(nx - 1)] = lu[I(nx - 2)] = lu[I(nx - 3)] = 0.0;
    lu[I(nx - 4)] += t.num[1][0] * s;
    s = lv[I(nx - 1)] + lv[I(nx - 2)];
    lv[I(nx - 1)] = lv[I(nx - 2)] = 0.0;
    lv[I(nx - 3)] += (2.0 * t.num[1][1] - 1.0) * s;
    s = lw[I(nx - 1)] + lw[I(nx - 2)];
    lw[I(nx - 1)] = lw[I(nx - 2)] = 0.0;
    lw[I(nx - 3)] += (2.0 * t.num[1][2] - 1.0) * s;
    // face x- (BC_0): u ghosts = inlet + num * u[2]
    s = lu[I(0)] + lu[I(1)];
    lu[I(0)] = lu[I(1)] = 0.0;
    if (linlet) linlet[q] += s;
    lu[I(2)] += t.num[0][0] * s;
    s = lv[I(0)] + lv[I(1)];
    lv[I(0)] = lv[I(1)] = 0.0;
    lv[I(2)] += (2.0 * t.num[0][1] - 1.0) * s;
    s = lw[I(0)] + lw[I(1)];
    lw[I(0)] = lw[I(1)] = 0.0;
    lw[I(2)] += (2.0 * t.num[0][2] - 1.0) * s;
  }
}

__global__ void __launch_bounds__(kBlock) k_adj_bc_y(Geo g, BcTable t, double *lu, double *lv, double *lw) {
  const int nxc = g.nxc, nzc = g.nzc, ny = g.ny;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nxc * nzc; q += gridDim.x * kBlock) {
    const int i = q / nzc + 2, k = q % nzc + 2;
    auto J = [&](int j) { return pidx(g, i, j, k); };
    // face y+ (BC_3)
    double s = lv[J(ny - 1)] + lv[J(ny - 2)] + lv[J(ny - 3)];
    lv[J(ny - 1)] = lv[J(ny - 2)] = lv[J(ny - 3)] = 0.0;
    lv[J(ny - 4)] += t.num[3][1] * s;
    s = lu[J(ny - 1)] + lu[J(ny - 2)];
    lu[J(ny - 1)] = lu[J(ny - 2)] = 0.0;
    lu[J(ny - 3)] += (2.0 * t.num[3][0] - 1.0) * s;
    s = lw[J(ny - 1)] + lw[J(ny - 2)];
    lw[J(ny - 1)] = lw[J(ny - 2)] = 0.0;
    lw[J(ny - 3)] += (2.0 * t.num[3][2] - 1.0) * s;
    // face y- (BC_2)
    s = lu[J(0)] + lu[J(1)];
    lu[J(0)] = lu[J(1)] = 0.0;
    lu[J(2)] += (2.0 * t.num[2][0] - 1.0) * s;
    s = lv[J(0)] + lv[J(1)];
    lv[J(0)] = lv[J(1)] = 0.0;
    lv[J(2)] += t.num[2][1] * s;
    s = lw[J(0)] + lw[J(1)];
    lw[J(0)] = lw[J(1)] = 0.0;
    lw[J(2)] += (2.0 * t.num[2][2] - 1.0) * s;
  }
}

__global__ void __launch_bounds__(kBlock) k_adj_bc_z(Geo g, BcTable t, double *lu, double *lv, double *lw) {
  const int nxc = g.nxc, nyc = g.nyc, nz = g.nz;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nxc * nyc; q += gridDim.x * kBlock) {
    const int i = q / nyc + 2, j = q % nyc + 2;
    const long long b = pidx(g, i, j, 0);
    // face z+ (BC_5)
    double s = lw[b + nz - 1] + lw[b + nz - 2] + lw[b + nz - 3];
    lw[b + nz - 1] = lw[b + nz - 2] = lw[b + nz - 3] = 0.0;
    lw[b + nz - 4] += t.num[5][2] * s;
    s = lu[b + nz - 1] + lu[b + nz - 2];
    lu[b + nz - 1] = lu[b + nz - 2] = 0.0;
    lu[b + nz - 3] += (2.0 * t.num[5][0] - 1.0) * s;
    s = lv[b + nz - 1] + lv[b + nz - 2];
    lv[b + nz - 1] = lv[b + nz - 2] = 0.0;
    lv[b + nz - 3] += (2.0 * t.num[5][1] - 1.0) * s;
    // face z- (BC_4)
    s = lu[b + 0] + lu[b + 1];
    lu[b + 0] = lu[b + 1] = 0.0;
    lu[b + 2] += (2.0 * t.num[4][0] - 1.0) * s;
    s = lv[b + 0] + lv[b + 1];
    lv[b + 0] = lv[b + 1] = 0.0;
    lv[b + 2] += (2.0 * t.num[4][1] - 1.0) * s;
    s = lw[b + 0] + lw[b + 1];
    lw[b + 0] = lw[b + 1] = 0.0;
    lw[b + 2] += t.num[4][2] * s;
  }
}

// ---- correction^T, per face: lambda of T2 = u* - dt grad p and of eta_f -------------------
// cw: weight of Cd^n in the objective times 2 / (lz dt) (0 outside the averaging window)
__global__ void __launch_bounds__(kBlock) k_adj_corr(Geo g, double dt, double cw, const double *__restrict__ eta,
                                                     const double *__restrict__ p, const double *__restrict__ us,
                                                     const double *__restrict__ vs, const double *__restrict__ ws,
                                                     const double *__restrict__ lu, const double *__restrict__ lv,
                                                     const double *__restrict__ lw, double *lus, double *lvs,
                                                     double *lws, double *lex, double *ley, double *lez) {
  ROWS(g) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const double ec = eta[c];
    if (i < g.nx - 3) {
      const long long cp = c + g.sx;
      const double T2 = us[c] - dt * (p[cp] - p[c]) * g.rDxs[i];
      const double e = ec + (eta[cp] - ec) * g.hfx[i];
      const double vol = g.Dx[i] * g.Dy[j] * g.Dz[k];
      lus[c] = (1.0 - e) * lu[c] + cw * e * vol;
      lex[c] = -T2 * lu[c] + cw * T2 * vol;
    } else {
      lus[c] = 0.0;
      lex[c] = 0.0;
    }
    if (j < g.ny - 3) {
      const long long cp = c + g.sy;
      const double T2 = vs[c] - dt * (p[cp] - p[c]) * g.rDys[j];
      const double e = ec + (eta[cp] - ec) * g.hfy[j];
      lvs[c] = (1.0 - e) * lv[c];
      ley[c] = -T2 * lv[c];
    } else {
      lvs[c] = 0.0;
      ley[c] = 0.0;
    }
    if (k < g.nz - 3) {
      const long long cp = c + 1;
      const double T2 = ws[c] - dt * (p[cp] - p[c]) * g.rDzs[k];
      const double e = ec + (eta[cp] - ec) * g.hfz[k];
      lws[c] = (1.0 - e) * lw[c];
      lez[c] = -T2 * lw[c];
    } else {
      lws[c] = 0.0;
      lez[c] = 0.0;
    }
  }
}

// per cell: lambda_p (compact) from the faces around it, and eta's share of the faces'
// interpolated solid fractions (accumulated over steps); ghost faces hold zeros
__global__ void __launch_bounds__(kBlock) k_adj_corr_gather(Geo g, double dt, const double *__restrict__ lus,
                                                            const double *__restrict__ lvs,
                                                            const double *__restrict__ lws,
                                                            const double *__restrict__ lex,
                                                            const double *__restrict__ ley,
                                                            const double *__restrict__ lez, double *lx, double *leta,
                                                            double *part, StepScal *ss) {
  double acc[1] = {0.0};
  ROWS(g) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const double l = dt * (lus[c] * g.rDxs[i] - lus[c - g.sx] * g.rDxs[i - 1] + lvs[c] * g.rDys[j] -
                           lvs[c - g.sy] * g.rDys[j - 1] + lws[c] * g.rDzs[k] - lws[c - 1] * g.rDzs[k - 1]);
    lx[row] = l;
    acc[0] += l;
    const double itx = g.hfx[i], itx1 = g.hfx[i - 1], ity = g.hfy[j], ity1 = g.hfy[j - 1];
    const double itz = g.hfz[k], itz1 = g.hfz[k - 1];
    leta[c] += (1.0 - itx) * lex[c] + itx1 * lex[c - g.sx] + (1.0 - ity) * ley[c] + ity1 * ley[c - g.sy] +
               (1.0 - itz) * lez[c] + itz1 * lez[c - 1];
  }
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[4], out) && threadIdx.x == 0) ss->fsum[0] = out[0];  // sum of lambda_x
}

// y -= mean (mean = sum / ncell taken from ss->fsum[0], written by the previous kernel)
__global__ void __launch_bounds__(kBlock) k_sub_mean(Geo g, double *y, const StepScal *ss) {
  const double m = ss->fsum[0] / (double)g.ncell;
  ROWS(g) y[row] -= m;
}
__global__ void __launch_bounds__(kBlock) k_sum(Geo g, const double *__restrict__ y, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  ROWS(g) acc[0] += y[row];
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[4], out) && threadIdx.x == 0) ss->fsum[0] = out[0];
}

// ---- RHS^T: b = -(1/dt) div u* ---------------------------------------------------------
// Interior faces feed lambda_u*; the faces T1 copies from U^n (x: i = 1 and nx-3; y, z
// alike) feed lambda_U^n directly.  Each face is owned by one thread.
__global__ void __launch_bounds__(kBlock) k_adj_rhs(Geo g, double dt, const double *__restrict__ lb, double *lus,
                                                    double *lvs, double *lws, double *lu, double *lv, double *lw) {
  const double ddt = 1.0 / dt;
  const long long nyz = (long long)g.nyc * g.nzc;
  ROWS(g) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const double l = lb[row];
    if (i < g.nx - 3) lus[c] += -ddt * g.rDx[i] * l + ddt * g.rDx[i + 1] * lb[row + nyz];
    else lu[c] += -ddt * g.rDx[i] * l;
    if (i == 2) lu[c - g.sx] += ddt * g.rDx[i] * l;
    if (j < g.ny - 3) lvs[c] += -ddt * g.rDy[j] * l + ddt * g.rDy[j + 1] * lb[row + g.nzc];
    else lv[c] += -ddt * g.rDy[j] * l;
    if (j == 2) lv[c - g.sy] += ddt * g.rDy[j] * l;
    if (k < g.nz - 3) lws[c] += -ddt * g.rDz[k] * l + ddt * g.rDz[k + 1] * lb[row + 1];
    else lw[c] += -ddt * g.rDz[k] * l;
    if (k == 2) lw[c - 1] += ddt * g.rDz[k] * l;
  }
}

// ---- CD^T: transposed QUICK convection-diffusion ---------------------------------------
// A face value of QuickUnitA/B (inc/source/Convection_Difussion.hpp:20-90) is, for the
// branch the face velocity selects, a fixed combination of three transported values: the
// cell's own and two along the axis (offsets -2..+2).  Divisions by the metrics are
// multiplications by their reciprocal tables (RN(1/D): the adjoint is the transpose of the
// step to within an ulp per term, which no gradient check resolves), so the kernel is not
// held to the FP64 division sequence.
// A face: its coefficients on the transported values at offsets -2..+2 along the axis
// (two of them zero, by branch) and its value.
struct Face {
  double c[5];
  double val;
};

__device__ __forceinline__ void face_set(Face &F, int lo, double c0, double c1, double c2, const double *phi,
                                         long long sb) {
  // the three coefficients sit at offsets lo, lo + 1, lo + 2 (lo in -2..0)
#pragma unroll
  for (int o = 0; o < 5; ++o) F.c[o] = 0.0;
  F.c[lo + 2] = c0;
  F.c[lo + 3] = c1;
  F.c[lo + 4] = c2;
  F.val = c0 * phi[lo * sb] + c1 * phi[(lo + 1) * sb] + c2 * phi[(lo + 2) * sb];
}

// QuickUnitA (the component's own axis); phi points at the cell, rDi / rDs the reciprocals
__device__ __forceinline__ void qa_lin(double Up, double Un, long long sb, const double *Di, const double *rDi,
                                       const double *rDs, int I, const double *phi, Face &P, Face &N) {
  if (Up > 0.0) {
    const double k1 = 0.125 * Di[I + 1] * Di[I + 1] * rDs[I], a = rDi[I + 1], b = rDi[I];
    face_set(P, -1, -k1 * b, 0.5 + k1 * a + k1 * b, 0.5 - k1 * a, phi, sb);
  } else {
    const double k2 = 0.125 * Di[I + 1] * Di[I + 1] * rDs[I + 1], a2 = rDi[I + 2], a1 = rDi[I + 1];
    face_set(P, 0, 0.5 - k2 * a1, 0.5 + k2 * a2 + k2 * a1, -k2 * a2, phi, sb);
  }
  if (Un > 0.0) {
    const double k3 = 0.125 * Di[I] * Di[I] * rDs[I - 1], a = rDi[I], b = rDi[I - 1];
    face_set(N, -2, -k3 * b, 0.5 + k3 * a + k3 * b, 0.5 - k3 * a, phi, sb);
  } else {
    const double k4 = 0.125 * Di[I] * Di[I] * rDs[I], a1 = rDi[I + 1], a0 = rDi[I];
    face_set(N, -1, 0.5 - k4 * a0, 0.5 + k4 * a1 + k4 * a0, -k4 * a1, phi, sb);
  }
}

// QuickUnitB (across)
__device__ __forceinline__ void qb_lin(double Up, double Un, long long sb, const double *Ds, const double *rDi,
                                       const double *rDs, int I, const double *phi, Face &P, Face &N) {
  if (Up > 0.0) {
    const double k = 0.125 * Ds[I] * Ds[I] * rDi[I], a = rDs[I], b = rDs[I - 1];
    face_set(P, -1, -k * b, 0.5 + k * a + k * b, 0.5 - k * a, phi, sb);
  } else {
    const double k = 0.125 * Ds[I] * Ds[I] * rDi[I + 1], a2 = rDs[I + 1], a1 = rDs[I];
    face_set(P, 0, 0.5 - k * a1, 0.5 + k * a2 + k * a1, -k * a2, phi, sb);
  }
  if (Un > 0.0) {
    const double k = 0.125 * Ds[I - 1] * Ds[I - 1] * rDi[I - 1], a = rDs[I - 1], b = rDs[I - 2];
    face_set(N, -2, -k * b, 0.5 + k * a + k * b, 0.5 - k * a, phi, sb);
  } else {
    const double k = 0.125 * Ds[I - 1] * Ds[I - 1] * rDi[I], a1 = rDs[I], a0 = rDs[I - 1];
    face_set(N, -1, 0.5 - k * a0, 0.5 + k * a1 + k * a0, -k * a1, phi, sb);
  }
}

// w times a face's coefficients into the per-offset accumulators
__device__ __forceinline__ void gather_lin(double (&acc)[5], const Face &F, double w) {
#pragma unroll
  for (int o = 0; o < 5; ++o) acc[o] = fma(w, F.c[o], acc[o]);
}

// Adjoint of one component (own axis A) of ConvectionDifussion at face c:
// u*_c = u_c - dt * sum_b conv_b + nu dt * sum_b diff_b.  Contributions to the three
// fields at the cell itself go to own[0..2] (the caller adds them once); the others are
// summed per target in registers and added with one atomic each.
template <int A>
__device__ __forceinline__ void adj_component(const Geo &g, double dt, double nu, const double *const *vel,
                                              double *const *lam, long long c, const int (&I)[3], double L,
                                              double (&own)[3]) {
  const long long s[3] = {g.sx, g.sy, 1};
  const double *D[3] = {g.Dx, g.Dy, g.Dz};
  const double *S[3] = {g.Dxs, g.Dys, g.Dzs};
  const double *rD[3] = {g.rDx, g.rDy, g.rDz};
  const double *rS[3] = {g.rDxs, g.rDys, g.rDzs};
  const double *hf[3] = {g.hfx, g.hfy, g.hfz};
  const double *phi = vel[A] + c;
  double *lphi = lam[A] + c;
  own[A] += L;  // u*_c = u_c + ...
  const double gc = -dt * L, h = nu * dt * L;
  const double IT = hf[A][I[A]];  // (Ds * 0.5) / D
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const long long sb = s[b];
    const int Ib = I[b];
    const double *Db = D[b], *Sb = S[b], *rDb = rD[b], *rSb = rS[b];
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // lam[A] at offsets -2..+2 along b
    // diffusion
    double ap, an;
    if (b == A) {
      ap = rDb[Ib + 1] * rSb[Ib];
      an = rDb[Ib] * rSb[Ib];
    } else {
      ap = rSb[Ib] * rDb[Ib];
      an = rSb[Ib - 1] * rDb[Ib];
    }
    acc[3] += h * ap;
    acc[1] += h * an;
    acc[2] -= h * (ap + an);
    // convection
    Face P, N;
    if (b == A) {
      const double Up = 0.5 * (phi[sb] + phi[0]), Un = 0.5 * (phi[-sb] + phi[0]);
      qa_lin(Up, Un, sb, Db, rDb, rSb, Ib, phi, P, N);
      const double w = gc * rSb[Ib];  // (P^2 - N^2) / Ds
      gather_lin(acc, P, w * 2.0 * P.val);
      gather_lin(acc, N, -w * 2.0 * N.val);
    } else {
      const double *vb = vel[b] + c;
      double *lvb = lam[b] + c;
      const long long sA = s[A];
      const double b0 = vb[0], bA = vb[sA], bm = vb[-sb], bmA = vb[-sb + sA];
      const double Bp = b0 + (bA - b0) * IT, Bn = bm + (bmA - bm) * IT;
      qb_lin(Bp, Bn, sb, Sb, rDb, rSb, Ib, phi, P, N);
      const double w = gc * rDb[Ib];  // (P Bp - N Bn) / D
      gather_lin(acc, P, w * Bp);
      gather_lin(acc, N, -w * Bn);
      const double lBp = w * P.val, lBn = -w * N.val;
      own[b] += (1.0 - IT) * lBp;
      atomicAdd(lvb + sA, IT * lBp);
      atomicAdd(lvb - sb, (1.0 - IT) * lBn);
      atomicAdd(lvb - sb + sA, IT * lBn);
    }
    own[A] += acc[2];
#pragma unroll
    for (int o = 0; o < 5; ++o)
      if (o != 2 && acc[o] != 0.0) atomicAdd(lphi + (o - 2) * sb, acc[o]);
  }
}

__global__ void __launch_bounds__(kBlock) k_adj_convdiff(Geo g, double dt, double nu, const double *u, const double *v,
                                                         const double *w, const double *__restrict__ lus,
                                                         const double *__restrict__ lvs,
                                                         const double *__restrict__ lws, double *lu, double *lv,
                                                         double *lw) {
  const double *vel[3] = {u, v, w};
  double *lam[3] = {lu, lv, lw};
  ROWS(g) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const int I[3] = {i, j, k};
    double own[3] = {0.0, 0.0, 0.0};
    if (i < g.nx - 3 && lus[c] != 0.0) adj_component<0>(g, dt, nu, vel, lam, c, I, lus[c], own);
    if (j < g.ny - 3 && lvs[c] != 0.0) adj_component<1>(g, dt, nu, vel, lam, c, I, lvs[c], own);
    if (k < g.nz - 3 && lws[c] != 0.0) adj_component<2>(g, dt, nu, vel, lam, c, I, lws[c], own);
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (own[a] != 0.0) atomicAdd(lam[a] + c, own[a]);
  }
}

// ---- launchers ----
static int grid_for(long long n, int cap) {
  long long b = (n + kBlock - 1) / kBlock;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

void launch_adj_bc(cudaStream_t s, const Geo &g, double *lu, double *lv, double *lw, double *linlet) {
  const BcTable t = flowpassing_table(g.walls);
  // reverse of the forward phase order x, y, z
  k_adj_bc_z<<<grid_for((long long)g.nxc * g.nyc, 1024), kBlock, 0, s>>>(g, t, lu, lv, lw);
  k_adj_bc_y<<<grid_for((long long)g.nxc * g.nzc, 1024), kBlock, 0, s>>>(g, t, lu, lv, lw);
  k_adj_bc_x<<<grid_for((long long)g.nyc * g.nzc, 1024), kBlock, 0, s>>>(g, t, lu, lv, lw, linlet);
}

void launch_adj_corr(cudaStream_t s, int nblk, const Geo &g, double dt, double cw, const double *eta, const double *p,
                     const double *us, const double *vs, const double *ws, const double *lu, const double *lv,
                     const double *lw, double *lus, double *lvs, double *lws, double *lex, double *ley, double *lez,
                     double *lx, double *leta, double *part, StepScal *ss) {
  k_adj_corr<<<nblk, kBlock, 0, s>>>(g, dt, cw, eta, p, us, vs, ws, lu, lv, lw, lus, lvs, lws, lex, ley, lez);
  k_adj_corr_gather<<<nblk, kBlock, 0, s>>>(g, dt, lus, lvs, lws, lex, ley, lez, lx, leta, part, ss);
}

void launch_remove_mean(cudaStream_t s, int nblk, const Geo &g, double *y, double *part, StepScal *ss, bool sum_known) {
  if (!sum_known) k_sum<<<nblk, kBlock, 0, s>>>(g, y, part, ss);
  k_sub_mean<<<nblk, kBlock, 0, s>>>(g, y, ss);
}

void launch_adj_rhs(cudaStream_t s, int nblk, const Geo &g, double dt, const double *lb, double *lus, double *lvs,
                    double *lws, double *lu, double *lv, double *lw) {
  k_adj_rhs<<<nblk, kBlock, 0, s>>>(g, dt, lb, lus, lvs, lws, lu, lv, lw);
}

void launch_adj_convdiff(cudaStream_t s, int nblk, const Geo &g, double dt, double nu, const double *u, const double *v,
                         const double *w, const double *lus, const double *lvs, const double *lws, double *lu,
                         double *lv, double *lw) {
  k_adj_convdiff<<<nblk, kBlock, 0, s>>>(g, dt, nu, u, v, w, lus, lvs, lws, lu, lv, lw);
}

// window storage of the adjoint: the pressure rounded to FP32 and back
__global__ void __launch_bounds__(kBlock) k_f64_to_f32(long long n, const double *__restrict__ a, float *__restrict__ b) {
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock)
    b[q] = (float)a[q];
}
__global__ void __launch_bounds__(kBlock) k_f32_to_f64(long long n, const float *__restrict__ a, double *__restrict__ b) {
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock)
    b[q] = (double)a[q];
}
void launch_f64_to_f32(cudaStream_t s, long long n, const double *a, float *b) {
  k_f64_to_f32<<<(int)std::min<long long>((n + kBlock - 1) / kBlock, 4096), kBlock, 0, s>>>(n, a, b);
}
void launch_f32_to_f64(cudaStream_t s, long long n, const float *a, double *b) {
  k_f32_to_f64<<<(int)std::min<long long>((n + kBlock - 1) / kBlock, 4096), kBlock, 0, s>>>(n, a, b);
}

}  // namespace cfdgb
