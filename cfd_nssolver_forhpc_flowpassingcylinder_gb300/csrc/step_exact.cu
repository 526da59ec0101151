// FP64 projection-step kernels that reproduce the reference's arithmetic exactly.
//
// This translation unit is compiled with -fmad=false and IEEE division, so every
// kernel performs the reference function's operations in the same order and rounding:
// the results are bit-identical to the reference (checked against its golden vectors).
// One thread per interior cell (grid-stride over compact rows, k fastest, so a warp
// reads contiguous k runs of each padded array).
#include <algorithm>
#include <cmath>

#include "cfdgb_internal.cuh"
#include "reduce.cuh"
#include "stepctl.cuh"
#include "kernels.h"

namespace cfdgb {

// inc/source/Convection_Difussion.hpp:20-51 (QuickUnitA)
__device__ __forceinline__ void quick_a(bool two, double Up, double Un, long long pp, long long p, long long ic,
                                        long long n, long long nn, const double *__restrict__ Di,
                                        const double *__restrict__ Ds, const double *__restrict__ rDi,
                                        const double *__restrict__ rDs, int I,
                                        const double *__restrict__ phi, double &P, double &N) {
  const double fc = phi[ic], fp = phi[p], fn = phi[n];
  auto oi = [&](double a, int q) { return div_by(a, Di[q], rDi[q], two); };  // a / Di[q]
  auto os = [&](double a, int q) { return div_by(a, Ds[q], rDs[q], two); };  // a / Ds[q]
  if (Up > 0.0)
    P = 0.5 * (fc + fp) - os(0.125 * Di[I + 1] * Di[I + 1], I) * (oi(fp - fc, I + 1) - oi(fc - fn, I));
  else
    P = 0.5 * (fc + fp) -
        os(0.125 * Di[I + 1] * Di[I + 1], I + 1) * (oi(phi[pp] - fp, I + 2) - oi(fp - fc, I + 1));
  if (Un > 0.0)
    N = 0.5 * (fn + fc) -
        os(0.125 * Di[I] * Di[I], I - 1) * (oi(fc - fn, I) - oi(fn - phi[nn], I - 1));
  else
    N = 0.5 * (fn + fc) - os(0.125 * Di[I] * Di[I], I) * (oi(fp - fc, I + 1) - oi(fc - fn, I));
}

// inc/source/Convection_Difussion.hpp:55-90 (QuickUnitB)
__device__ __forceinline__ void quick_b(bool two, double Up, double Un, long long pp, long long p, long long ic,
                                        long long n, long long nn, const double *__restrict__ Di,
                                        const double *__restrict__ Ds, const double *__restrict__ rDi,
                                        const double *__restrict__ rDs, int I,
                                        const double *__restrict__ phi, double &P, double &N) {
  const double fc = phi[ic], fp = phi[p], fn = phi[n];
  auto oi = [&](double a, int q) { return div_by(a, Di[q], rDi[q], two); };  // a / Di[q]
  auto os = [&](double a, int q) { return div_by(a, Ds[q], rDs[q], two); };  // a / Ds[q]
  if (Up > 0.0)
    P = 0.5 * (fc + fp) - oi(0.125 * Ds[I] * Ds[I], I) * (os(fp - fc, I) - os(fc - fn, I - 1));
  else
    P = 0.5 * (fc + fp) -
        oi(0.125 * Ds[I] * Ds[I], I + 1) * (os(phi[pp] - fp, I + 1) - os(fp - fc, I));
  if (Un > 0.0)
    N = 0.5 * (fn + fc) -
        oi(0.125 * Ds[I - 1] * Ds[I - 1], I - 1) * (os(fc - fn, I - 1) - os(fn - phi[nn], I - 2));
  else
    N = 0.5 * (fn + fc) - oi(0.125 * Ds[I - 1] * Ds[I - 1], I) * (os(fp - fc, I) - os(fc - fn, I - 1));
}

// inc/source/Convection_Difussion.hpp:96-147 (LudUnitA; LudUnitB has the same body)
__device__ __forceinline__ void lud(bool two, double Up, double Un, long long pp, long long p, long long ic, long long n,
                                    long long nn, const double *__restrict__ Di, const double *__restrict__ Ds,
                                    const double *__restrict__ rDi, const double *__restrict__ rDs, int I,
                                    const double *__restrict__ phi, double &P, double &N) {
  const double fc = phi[ic], fp = phi[p], fn = phi[n];
  auto oi = [&](double a, int q) { return div_by(a, Di[q], rDi[q], two); };  // a / Di[q]
  if (Up > 0.0)
    P = (fc + oi(0.5 * Ds[I] * (fc - fn), I));
  else
    P = (fp + oi(0.5 * Ds[I + 1] * (fp - phi[pp]), I + 1));
  if (Un > 0.0)
    N = (fn + oi(0.5 * Ds[I - 1] * (fn - phi[nn]), I - 1));
  else
    N = (fc + oi(0.5 * Ds[I] * (fc - fp), I + 1));
}

// face values of one axis under the convection switch (inc/0_General.hpp:114-118): QUICK,
// LUD or UD (UdUnit, :150-168); OWN: the component's own axis (the "A" units)
template <int S, bool OWN>
__device__ __forceinline__ void face(bool two, double Up, double Un, long long pp, long long p, long long ic, long long n,
                                     long long nn, const double *__restrict__ Di, const double *__restrict__ Ds,
                                     const double *__restrict__ rDi, const double *__restrict__ rDs, int I,
                                     const double *__restrict__ phi, double &P, double &N) {
  if (S == CFDGB_LUD) {
    lud(two, Up, Un, pp, p, ic, n, nn, Di, Ds, rDi, rDs, I, phi, P, N);
  } else if (S == CFDGB_UD) {
    P = Up > 0.0 ? phi[ic] : phi[p];
    N = Un > 0.0 ? phi[n] : phi[ic];
  } else if (OWN) {
    quick_a(two, Up, Un, pp, p, ic, n, nn, Di, Ds, rDi, rDs, I, phi, P, N);
  } else {
    quick_b(two, Up, Un, pp, p, ic, n, nn, Di, Ds, rDi, rDs, I, phi, P, N);
  }
}

// inc/source/SmagorinskyModel.hpp:30-79 with GradientGauss (:6-26), CS = 0.18: eddy
// viscosity of T0 per cell, nut[row] = l2[row] sqrt|2 ux^2 + vy^2 + wz^2 + (uy + vx)^2 +
// (uz + wx)^2 + (vz + wy)^2| with the reference's central differences (u over Dxs, Dy, Dz;
// v over Dx, Dys, Dz; w over Dx, Dy, Dzs; the sum as the reference writes it).  l2 =
// (CS cbrt(Dx Dy Dz))^2 per cell, computed once on the host with the same pow.
__global__ void __launch_bounds__(kBlock) k_smagorinsky(Geo g, const double *__restrict__ l2,
                                                        const double *__restrict__ u, const double *__restrict__ v,
                                                        const double *__restrict__ w, double *__restrict__ nut) {
  const long long sx = g.sx, sy = g.sy;
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const bool two = g.div2 != 0;
    auto h = [&](double d, double r) { return div_by(0.5, d, r, two); };  // 0.5 / d
    const double ux = h(g.Dxs[i], g.rDxs[i]) * (u[c - sx] - u[c + sx]);
    const double uy = h(g.Dy[j], g.rDy[j]) * (u[c - sy] - u[c + sy]);
    const double uz = h(g.Dz[k], g.rDz[k]) * (u[c - 1] - u[c + 1]);
    const double vx = h(g.Dx[i], g.rDx[i]) * (v[c - sx] - v[c + sx]);
    const double vy = h(g.Dys[j], g.rDys[j]) * (v[c - sy] - v[c + sy]);
    const double vz = h(g.Dz[k], g.rDz[k]) * (v[c - 1] - v[c + 1]);
    const double wx = h(g.Dx[i], g.rDx[i]) * (w[c - sx] - w[c + sx]);
    const double wy = h(g.Dy[j], g.rDy[j]) * (w[c - sy] - w[c + sy]);
    const double wz = h(g.Dzs[k], g.rDzs[k]) * (w[c - 1] - w[c + 1]);
    const double a = uy + vx, b = uz + wx, e = vz + wy;
    const double temp = fabs(2.0 * (ux * ux) + vy * vy + wz * wz + a * a + b * b + e * e);
    nut[row] = l2[row] * sqrt(temp);
  }
}

// inc/source/Convection_Difussion.hpp:174-450: explicit Euler convection (QUICK, LUD or UD)
// + central diffusion; the last face along a component's own axis is a boundary face and
// skipped.
// S: the convection scheme; nut (compact, may be null): the Smagorinsky eddy viscosity
// added to nu per cell (Convection_Difussion.hpp:251-256).
// Fused with get_Cfl (inc/analyses/cfl.hpp:3-78, called on u* right after this function,
// src/RUN_CPU.cpp:274): each thread takes u*, v*, w* of its cell from registers, with the
// reference's division and order (c = u/Dxs + v/Dys + w/Dzs, a term left out on the last
// face of its axis), so the CFL number and extremes are those of get_Cfl bit for bit; the
// maxima are exact in any order.  The last block also sets the next dt (StepCtl).
// Two resident blocks per SM (at most 128 registers a thread): the kernel is bound by the
// FP64 pipe, and one block of 8 warps per SM leaves it waiting on latency.
template <int S, bool AB>
__global__ void __launch_bounds__(kBlock, 2) k_convdiff_exact(Geo g, double dt_arg, double nu0,
                                                           const double *__restrict__ nut,
                                                           const double *__restrict__ u,
                                                           const double *__restrict__ v,
                                                           const double *__restrict__ w,
                                                           double *__restrict__ us,
                                                           double *__restrict__ vs,
                                                           double *__restrict__ ws, StepCtl sc) {
  const double dt = step_dt(sc, dt_arg);
  const bool two = g.div2 != 0;
  CflAcc cfl;
  AbStep ab;
  if (AB) ab.init(sc, dt);
  const long long sx = g.sx, sy = g.sy, sz = 1;
  const double *Dx = g.Dx, *Dy = g.Dy, *Dz = g.Dz, *Dxs = g.Dxs, *Dys = g.Dys, *Dzs = g.Dzs;
  const double *rDx = g.rDx, *rDy = g.rDy, *rDz = g.rDz, *rDxs = g.rDxs, *rDys = g.rDys, *rDzs = g.rDzs;
  // a / D[q] of each metric array (div_by with the array's reciprocals)
  auto ox = [&](double a, int q) { return div_by(a, Dx[q], rDx[q], two); };
  auto oy = [&](double a, int q) { return div_by(a, Dy[q], rDy[q], two); };
  auto oz = [&](double a, int q) { return div_by(a, Dz[q], rDz[q], two); };
  auto oxs = [&](double a, int q) { return div_by(a, Dxs[q], rDxs[q], two); };
  auto oys = [&](double a, int q) { return div_by(a, Dys[q], rDys[q], two); };
  auto ozs = [&](double a, int q) { return div_by(a, Dzs[q], rDzs[q], two); };
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const double nu = nut ? nu0 + nut[row] : nu0;
    const long long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz, zp = ic + sz;
    double ccfl = 0.0;
    if (i < g.nx - 3) {  // u
      const double IT = ox(Dxs[i] * 0.5, i);
      const double uc = u[ic], uxp = u[xp], uxm = u[xm];
      const double Up = 0.5 * (uxp + uc);
      const double Un = 0.5 * (uxm + uc);
      const double Vp = v[ic] + (v[xp] - v[ic]) * IT;
      const double Vn = v[ym] + (v[ym + xp - ic] - v[ym]) * IT;
      const double Wp = w[ic] + (w[xp] - w[ic]) * IT;
      const double Wn = w[zm] + (w[zm + xp - ic] - w[zm]) * IT;
      double uPx, uNx, uPy, uNy, uPz, uNz;
      face<S, true>(two, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, rDx, rDxs, i, u, uPx, uNx);
      face<S, false>(two, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, rDy, rDys, j, u, uPy, uNy);
      face<S, false>(two, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, rDz, rDzs, k, u, uPz, uNz);
      const double convection = -dt * (oxs(uPx * uPx - uNx * uNx, i) + oy(uPy * Vp - uNy * Vn, j) +
                                       oz(uPz * Wp - uNz * Wn, k));
      const double difussion =
          nu * dt *
          (oxs(ox(uxp - uc, i + 1) - ox(uc - uxm, i), i) +
           oy(oys(u[yp] - uc, j) - oys(uc - u[ym], j - 1), j) +
           oz(ozs(u[zp] - uc, k) - ozs(uc - u[zm], k - 1), k));
      const double r = AB ? ab.value(0, ic, uc, convection, difussion) : uc + convection + difussion;
      us[ic] = r;
      ccfl += oxs(r, i);
      cfl.comp(0, r);
    }
    if (j < g.ny - 3) {  // v
      const double IT = oy(Dys[j] * 0.5, j);
      const double vc = v[ic], vyp = v[yp], vym = v[ym];
      const double Vp = 0.5 * (vyp + vc);
      const double Vn = 0.5 * (vym + vc);
      const double Up = u[ic] + (u[yp] - u[ic]) * IT;
      const double Un = u[xm] + (u[xm + yp - ic] - u[xm]) * IT;
      const double Wp = w[ic] + (w[yp] - w[ic]) * IT;
      const double Wn = w[zm] + (w[zm + yp - ic] - w[zm]) * IT;
      double vPx, vNx, vPy, vNy, vPz, vNz;
      face<S, false>(two, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, rDx, rDxs, i, v, vPx, vNx);
      face<S, true>(two, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, rDy, rDys, j, v, vPy, vNy);
      face<S, false>(two, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, rDz, rDzs, k, v, vPz, vNz);
      const double convection = -dt * (ox(Up * vPx - Un * vNx, i) + oys(vPy * vPy - vNy * vNy, j) +
                                       oz(Wp * vPz - Wn * vNz, k));
      const double difussion =
          nu * dt *
          (ox(oxs(v[xp] - vc, i) - oxs(vc - v[xm], i - 1), i) +
           oys(oy(vyp - vc, j + 1) - oy(vc - vym, j), j) +
           oz(ozs(v[zp] - vc, k) - ozs(vc - v[zm], k - 1), k));
      const double r = AB ? ab.value(1, ic, vc, convection, difussion) : vc + convection + difussion;
      vs[ic] = r;
      ccfl += oys(r, j);
      cfl.comp(1, r);
    }
    if (k < g.nz - 3 + g.pz) {  // w (periodic z: the top face too)
      const double IT = oz(Dzs[k] * 0.5, k);
      const double wc = w[ic], wzp = w[zp], wzm = w[zm];
      const double Wp = 0.5 * (wzp + wc);
      const double Wn = 0.5 * (wzm + wc);
      const double Up = u[ic] + (u[zp] - u[ic]) * IT;
      const double Un = u[xm] + (u[xm + zp - ic] - u[xm]) * IT;
      const double Vp = v[ic] + (v[zp] - v[ic]) * IT;
      const double Vn = v[ym] + (v[ym + zp - ic] - v[ym]) * IT;
      double wPx, wNx, wPy, wNy, wPz, wNz;
      face<S, false>(two, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, rDx, rDxs, i, w, wPx, wNx);
      face<S, false>(two, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, rDy, rDys, j, w, wPy, wNy);
      face<S, true>(two, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, rDz, rDzs, k, w, wPz, wNz);
      const double convection = -dt * (ox(Up * wPx - Un * wNx, i) + oy(Vp * wPy - Vn * wNy, j) +
                                       ozs(wPz * wPz - wNz * wNz, k));
      const double difussion =
          nu * dt *
          (ox(oxs(w[xp] - wc, i) - oxs(wc - w[xm], i - 1), i) +
           oy(oys(w[yp] - wc, j) - oys(wc - w[ym], j - 1), j) +
           ozs(oz(wzp - wc, k + 1) - oz(wc - wzm, k), k));
      const double r = AB ? ab.value(2, ic, wc, convection, difussion) : wc + convection + difussion;
      ws[ic] = r;
      ccfl += ozs(r, k);
      cfl.comp(2, r);
    }
    cfl.cell(ccfl);
  }
  if (sc.ss) cfl_finish(cfl, dt, sc);
}

// inc/matrix/b_matrix.hpp:35-98: b = -(jp)(1/dt) div(u*), one-sided differences
__global__ void __launch_bounds__(kBlock) k_rhs_exact(Geo g, double dt_arg, const double *dtp,
                                                      const double *__restrict__ us,
                                                      const double *__restrict__ vs,
                                                      const double *__restrict__ ws, int jacobi,
                                                      Stencil<double> st, double *__restrict__ b) {
  const double ddt = 1.0 / (dtp ? *dtp : dt_arg);
  const bool two = g.div2 != 0;
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    // periodic z: the bottom face of the first cell is the top face nz-3
    const long long zb = (g.pz && k == 2) ? ic + g.nzc - 1 : ic - 1;
    const double div = div_by(us[ic] - us[ic - g.sx], g.Dx[i], g.rDx[i], two) +
                       div_by(vs[ic] - vs[ic - g.sy], g.Dy[j], g.rDy[j], two) +
                       div_by(ws[ic] - ws[zb], g.Dz[k], g.rDz[k], two);
    if (jacobi) {
      b[row] = -row_jp(g, st, i - 2, j - 2, k - 2, row) * ddt * div;
    } else {
      b[row] = -ddt * div;
    }
  }
}

// SPE_matrix::multiply_omp / CSR_matrix::multiply_omp with the reference's entry values
__global__ void __launch_bounds__(kBlock) k_spmv_exact(Geo g, Stencil<double> st, const double *__restrict__ x,
                                                       double *__restrict__ y) {
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int ic, jc, kc;
    row_cijk(row, g.nyc, g.nzc, ic, jc, kc);
    y[row] = stencil_row_g(g, st, x, row, ic, jc, kc);
  }
}

// inc/analyses/cfl.hpp:3-78 (get_Cfl) on u*: per cell c = u/Dxs + v/Dys + w/Dzs, each term
// left out on the last face of its own axis (the loops' "-d"), added in that order; the
// maximum of c times dt, and the extremes of each component over its faces.  ss->cfl.
// (The time step computes the same inside k_convdiff_exact; this is the single call.)
__global__ void __launch_bounds__(kBlock) k_cfl(Geo g, double dt, const double *__restrict__ us,
                                                 const double *__restrict__ vs, const double *__restrict__ ws,
                                                 StepCtl sc) {
  const bool two = g.div2 != 0;
  CflAcc cfl;
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    double c = 0.0;
    if (i < g.nx - 3) {
      c += div_by(us[ic], g.Dxs[i], g.rDxs[i], two);
      cfl.comp(0, us[ic]);
    }
    if (j < g.ny - 3) {
      c += div_by(vs[ic], g.Dys[j], g.rDys[j], two);
      cfl.comp(1, vs[ic]);
    }
    if (k < g.nz - 3 + g.pz) {
      c += div_by(ws[ic], g.Dzs[k], g.rDzs[k], two);
      cfl.comp(2, ws[ic]);
    }
    cfl.cell(c);
  }
  cfl_finish(cfl, dt, sc);
}

// Plot3D solution arrays (inc/io/Plot3D/qfile.hpp:62-103) in k-j-i order, i fastest, as
// float32: p, the cell-centred u, v, w (face means, rounded once) and eta
__global__ void __launch_bounds__(kBlock) k_plot3d_pack(Geo g, const double *__restrict__ p,
                                                         const double *__restrict__ u, const double *__restrict__ v,
                                                         const double *__restrict__ w, const double *__restrict__ eta,
                                                         float *__restrict__ out) {
  const long long n = g.ncell;
  for (long long o = blockIdx.x * (long long)kBlock + threadIdx.x; o < n; o += (long long)gridDim.x * kBlock) {
    const int ic = (int)(o % g.nxc);
    const long long r = o / g.nxc;
    const int jc = (int)(r % g.nyc), kc = (int)(r / g.nyc);
    const long long c = pidx(g, ic + 2, jc + 2, kc + 2);
    out[o] = (float)p[c];
    out[n + o] = (float)(0.5 * (u[c - g.sx] + u[c]));
    out[2 * n + o] = (float)(0.5 * (v[c - g.sy] + v[c]));
    out[3 * n + o] = (float)(0.5 * (w[c - 1] + w[c]));
    out[4 * n + o] = (float)eta[c];
  }
}

// QfileRead (inc/io/Plot3D/qfileRead.hpp:66-97): the five cell-centred float32 arrays of a
// .q file (p, u, v, w, eta; i fastest) back to padded fields.  p and eta are copied; u, v, w
// go to faces as the float sum of the cells on both sides, halved in double, and the last
// face of each axis takes its own cell's value.  Interior cells only; eta may be null.
__global__ void __launch_bounds__(kBlock) k_plot3d_unpack(Geo g, const float *__restrict__ in,
                                                           double *__restrict__ p, double *__restrict__ u,
                                                           double *__restrict__ v, double *__restrict__ w,
                                                           double *__restrict__ eta) {
  const long long n = g.ncell, sj = g.nxc, sk = (long long)g.nxc * g.nyc;
  const float *U = in + n, *V = in + 2 * n, *W = in + 3 * n;
  for (long long o = blockIdx.x * (long long)kBlock + threadIdx.x; o < n; o += (long long)gridDim.x * kBlock) {
    const int ic = (int)(o % g.nxc);
    const long long r = o / g.nxc;
    const int jc = (int)(r % g.nyc), kc = (int)(r / g.nyc);
    const long long c = pidx(g, ic + 2, jc + 2, kc + 2);
    p[c] = (double)in[o];
    u[c] = ic == g.nxc - 1 ? (double)U[o] : (double)__fadd_rn(U[o], U[o + 1]) / 2.0;
    v[c] = jc == g.nyc - 1 ? (double)V[o] : (double)__fadd_rn(V[o], V[o + sj]) / 2.0;
    w[c] = kc == g.nzc - 1 ? (double)W[o] : (double)__fadd_rn(W[o], W[o + sk]) / 2.0;
    if (eta) eta[c] = (double)in[4 * n + o];
  }
}

// inc/pressure/Transform.hpp:8-20
__global__ void __launch_bounds__(kBlock) k_transform(Geo g, const double *__restrict__ x, double *__restrict__ p) {
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    p[pidx(g, i, j, k)] = x[row];
  }
}

// inc/dfib/updateUandF.hpp:90-180 (solid velocity 0), fused with the drag/lift sums of
// virtualF_Int (inc/dfib/virtualForceIntergrator.hpp:67-90) and, in the time step, with
// the part of copyVel (inc/source/copyVel.hpp:4) that matters: the faces update_UandF
// never writes keep the initial values (ui, vi, wi) they hold in the reference's T3.
__global__ void __launch_bounds__(kBlock) k_update_uf_exact(
    Geo g, double dt_arg, const double *dtp, int in_step /* step_end mode */, double lz, const double *__restrict__ eta,
    const double *__restrict__ p, const double *__restrict__ us, const double *__restrict__ vs,
    const double *__restrict__ ws, double *__restrict__ u3, double *__restrict__ v3, double *__restrict__ w3,
    double *__restrict__ f, const double *__restrict__ ui, const double *__restrict__ vi,
    const double *__restrict__ wi, double *part, StepScal *ss) {
  const double dt = dtp ? *dtp : dt_arg;
  const bool two = g.div2 != 0;
  const long long tot = (long long)g.nx * g.ny * g.nz;
  const double uS = 0.0, vS = 0.0, wS = 0.0;
  const double rdt = 1.0 / dt;
  double acc[2] = {0.0, 0.0};
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const double vol = g.Dx[i] * g.Dy[j] * g.Dz[k];
    const double ec = eta[ic];
    if (i < g.nx - 3) {
      const long long icP = ic + g.sx;
      const double T2u = us[ic] - div_by(dt * (p[icP] - p[ic]), g.Dxs[i], g.rDxs[i], two);
      const double e = ec + (eta[icP] - ec) * g.hfx[i];
      const double nu3 = ec * uS + (1.0 - e) * T2u;
      const double fx = div_by(nu3 - T2u, dt, rdt, two);
      u3[ic] = nu3;
      if (f) f[ic] = fx;
      acc[0] += fx * vol;
    } else if (ui) {
      u3[ic] = ui[ic];
    }
    if (j < g.ny - 3) {
      const long long icP = ic + g.sy;
      const double T2v = vs[ic] - div_by(dt * (p[icP] - p[ic]), g.Dys[j], g.rDys[j], two);
      const double e = ec + (eta[icP] - ec) * g.hfy[j];
      const double nv3 = ec * vS + (1.0 - e) * T2v;
      const double fy = div_by(nv3 - T2v, dt, rdt, two);
      v3[ic] = nv3;
      if (f) f[ic + tot] = fy;
      acc[1] += fy * vol;
    } else if (vi) {
      v3[ic] = vi[ic];
    }
    if (k < g.nz - 3 + g.pz) {  // periodic z: the top face, its upper cell the first one
      const long long icP = (g.pz && k == g.nz - 3) ? ic - (g.nzc - 1) : ic + 1;
      const double T2w = ws[ic] - div_by(dt * (p[icP] - p[ic]), g.Dzs[k], g.rDzs[k], two);
      const double e = ec + (eta[icP] - ec) * g.hfz[k];
      const double nw3 = ec * wS + (1.0 - e) * T2w;
      w3[ic] = nw3;
      if (f) f[ic + 2 * tot] = div_by(nw3 - T2w, dt, rdt, two);
    } else if (wi) {
      w3[ic] = wi[ic];
    }
  }
  double out[2];
  if (grid_sum<2>(acc, part, &ss->cnt[0], out) && threadIdx.x == 0) {
    ss->fsum[0] = out[0];
    ss->fsum[1] = out[1];
    ss->cd = -2.0 * out[0] / lz;  // CD_CL, virtualForceIntergrator.hpp:309-314
    ss->cl = -2.0 * out[1] / lz;
    ss->nan_flag = !(isfinite(out[0]) && isfinite(out[1]));
    step_end(ss, dt, in_step);
  }
}

// ---- ghost fill: BC_staggered_main (Boundary_Condition.hpp:37-176) in three phases that
// keep its one-thread order (x faces, then y, then z; each later phase reads cells the
// earlier ones wrote), each fused with the matching part of BC_staggered_copy
// (updateBC.hpp:6-108), whose cells no later phase touches.  bc: Dir/Num table
// (FLOWpassing.hpp:6-40, BcTable).  inlet: optional per-(j,k) inlet velocity taking the
// place of Dir[0][0] (all 1.0 reproduces the reference).
// Two options that are not in the reference: a convective outflow in place of face 1's
// rows (k_outflow_flux first, then k_bc_x), and periodic z in place of faces 4 and 5.

// Convective outflow at the x+ face: d(phi)/dt + Uc d(phi)/dx = 0 for the outlet u face and
// the v, w ghost cells beyond it, implicit upwind in time.  In a step (conv) the outlet u
// before the flux correction is (u_b + cu u_(nx-4)) / (1 + cu), u_b the last step's value
// (the copy in us, which no kernel of the step writes), cu = Uc dt / Dx[nx-3]; at init the
// zero-gradient value u_(nx-4).  The ghosts: (phi_g + cv phi_(nx-3)) / (1 + cv), cv =
// Uc dt / Dxs[nx-3], or phi_(nx-3) at init.
__device__ __forceinline__ double outlet_u(const Geo &g, const double *u, const double *us, double cu, int j,
                                           int k) {
  const double un = u[pidx(g, g.nx - 4, j, k)];
  return us ? (us[pidx(g, g.nx - 3, j, k)] + cu * un) / (1.0 + cu) : un;
}
__device__ __forceinline__ double outlet_ghost(const Geo &g, const double *f, const double *fs, double cv, int j,
                                               int k) {
  const double fn = f[pidx(g, g.nx - 3, j, k)];
  return fs ? (fs[pidx(g, g.nx - 2, j, k)] + cv * fn) / (1.0 + cv) : fn;
}
// cu, cv of a step: dt is the step's (set by the velocity correction's step_end)
__device__ __forceinline__ void outlet_coeffs(const Geo &g, const StepScal *ss, bool conv, double &cu,
                                              double &cv) {
  cu = cv = 0.0;
  if (!conv) return;
  const double dt = ss->dt_step;
  cu = g.uconv * dt / g.Dx[g.nx - 3];
  cv = g.uconv * dt / g.Dxs[g.nx - 3];
}

// The outlet correction: the net flux through the boundary with the outlet faces at
// outlet_u -- inlet u faces, outlet faces, the y-wall v faces and (not periodic) the z-wall
// w faces at the values the ghost fill gives them, each times its face area -- divided by
// the outlet's area, into ss->oflux.  One grid-stride pass over the three face sets.
__global__ void __launch_bounds__(kBlock) k_outflow_flux(Geo g, BcTable t, const double *__restrict__ inlet,
                                                         const double *__restrict__ u, const double *__restrict__ v,
                                                         const double *__restrict__ w, const double *__restrict__ us,
                                                         double *part, StepScal *ss) {
  double cu, cv;
  outlet_coeffs(g, ss, us != nullptr, cu, cv);
  const long long nx_ = g.nyc * (long long)g.nzc, ny_ = g.nxc * (long long)g.nzc,
                  nz_ = g.pz ? 0 : g.nxc * (long long)g.nyc;
  double acc[2] = {0.0, 0.0};  // flux, outlet area
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < nx_ + ny_ + nz_;
       q += (long long)gridDim.x * kBlock) {
    if (q < nx_) {
      const int j = (int)(q / g.nzc) + 2, k = (int)(q % g.nzc) + 2;
      const double a = g.Dy[j] * g.Dz[k];
      const double uin = (inlet ? inlet[q] : t.dir[0][0]) + t.num[0][0] * u[pidx(g, 2, j, k)];
      acc[0] += (uin - outlet_u(g, u, us, cu, j, k)) * a;
      acc[1] += a;
    } else if (q < nx_ + ny_) {
      const long long r = q - nx_;
      const int i = (int)(r / g.nzc) + 2, k = (int)(r % g.nzc) + 2;
      const double vb = t.dir[2][1] + t.num[2][1] * v[pidx(g, i, 2, k)];
      const double vt = t.dir[3][1] + t.num[3][1] * v[pidx(g, i, g.ny - 4, k)];
      acc[0] += (vb - vt) * (g.Dx[i] * g.Dz[k]);
    } else {
      const long long r = q - nx_ - ny_;
      const int i = (int)(r / g.nyc) + 2, j = (int)(r % g.nyc) + 2;
      const double wb = t.dir[4][2] + t.num[4][2] * w[pidx(g, i, j, 2)];
      const double wt = t.dir[5][2] + t.num[5][2] * w[pidx(g, i, j, g.nz - 4)];
      acc[0] += (wb - wt) * (g.Dx[i] * g.Dy[j]);
    }
  }
  double out[2];
  if (grid_sum<2>(acc, part, &ss->cnt[8], out) && threadIdx.x == 0) ss->oflux = out[0] / out[1];
}

__global__ void __launch_bounds__(kBlock) k_bc_x(Geo g, BcTable t, const double *__restrict__ inlet, double *u,
                                                 double *v, double *w, double *p, double *us, double *vs, double *ws,
                                                 int do_main, int conv, const StepScal *ss) {
  const int nyc = g.nyc, nzc = g.nzc, nx = g.nx;
  double cu = 0.0, cv = 0.0, corr = 0.0;
  if (do_main && g.outflow) {
    outlet_coeffs(g, ss, conv != 0, cu, cv);
    corr = ss->oflux;
  }
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nyc * nzc; q += gridDim.x * kBlock) {
    const int j = q / nzc + 2, k = q % nzc + 2;
    auto I = [&](int i) { return pidx(g, i, j, k); };
    if (do_main) {
      const double din = inlet ? inlet[q] : t.dir[0][0];
      u[I(1)] = u[I(0)] = din + t.num[0][0] * u[I(2)];
      v[I(1)] = v[I(0)] = t.dir[0][1] * 2. + (2.0 * t.num[0][1] - 1.0) * v[I(2)];
      w[I(1)] = w[I(0)] = t.dir[0][2] * 2. + (2.0 * t.num[0][2] - 1.0) * w[I(2)];
      if (g.outflow) {
        const double *os = conv ? us : nullptr;
        const double ub = outlet_u(g, u, os, cu, j, k) + corr;
        const double vg = outlet_ghost(g, v, conv ? vs : nullptr, cv, j, k);
        const double wg = outlet_ghost(g, w, conv ? ws : nullptr, cv, j, k);
        u[I(nx - 1)] = u[I(nx - 2)] = u[I(nx - 3)] = ub;
        v[I(nx - 1)] = v[I(nx - 2)] = vg;
        w[I(nx - 1)] = w[I(nx - 2)] = wg;
      } else {
        u[I(nx - 1)] = u[I(nx - 2)] = u[I(nx - 3)] = t.dir[1][0] + t.num[1][0] * u[I(nx - 4)];
        v[I(nx - 1)] = v[I(nx - 2)] = t.dir[1][1] * 2. + (2.0 * t.num[1][1] - 1.0) * v[I(nx - 3)];
        w[I(nx - 1)] = w[I(nx - 2)] = t.dir[1][2] * 2. + (2.0 * t.num[1][2] - 1.0) * w[I(nx - 3)];
      }
      if (p) {
        p[I(1)] = p[I(0)] = p[I(2)];
        p[I(nx - 2)] = p[I(nx - 1)] = p[I(nx - 3)];
      }
    }
    if (us) {
      const int iu[5] = {0, 1, nx - 1, nx - 3, nx - 2};
#pragma unroll
      for (int a = 0; a < 5; ++a) us[I(iu[a])] = u[I(iu[a])];
      const int iv[4] = {0, 1, nx - 2, nx - 1};
#pragma unroll
      for (int a = 0; a < 4; ++a) { vs[I(iv[a])] = v[I(iv[a])]; ws[I(iv[a])] = w[I(iv[a])]; }
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_bc_y(Geo g, BcTable t, double *u, double *v, double *w, double *p,
                                                 double *us, double *vs, double *ws, int do_main) {
  const int nxc = g.nxc, nzc = g.nzc, ny = g.ny;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nxc * nzc; q += gridDim.x * kBlock) {
    const int i = q / nzc + 2, k = q % nzc + 2;
    auto J = [&](int j) { return pidx(g, i, j, k); };
    if (do_main) {
      u[J(1)] = u[J(0)] = t.dir[2][0] * 2. + (2.0 * t.num[2][0] - 1.0) * u[J(2)];
      v[J(1)] = v[J(0)] = t.dir[2][1] + t.num[2][1] * v[J(2)];
      w[J(1)] = w[J(0)] = t.dir[2][2] * 2. + (2.0 * t.num[2][2] - 1.0) * w[J(2)];
      v[J(ny - 1)] = v[J(ny - 2)] = v[J(ny - 3)] = t.dir[3][1] + t.num[3][1] * v[J(ny - 4)];
      u[J(ny - 1)] = u[J(ny - 2)] = t.dir[3][0] * 2. + (2.0 * t.num[3][0] - 1.0) * u[J(ny - 3)];
      w[J(ny - 1)] = w[J(ny - 2)] = t.dir[3][2] * 2. + (2.0 * t.num[3][2] - 1.0) * w[J(ny - 3)];
      if (p) {
        p[J(1)] = p[J(0)] = p[J(2)];
        p[J(ny - 2)] = p[J(ny - 1)] = p[J(ny - 3)];
      }
    }
    if (us) {
      const int ju[4] = {0, 1, ny - 2, ny - 1};
#pragma unroll
      for (int a = 0; a < 4; ++a) { us[J(ju[a])] = u[J(ju[a])]; ws[J(ju[a])] = w[J(ju[a])]; }
      const int jv[5] = {0, 1, ny - 3, ny - 2, ny - 1};
#pragma unroll
      for (int a = 0; a < 5; ++a) vs[J(jv[a])] = v[J(jv[a])];
    }
  }
}

// periodic z: the two ghost layers on each side take the images nzc cells away (w's face
// 1 is the image of the top face nz-3), over the whole padded (i, j) plane so that the
// edges and corners next to the z ghosts are periodic too; the copy into T1 as the
// reference's (interior (i, j), the z ghosts and w's face nz-3)
__global__ void __launch_bounds__(kBlock) k_bc_zp(Geo g, double *u, double *v, double *w, double *p, double *us,
                                                  double *vs, double *ws, int do_main) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nx * ny; q += gridDim.x * kBlock) {
    const int i = q / ny, j = q % ny;
    const long long base = pidx(g, i, j, 0);
    if (do_main) {
      double *f[4] = {u, v, w, p};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        if (!f[a]) continue;
        f[a][base + 0] = f[a][base + nz - 4];
        f[a][base + 1] = f[a][base + nz - 3];
        f[a][base + nz - 2] = f[a][base + 2];
        f[a][base + nz - 1] = f[a][base + 3];
      }
    }
    if (us && i >= 2 && i < nx - 2 && j >= 2 && j < ny - 2) {
      const int ku[4] = {0, 1, nz - 2, nz - 1};
#pragma unroll
      for (int a = 0; a < 4; ++a) { us[base + ku[a]] = u[base + ku[a]]; vs[base + ku[a]] = v[base + ku[a]]; }
      const int kw[5] = {0, 1, nz - 3, nz - 2, nz - 1};
#pragma unroll
      for (int a = 0; a < 5; ++a) ws[base + kw[a]] = w[base + kw[a]];
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_bc_z(Geo g, BcTable t, double *__restrict__ u, double *__restrict__ v,
                                                 double *__restrict__ w, double *__restrict__ p,
                                                 double *__restrict__ us, double *__restrict__ vs,
                                                 double *__restrict__ ws, int do_main) {
  const int nxc = g.nxc, nyc = g.nyc, nz = g.nz;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < nxc * nyc; q += gridDim.x * kBlock) {
    const int i = q / nyc + 2, j = q % nyc + 2;
    const long long base = pidx(g, i, j, 0);
    if (do_main) {
      // every source value first (each line's ends lie 8 B x nz apart: the loads of all
      // four fields are in flight together), then the ghosts
      const double u2 = u[base + 2], v2 = v[base + 2], w2 = w[base + 2];
      const double uT = u[base + nz - 3], vT = v[base + nz - 3], wT = w[base + nz - 4];
      const double p2 = p ? p[base + 2] : 0.0, pT = p ? p[base + nz - 3] : 0.0;
      const double ub = t.dir[4][0] * 2. + (2.0 * t.num[4][0] - 1.0) * u2;
      const double vb = t.dir[4][1] * 2. + (2.0 * t.num[4][1] - 1.0) * v2;
      const double wb = t.dir[4][2] + t.num[4][2] * w2;
      const double wt = t.dir[5][2] + t.num[5][2] * wT;
      const double ut = t.dir[5][0] * 2. + (2.0 * t.num[5][0] - 1.0) * uT;
      const double vt = t.dir[5][1] * 2. + (2.0 * t.num[5][1] - 1.0) * vT;
      u[base + 1] = u[base + 0] = ub;
      v[base + 1] = v[base + 0] = vb;
      w[base + 1] = w[base + 0] = wb;
      w[base + nz - 1] = w[base + nz - 2] = w[base + nz - 3] = wt;
      u[base + nz - 1] = u[base + nz - 2] = ut;
      v[base + nz - 1] = v[base + nz - 2] = vt;
      if (p) {
        p[base + 1] = p[base + 0] = p2;
        p[base + nz - 2] = p[base + nz - 1] = pT;
      }
      if (us) {  // the copies of what this thread just wrote
        us[base + 0] = us[base + 1] = ub;
        us[base + nz - 2] = us[base + nz - 1] = ut;
        vs[base + 0] = vs[base + 1] = vb;
        vs[base + nz - 2] = vs[base + nz - 1] = vt;
        ws[base + 0] = ws[base + 1] = wb;
        ws[base + nz - 3] = ws[base + nz - 2] = ws[base + nz - 1] = wt;
      }
      continue;
    }
    if (us) {
      const int ku[4] = {0, 1, nz - 2, nz - 1};
#pragma unroll
      for (int a = 0; a < 4; ++a) { us[base + ku[a]] = u[base + ku[a]]; vs[base + ku[a]] = v[base + ku[a]]; }
      const int kw[5] = {0, 1, nz - 3, nz - 2, nz - 1};
#pragma unroll
      for (int a = 0; a < 5; ++a) ws[base + kw[a]] = w[base + kw[a]];
    }
  }
}

// inc/dfib/setEta.hpp:136-198: per (i,j) column, solid fraction at k = 0 by 100x100
// sub-sampling of cells within half a cell diagonal of the circle.  One warp per column:
// the lanes split the 100 sub-rows and the warp adds their integer counts (exact in any
// order), so a band column costs 400 sample tests per lane instead of 10000 in one thread.
__global__ void __launch_bounds__(kBlock) k_eta_plane(Geo g, const double *__restrict__ X,
                                                      const double *__restrict__ Y, double cx, double cy,
                                                      double R, double *__restrict__ eta) {
  const int nxc = g.nxc, nyc = g.nyc;
  const int lane = threadIdx.x & 31, wpb = kBlock / 32;
  for (long long q = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); q < (long long)nxc * nyc;
       q += (long long)gridDim.x * wpb) {
    const int i = (int)(q / nyc) + 2, j = (int)(q % nyc) + 2;
    const long long icel = pidx(g, i, j, 0);
    const double Diagonal = sqrt(g.Dx[i] * g.Dx[i] + g.Dy[j] * g.Dy[j]) * 0.5;
    const double ddx = ((X[i] + X[i + 1]) * 0.5) - cx;
    const double ddy = ((Y[j] + Y[j + 1]) * 0.5) - cy;
    const double Distance = sqrt(ddx * ddx + ddy * ddy);
    if (fabs(Distance - R) < Diagonal) {
      const int nsub = 100;
      const double dyg = g.Dy[j] / (double)nsub;
      const double dxg = g.Dx[i] / (double)nsub;
      unsigned xi = 0;
      for (int ii = lane; ii < nsub; ii += 32) {
        const double sx0 = X[i] + (double)ii * dxg, sx1 = X[i] + (double)(ii + 1) * dxg;
        const double a = (sx0 + sx1) * 0.5 - cx;
        for (int jj = 0; jj < nsub; ++jj) {
          const double sy0 = Y[j] + (double)jj * dyg, sy1 = Y[j] + (double)(jj + 1) * dyg;
          const double b = (sy0 + sy1) * 0.5 - cy;
          if (sqrt(a * a + b * b) <= R) ++xi;
        }
      }
      xi = __reduce_add_sync(0xffffffffu, xi);
      if (lane == 0) eta[icel] = (double)xi * (1.0 / ((double)nsub * (double)nsub));
    } else if (lane == 0) {
      eta[icel] = Distance > R ? 0. : 1.;
    }
  }
}

// setEta.hpp:200-203: copy plane k = 0 to k in [1, nz-1) for i < nx-1, j < ny-1
__global__ void __launch_bounds__(kBlock) k_eta_extrude(Geo g, double *__restrict__ eta) {
  const long long n = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 2);
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock) {
    const int k = (int)(q % (g.nz - 2)) + 1;
    const long long ij = q / (g.nz - 2);
    const int j = (int)(ij % (g.ny - 1)), i = (int)(ij / (g.ny - 1));
    eta[pidx(g, i, j, k)] = eta[pidx(g, i, j, 0)];
  }
}

// ---- launchers ----
template <bool AB>
static void convdiff_exact(cudaStream_t s, int nblk, const Geo &g, int scheme, double dt, double nu, const double *nut,
                           const double *u, const double *v, const double *w, double *us, double *vs, double *ws,
                           const StepCtl &sc) {
  if (scheme == CFDGB_LUD)
    k_convdiff_exact<CFDGB_LUD, AB><<<nblk, kBlock, 0, s>>>(g, dt, nu, nut, u, v, w, us, vs, ws, sc);
  else if (scheme == CFDGB_UD)
    k_convdiff_exact<CFDGB_UD, AB><<<nblk, kBlock, 0, s>>>(g, dt, nu, nut, u, v, w, us, vs, ws, sc);
  else
    k_convdiff_exact<CFDGB_QUICK, AB><<<nblk, kBlock, 0, s>>>(g, dt, nu, nut, u, v, w, us, vs, ws, sc);
}
void launch_convdiff_exact(cudaStream_t s, int nblk, const Geo &g, int scheme, double dt, double nu,
                           const double *nut, const double *u, const double *v, const double *w, double *us,
                           double *vs, double *ws, const StepCtl &sc) {
  if (sc.time_order > 1)
    convdiff_exact<true>(s, nblk, g, scheme, dt, nu, nut, u, v, w, us, vs, ws, sc);
  else
    convdiff_exact<false>(s, nblk, g, scheme, dt, nu, nut, u, v, w, us, vs, ws, sc);
}
void launch_smagorinsky(cudaStream_t s, int nblk, const Geo &g, const double *l2, const double *u, const double *v,
                        const double *w, double *nut) {
  k_smagorinsky<<<nblk, kBlock, 0, s>>>(g, l2, u, v, w, nut);
}
void launch_rhs_exact(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, const double *us,
                      const double *vs, const double *ws, int jacobi, const Stencil<double> &st, double *b) {
  k_rhs_exact<<<nblk, kBlock, 0, s>>>(g, dt, dtp, us, vs, ws, jacobi, st, b);
}
void launch_spmv_exact(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *x,
                       double *y) {
  k_spmv_exact<<<nblk, kBlock, 0, s>>>(g, st, x, y);
}
void launch_cfl(cudaStream_t s, int nblk, const Geo &g, double dt, const double *us, const double *vs,
                const double *ws, double *part, StepScal *ss) {
  StepCtl sc{};
  sc.ss = ss;
  sc.part = part;
  k_cfl<<<nblk, kBlock, 0, s>>>(g, dt, us, vs, ws, sc);
}
void launch_plot3d_pack(cudaStream_t s, int nblk, const Geo &g, const double *p, const double *u, const double *v,
                        const double *w, const double *eta, float *out) {
  k_plot3d_pack<<<nblk, kBlock, 0, s>>>(g, p, u, v, w, eta, out);
}
void launch_plot3d_unpack(cudaStream_t s, int nblk, const Geo &g, const float *in, double *p, double *u, double *v,
                          double *w, double *eta) {
  k_plot3d_unpack<<<nblk, kBlock, 0, s>>>(g, in, p, u, v, w, eta);
}
void launch_transform(cudaStream_t s, int nblk, const Geo &g, const double *x, double *p) {
  k_transform<<<nblk, kBlock, 0, s>>>(g, x, p);
}
void launch_update_uf_exact(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, int step_mode,
                            double lz, const double *eta, const double *p, const double *us, const double *vs,
                            const double *ws, double *u3, double *v3, double *w3, double *f, const double *ui,
                            const double *vi, const double *wi, double *part, StepScal *ss) {
  k_update_uf_exact<<<nblk, kBlock, 0, s>>>(g, dt, dtp, step_mode, lz, eta, p, us, vs, ws, u3, v3, w3, f, ui, vi,
                                            wi, part, ss);
}
void launch_bc(cudaStream_t s, const Geo &g, double *u, double *v, double *w, double *p, double *us,
               double *vs, double *ws, int do_main, const double *inlet, int conv, double *part, StepScal *ss,
               int nblk) {
  const BcTable t = flowpassing_table(g.walls);
  auto blocks = [](long long n) { return (int)((n + kBlock - 1) / kBlock < 1024 ? (n + kBlock - 1) / kBlock : 1024); };
  conv = conv && us;  // the last step's outlet values live in T1
  if (do_main && g.outflow) {
    const long long nf = (long long)g.nyc * g.nzc + (long long)g.nxc * g.nzc + (g.pz ? 0LL : (long long)g.nxc * g.nyc);
    const int fb = (int)std::min<long long>((nf + kBlock - 1) / kBlock, (long long)nblk);
    k_outflow_flux<<<fb, kBlock, 0, s>>>(g, t, inlet, u, v, w, conv ? us : nullptr, part, ss);
  }
  k_bc_x<<<blocks((long long)g.nyc * g.nzc), kBlock, 0, s>>>(g, t, inlet, u, v, w, p, us, vs, ws, do_main, conv, ss);
  k_bc_y<<<blocks((long long)g.nxc * g.nzc), kBlock, 0, s>>>(g, t, u, v, w, p, us, vs, ws, do_main);
  if (g.pz)
    k_bc_zp<<<blocks((long long)g.nx * g.ny), kBlock, 0, s>>>(g, u, v, w, p, us, vs, ws, do_main);
  else
    k_bc_z<<<blocks((long long)g.nxc * g.nyc), kBlock, 0, s>>>(g, t, u, v, w, p, us, vs, ws, do_main);
}
void launch_eta(cudaStream_t s, int nblk, const Geo &g, const double *X, const double *Y, double cx, double cy,
                double R, double *eta) {
  const long long cols = (long long)g.nxc * g.nyc;
  const int wpb = kBlock / 32;
  const int blocks = (int)std::min<long long>((cols + wpb - 1) / wpb, 65535LL * 8);
  k_eta_plane<<<blocks, kBlock, 0, s>>>(g, X, Y, cx, cy, R, eta);
  k_eta_extrude<<<nblk, kBlock, 0, s>>>(g, eta);
}

}  // namespace cfdgb

// ---- self-check of div_by against IEEE division (this file is built with -prec-div=true) ----
namespace cfdgb {
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void __launch_bounds__(kBlock) k_check_div(long long n, unsigned long long seed, double b, double y,
                                                      bool two, unsigned long long *bad) {
  unsigned long long miss = 0;
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock) {
    const unsigned long long h1 = mix64(seed ^ (unsigned long long)q), h2 = mix64(h1);
    double a;
    if (q % 1000 == 0) {
      a = (q % 2000 == 0) ? 0.0 : -0.0;
    } else if (q % 10 == 0) {
      a = b * (double)(long long)(h2 % 1000000);  // exact quotients
    } else {
      const double m = 1.0 + (double)(h1 >> 12) * 0x1.0p-52;  // [1, 2), 52 random bits
      a = scalbn(m, (int)(h2 % 81) - 40) * ((h2 >> 40) & 1 ? -1.0 : 1.0);
    }
    if (__double_as_longlong(a / b) != __double_as_longlong(div_by(a, b, y, two))) ++miss;
  }
  if (miss) atomicAdd(bad, miss);
}
}  // namespace cfdgb

extern "C" int cfdgb_check_division(long long n, uint64_t seed, double b, unsigned long long *mismatches) {
  using namespace cfdgb;
  if (!mismatches || n < 0 || !(b != 0.0) || !std::isfinite(b)) return CFDGB_EINVAL;
  unsigned long long *d = nullptr;
  if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return CFDGB_ECUDA;
  cudaMemset(d, 0, sizeof(*d));
  // the form the library uses for a context whose only divisor is b
  k_check_div<<<1216, kBlock>>>(n, seed, b, 1.0 / b, !div_certified(b), d);
  const cudaError_t e = cudaMemcpy(mismatches, d, sizeof(*d), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? CFDGB_OK : CFDGB_ECUDA;
}
