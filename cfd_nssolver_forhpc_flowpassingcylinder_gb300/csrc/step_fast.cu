// MIXED precision step kernels.
//
// Stencil sweep: QUICK convection-diffusion (the same discretisation as
// inc/source/Convection_Difussion.hpp:174) computed in FP32 on FP32 copies of the FP64
// state.  All divisions by the metric arrays are replaced by per-axis FP32 coefficient
// tables, so the per-cell work is FP32 FMAs; only the final u* = u + increment is FP64.
// On this GPU the FP64 pipe runs at about 1/70 of the FP32 rate and also executes the
// FP64 <-> FP32 conversions, so the state is converted once per step (launch_mirror32,
// integer rounding) instead of once per neighbour read, and the increment is widened by
// integer operations (exact).
// Velocity correction: update_UandF with reciprocal multiplications and the DFIB
// arithmetic only on faces that touch the body.
#include <algorithm>

#include "cfdgb_internal.cuh"
#include "reduce.cuh"
#include "stepctl.cuh"
#include "kernels.h"

namespace cfdgb {

__global__ void __launch_bounds__(kBlock) k_mirror32(long long n, const double *__restrict__ u,
                                                     const double *__restrict__ v, const double *__restrict__ w,
                                                     float *__restrict__ u32, float *__restrict__ v32,
                                                     float *__restrict__ w32) {
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock) {
    u32[q] = d2f_int(u[q]);
    v32[q] = d2f_int(v[q]);
    w32[q] = d2f_int(w[q]);
  }
}

// Per-axis table rows (each of length L = tab_len): see host_tables_f32 in api.cu.
enum TabRow { T_ID = 0, T_IDS, T_IT, T_AP1, T_AP2, T_AN1, T_AN2, T_BP1, T_BP2, T_BN1, T_BN2, T_NROW };

struct FastArgs {
  int L;  // table row length
  float dt, nu;
  // a uniform grid's tables: every row is one value per axis, passed as kernel parameters
  // (the UNI kernel reads these instead of loading the table at every term)
  float uni[3][T_NROW];
};

// table entry (axis, row, I): the parameter of a uniform grid, else a load
template <bool UNI>
__device__ __forceinline__ float tb(const FastArgs &fa, const float *__restrict__ tab, int axis, int row, int I) {
  if (UNI) return fa.uni[axis][row];
  return __ldg(tab + ((axis * T_NROW + row) * fa.L + I));
}

// QUICK along the component's own axis (QuickUnitA, :20-51)
template <bool UNI>
__device__ __forceinline__ void qa(float Up, float Un, float pp, float p, float c, float n, float nn,
                                   const FastArgs &fa, const float *tab, int ax, int I, float &P, float &N) {
  const float iDm1 = tb<UNI>(fa, tab, ax, T_ID, I - 1), iD0 = tb<UNI>(fa, tab, ax, T_ID, I),
              iD1 = tb<UNI>(fa, tab, ax, T_ID, I + 1), iD2 = tb<UNI>(fa, tab, ax, T_ID, I + 2);
  P = 0.5f * (c + p) - (Up > 0.0f ? tb<UNI>(fa, tab, ax, T_AP1, I) * ((p - c) * iD1 - (c - n) * iD0)
                                  : tb<UNI>(fa, tab, ax, T_AP2, I) * ((pp - p) * iD2 - (p - c) * iD1));
  N = 0.5f * (n + c) - (Un > 0.0f ? tb<UNI>(fa, tab, ax, T_AN1, I) * ((c - n) * iD0 - (n - nn) * iDm1)
                                  : tb<UNI>(fa, tab, ax, T_AN2, I) * ((p - c) * iD1 - (c - n) * iD0));
}
// QUICK across (QuickUnitB, :55-90)
template <bool UNI>
__device__ __forceinline__ void qb(float Up, float Un, float pp, float p, float c, float n, float nn,
                                   const FastArgs &fa, const float *tab, int ax, int I, float &P, float &N) {
  const float iSm2 = tb<UNI>(fa, tab, ax, T_IDS, I - 2), iSm1 = tb<UNI>(fa, tab, ax, T_IDS, I - 1),
              iS0 = tb<UNI>(fa, tab, ax, T_IDS, I), iS1 = tb<UNI>(fa, tab, ax, T_IDS, I + 1);
  P = 0.5f * (c + p) - (Up > 0.0f ? tb<UNI>(fa, tab, ax, T_BP1, I) * ((p - c) * iS0 - (c - n) * iSm1)
                                  : tb<UNI>(fa, tab, ax, T_BP2, I) * ((pp - p) * iS1 - (p - c) * iS0));
  N = 0.5f * (n + c) - (Un > 0.0f ? tb<UNI>(fa, tab, ax, T_BN1, I) * ((c - n) * iSm1 - (n - nn) * iSm2)
                                  : tb<UNI>(fa, tab, ax, T_BN2, I) * ((p - c) * iS0 - (c - n) * iSm1));
}

// The FP32 increment of one staggered component whose own axis is A.  vel[0..2] = the FP32
// copies of u, v, w, each already offset to the cell; sx, sy the padded strides (the
// padded field is below 2^31 entries, so neighbour offsets are 32-bit).
template <int A, bool UNI>
__device__ __forceinline__ float component(const FastArgs &fa, const float *__restrict__ tab,
                                           const float *__restrict__ const *vel, int sx, int sy, const int (&I)[3]) {
  const int s[3] = {sx, sy, 1};
  const float *phi = vel[A];
  const float c = __ldg(phi);
  float conv = 0.0f, diff = 0.0f;
  const float IT = tb<UNI>(fa, tab, A, T_IT, I[A]);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const int sb = s[b];
    const int Ib = I[b];
    const float p = __ldg(phi + sb), n = __ldg(phi - sb), pp = __ldg(phi + 2 * sb), nn = __ldg(phi - 2 * sb);
    float P, N;
    if (b == A) {
      const float Up = 0.5f * (p + c), Un = 0.5f * (n + c);
      qa<UNI>(Up, Un, pp, p, c, n, nn, fa, tab, b, Ib, P, N);
      conv += (P - N) * (P + N) * tb<UNI>(fa, tab, b, T_IDS, Ib);
      diff += ((p - c) * tb<UNI>(fa, tab, b, T_ID, Ib + 1) - (c - n) * tb<UNI>(fa, tab, b, T_ID, Ib)) *
              tb<UNI>(fa, tab, b, T_IDS, Ib);
    } else {
      // velocity normal to the b-faces of this control volume, interpolated along A
      const float *vb = vel[b];
      const float b0 = __ldg(vb), bA = __ldg(vb + s[A]);
      const float bm = __ldg(vb - sb), bmA = __ldg(vb - sb + s[A]);
      const float Bp = b0 + (bA - b0) * IT, Bn = bm + (bmA - bm) * IT;
      qb<UNI>(Bp, Bn, pp, p, c, n, nn, fa, tab, b, Ib, P, N);
      conv += (P * Bp - N * Bn) * tb<UNI>(fa, tab, b, T_ID, Ib);
      diff += ((p - c) * tb<UNI>(fa, tab, b, T_IDS, Ib) - (c - n) * tb<UNI>(fa, tab, b, T_IDS, Ib - 1)) *
              tb<UNI>(fa, tab, b, T_ID, Ib);
    }
  }
  return fa.nu * fa.dt * diff - fa.dt * conv;
}

// FP32 CFL state of one thread: the sum u*/Dxs + v*/Dys + w*/Dzs per cell from the FP32
// u* (u32 + increment) and the FP32 reciprocals; the extremes of each component
struct CflAccF {
  float m[7] = {-3e38f, -1e10f, -1e10f, -1e10f, -1e10f, -1e10f, -1e10f};
  __device__ __forceinline__ void comp(int a, float x) {
    m[1 + a] = fmaxf(m[1 + a], x);
    m[4 + a] = fmaxf(m[4 + a], -x);
  }
};

template <bool UNI>
__global__ void __launch_bounds__(kBlock) k_convdiff_f32(Geo g, FastArgs fa, double dt_arg, const float *__restrict__ tab,
                                                         const double *__restrict__ u, const double *__restrict__ v,
                                                         const double *__restrict__ w, const float *__restrict__ u32,
                                                         const float *__restrict__ v32, const float *__restrict__ w32,
                                                         double *__restrict__ us, double *__restrict__ vs,
                                                         double *__restrict__ ws, StepCtl sc) {
  const double dt = step_dt(sc, dt_arg);
  fa.dt = (float)dt;
  const int sx = (int)g.sx, sy = (int)g.sy;
  CflAccF cfl;
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const int I[3] = {i, j, k};
    const float *vel[3] = {u32 + ic, v32 + ic, w32 + ic};
    float c = 0.0f;
    if (i < g.nx - 3) {
      const float d = component<0, UNI>(fa, tab, vel, sx, sy, I);
      us[ic] = u[ic] + f2d_int(d);
      const float r = u32[ic] + d;
      c += r * tb<UNI>(fa, tab, 0, T_IDS, i);
      cfl.comp(0, r);
    }
    if (j < g.ny - 3) {
      const float d = component<1, UNI>(fa, tab, vel, sx, sy, I);
      vs[ic] = v[ic] + f2d_int(d);
      const float r = v32[ic] + d;
      c += r * tb<UNI>(fa, tab, 1, T_IDS, j);
      cfl.comp(1, r);
    }
    if (k < g.nz - 3 + g.pz) {  // periodic z: the top face too
      const float d = component<2, UNI>(fa, tab, vel, sx, sy, I);
      ws[ic] = w[ic] + f2d_int(d);
      const float r = w32[ic] + d;
      c += r * tb<UNI>(fa, tab, 2, T_IDS, k);
      cfl.comp(2, r);
    }
    cfl.m[0] = fmaxf(cfl.m[0], c);
  }
  if (sc.ss) {
    CflAcc acc;
    for (int q = 0; q < 7; ++q) acc.m[q] = (double)cfl.m[q];
    cfl_finish(acc, dt, sc);
  }
}

// ---- transpose of k_convdiff_f32, for the adjoint of a MIXED context ----
// The FP32 stencil above, transposed with its own FP32 coefficients and upwind branches
// (the face velocities of the same FP32 copies), so that the adjoint is that of the step
// the MIXED forward ran.  The identity part of u* = u + increment adds lambda in FP64; the
// increment's part is computed in FP32 (dt times the stencil: ~0.1 of lambda per step),
// summed per target in registers and added to the FP64 adjoint fields with one FP64 atomic
// per target (converted exactly, by integer operations).
struct Face32 {
  float c[5];  // coefficients on offsets -2..+2 along the axis (two of them zero)
  float val;
};
__device__ __forceinline__ void face32(Face32 &F, int lo, float c0, float c1, float c2, const float *phi, int sb) {
#pragma unroll
  for (int o = 0; o < 5; ++o) F.c[o] = 0.0f;
  F.c[lo + 2] = c0;
  F.c[lo + 3] = c1;
  F.c[lo + 4] = c2;
  F.val = c0 * __ldg(phi + lo * sb) + c1 * __ldg(phi + (lo + 1) * sb) + c2 * __ldg(phi + (lo + 2) * sb);
}

template <int A, bool UNI>
__device__ __forceinline__ void adj_component32(const FastArgs &fa, const float *__restrict__ tab,
                                                const float *const *vel, double *const *lam, int sx, int sy,
                                                const int (&I)[3], float L, float (&own)[3]) {
  const int s[3] = {sx, sy, 1};
  const float *phi = vel[A];
  const float gc = -fa.dt * L, h = fa.nu * fa.dt * L;
  const float IT = tb<UNI>(fa, tab, A, T_IT, I[A]);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const int sb = s[b], Ib = I[b];
    float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    Face32 P, N;
    if (b == A) {
      const float iDm1 = tb<UNI>(fa, tab, b, T_ID, Ib - 1), iD0 = tb<UNI>(fa, tab, b, T_ID, Ib),
                  iD1 = tb<UNI>(fa, tab, b, T_ID, Ib + 1), iD2 = tb<UNI>(fa, tab, b, T_ID, Ib + 2);
      const float iS = tb<UNI>(fa, tab, b, T_IDS, Ib);
      const float ap = iD1 * iS, an = iD0 * iS;  // diffusion
      acc[3] += h * ap;
      acc[1] += h * an;
      acc[2] -= h * (ap + an);
      const float c = __ldg(phi), Up = 0.5f * (__ldg(phi + sb) + c), Un = 0.5f * (__ldg(phi - sb) + c);
      if (Up > 0.0f) {
        const float k = tb<UNI>(fa, tab, b, T_AP1, Ib);
        face32(P, -1, -k * iD0, 0.5f + k * iD1 + k * iD0, 0.5f - k * iD1, phi, sb);
      } else {
        const float k = tb<UNI>(fa, tab, b, T_AP2, Ib);
        face32(P, 0, 0.5f - k * iD1, 0.5f + k * iD2 + k * iD1, -k * iD2, phi, sb);
      }
      if (Un > 0.0f) {
        const float k = tb<UNI>(fa, tab, b, T_AN1, Ib);
        face32(N, -2, -k * iDm1, 0.5f + k * iD0 + k * iDm1, 0.5f - k * iD0, phi, sb);
      } else {
        const float k = tb<UNI>(fa, tab, b, T_AN2, Ib);
        face32(N, -1, 0.5f - k * iD0, 0.5f + k * iD1 + k * iD0, -k * iD1, phi, sb);
      }
      const float w = gc * iS;  // (P^2 - N^2) / Ds
      const float wP = w * 2.0f * P.val, wN = -w * 2.0f * N.val;
#pragma unroll
      for (int o = 0; o < 5; ++o) acc[o] = fmaf(wP, P.c[o], fmaf(wN, N.c[o], acc[o]));
    } else {
      const float iSm2 = tb<UNI>(fa, tab, b, T_IDS, Ib - 2), iSm1 = tb<UNI>(fa, tab, b, T_IDS, Ib - 1),
                  iS0 = tb<UNI>(fa, tab, b, T_IDS, Ib), iS1 = tb<UNI>(fa, tab, b, T_IDS, Ib + 1);
      const float iD = tb<UNI>(fa, tab, b, T_ID, Ib);
      const float ap = iS0 * iD, an = iSm1 * iD;  // diffusion
      acc[3] += h * ap;
      acc[1] += h * an;
      acc[2] -= h * (ap + an);
      const float *vb = vel[b];
      const int sA = s[A];
      const float b0 = __ldg(vb), bA = __ldg(vb + sA), bm = __ldg(vb - sb), bmA = __ldg(vb - sb + sA);
      const float Bp = b0 + (bA - b0) * IT, Bn = bm + (bmA - bm) * IT;
      if (Bp > 0.0f) {
        const float k = tb<UNI>(fa, tab, b, T_BP1, Ib);
        face32(P, -1, -k * iSm1, 0.5f + k * iS0 + k * iSm1, 0.5f - k * iS0, phi, sb);
      } else {
        const float k = tb<UNI>(fa, tab, b, T_BP2, Ib);
        face32(P, 0, 0.5f - k * iS0, 0.5f + k * iS1 + k * iS0, -k * iS1, phi, sb);
      }
      if (Bn > 0.0f) {
        const float k = tb<UNI>(fa, tab, b, T_BN1, Ib);
        face32(N, -2, -k * iSm2, 0.5f + k * iSm1 + k * iSm2, 0.5f - k * iSm1, phi, sb);
      } else {
        const float k = tb<UNI>(fa, tab, b, T_BN2, Ib);
        face32(N, -1, 0.5f - k * iSm1, 0.5f + k * iS0 + k * iSm1, -k * iS0, phi, sb);
      }
      const float w = gc * iD;  // (P Bp - N Bn) / D
      const float wP = w * Bp, wN = -w * Bn;
#pragma unroll
      for (int o = 0; o < 5; ++o) acc[o] = fmaf(wP, P.c[o], fmaf(wN, N.c[o], acc[o]));
      const float lBp = w * P.val, lBn = -w * N.val;  // the face velocities, interpolated along A
      own[b] += (1.0f - IT) * lBp;
      double *lvb = lam[b];
      atomicAdd(lvb + sA, f2d_int(IT * lBp));
      atomicAdd(lvb - sb, f2d_int((1.0f - IT) * lBn));
      atomicAdd(lvb - sb + sA, f2d_int(IT * lBn));
    }
    own[A] += acc[2];
#pragma unroll
    for (int o = 0; o < 5; ++o)
      if (o != 2 && acc[o] != 0.0f) atomicAdd(lam[A] + (o - 2) * sb, f2d_int(acc[o]));
  }
}

template <bool UNI>
__global__ void __launch_bounds__(kBlock) k_adj_convdiff_f32(Geo g, FastArgs fa, const float *__restrict__ tab,
                                                             const float *__restrict__ u32,
                                                             const float *__restrict__ v32,
                                                             const float *__restrict__ w32,
                                                             const double *__restrict__ lus,
                                                             const double *__restrict__ lvs,
                                                             const double *__restrict__ lws, double *lu, double *lv,
                                                             double *lw) {
  const int sx = (int)g.sx, sy = (int)g.sy;
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long c = pidx(g, i, j, k);
    const int I[3] = {i, j, k};
    const float *vel[3] = {u32 + c, v32 + c, w32 + c};
    double *lam[3] = {lu + c, lv + c, lw + c};
    const double L64[3] = {i < g.nx - 3 ? lus[c] : 0.0, j < g.ny - 3 ? lvs[c] : 0.0,
                           k < g.nz - 3 + g.pz ? lws[c] : 0.0};
    float own[3] = {0.0f, 0.0f, 0.0f};
    if (L64[0] != 0.0) adj_component32<0, UNI>(fa, tab, vel, lam, sx, sy, I, d2f_int(L64[0]), own);
    if (L64[1] != 0.0) adj_component32<1, UNI>(fa, tab, vel, lam, sx, sy, I, d2f_int(L64[1]), own);
    if (L64[2] != 0.0) adj_component32<2, UNI>(fa, tab, vel, lam, sx, sy, I, d2f_int(L64[2]), own);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double t = L64[a] + f2d_int(own[a]);  // u*_c = u_c + ...: lambda in FP64
      if (t != 0.0) atomicAdd(lam[a], t);
    }
  }
}

void launch_adj_convdiff_f32(cudaStream_t s, int nblk, const Geo &g, const float *tab, const float *uni, double dt,
                             double nu, const float *u32, const float *v32, const float *w32, const double *lus,
                             const double *lvs, const double *lws, double *lu, double *lv, double *lw) {
  FastArgs fa{};
  fa.L = (g.nx > g.ny ? (g.nx > g.nz ? g.nx : g.nz) : (g.ny > g.nz ? g.ny : g.nz)) + 1;
  fa.dt = (float)dt;
  fa.nu = (float)nu;
  if (uni) {
    for (int a = 0; a < 3; ++a)
      for (int r = 0; r < T_NROW; ++r) fa.uni[a][r] = uni[a * T_NROW + r];
    k_adj_convdiff_f32<true><<<nblk, kBlock, 0, s>>>(g, fa, tab, u32, v32, w32, lus, lvs, lws, lu, lv, lw);
  } else {
    k_adj_convdiff_f32<false><<<nblk, kBlock, 0, s>>>(g, fa, tab, u32, v32, w32, lus, lvs, lws, lu, lv, lw);
  }
}

// update_UandF (inc/dfib/updateUandF.hpp:90-180, solid velocity 0) for the MIXED mode:
// T2 = u* - (dt / Ds) (p+ - p) with the reciprocal metric, and the DFIB fraction, velocity
// and force only on faces where eta is non-zero on either side (elsewhere u = T2 and the
// force is zero); drag and lift summed as the exact kernel does.
// DFIB on a face next to the body (eta non-zero on either side): the forced value
// (1 - e) T2 and, when f is wanted, the face's force (n3 - T2) / dt dV.  Out of line, so
// that the branch stays a branch: the faces away from the body (all but a few per mille)
// then carry none of this FP64 work.
struct DfibFace {
  double n3, f;
};
// (the cell volume is formed inside, from the metric entries, so that none of it is
// evaluated ahead of the branch; dz null: no force wanted)
__device__ __noinline__ DfibFace dfib_face(double T2, double en, double ec, double hf, double rdt,
                                           const double *dx, const double *dy, const double *dz) {
  DfibFace r;
  const double e = fma(en - ec, hf, ec);
  r.n3 = (1.0 - e) * T2;
  r.f = dz ? (r.n3 - T2) * rdt * (*dx * *dy * *dz) : 0.0;
  return r;
}

template <bool UNI>
__global__ void __launch_bounds__(kBlock) k_update_uf_fast(
    Geo g, double dt_arg, const double *dtp, int step_mode, double lz, const double *__restrict__ eta,
    const double *__restrict__ p, const double *__restrict__ us, const double *__restrict__ vs,
    const double *__restrict__ ws, double *__restrict__ u3, double *__restrict__ v3, double *__restrict__ w3,
    const double *__restrict__ ui, const double *__restrict__ vi, const double *__restrict__ wi, double *part,
    StepScal *ss) {
  const double dt = dtp ? *dtp : dt_arg;
  const double rdt = 1.0 / dt;
  auto nonzero = [](double e) { return (__double_as_longlong(e) << 1) != 0; };  // +-0 is zero
  // UNI: -dt / Ds per axis once per thread (a uniform grid: the same product at every index)
  double gx = 0.0, gy = 0.0, gz = 0.0;
  if (UNI) {
    gx = -(dt * g.rDxs[2]);
    gy = -(dt * g.rDys[2]);
    gz = -(dt * g.rDzs[2]);
  }
  double acc[2] = {0.0, 0.0};
#pragma unroll 2
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const double ec = eta[ic];
    const bool bc = nonzero(ec);
    if (i < g.nx - 3) {
      const long long icP = ic + g.sx;
      const double T2 = fma(UNI ? gx : -(dt * g.rDxs[i]), p[icP] - p[ic], us[ic]);
      const double en = eta[icP];
      double n3 = T2;
      if (bc || nonzero(en)) {
        const DfibFace d = dfib_face(T2, en, ec, g.hfx[i], rdt, g.Dx + i, g.Dy + j, g.Dz + k);
        n3 = d.n3;
        acc[0] += d.f;
      }
      u3[ic] = n3;
    } else if (ui) {
      u3[ic] = ui[ic];
    }
    if (j < g.ny - 3) {
      const long long icP = ic + g.sy;
      const double T2 = fma(UNI ? gy : -(dt * g.rDys[j]), p[icP] - p[ic], vs[ic]);
      const double en = eta[icP];
      double n3 = T2;
      if (bc || nonzero(en)) {
        const DfibFace d = dfib_face(T2, en, ec, g.hfy[j], rdt, g.Dx + i, g.Dy + j, g.Dz + k);
        n3 = d.n3;
        acc[1] += d.f;
      }
      v3[ic] = n3;
    } else if (vi) {
      v3[ic] = vi[ic];
    }
    if (k < g.nz - 3 + g.pz) {  // periodic z: the top face, its upper cell the first one
      const long long icP = (g.pz && k == g.nz - 3) ? ic - (g.nzc - 1) : ic + 1;
      const double T2 = fma(UNI ? gz : -(dt * g.rDzs[k]), p[icP] - p[ic], ws[ic]);
      const double en = eta[icP];
      w3[ic] = (bc || nonzero(en)) ? dfib_face(T2, en, ec, g.hfz[k], rdt, nullptr, nullptr, nullptr).n3 : T2;
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
    step_end(ss, dt, step_mode);
  }
}

// createBMatrix_omp (inc/matrix/b_matrix.hpp:35-98) for the MIXED mode: b = -(jp)(1/dt)
// div(u*) with the reciprocal metrics (multiplications, not the reference's divisions)
__global__ void __launch_bounds__(kBlock) k_rhs_fast(Geo g, double dt_arg, const double *dtp,
                                                     const double *__restrict__ us, const double *__restrict__ vs,
                                                     const double *__restrict__ ws, int jacobi, Stencil<double> st,
                                                     double *__restrict__ b) {
  const double ndt = -1.0 / (dtp ? *dtp : dt_arg);
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const long long zb = (g.pz && k == 2) ? ic + g.nzc - 1 : ic - 1;  // periodic z: face nz-3
    const double div = fma(us[ic] - us[ic - g.sx], g.rDx[i],
                           fma(vs[ic] - vs[ic - g.sy], g.rDy[j], (ws[ic] - ws[zb]) * g.rDz[k]));
    b[row] = (jacobi ? row_jp(g, st, i - 2, j - 2, k - 2, row) * ndt : ndt) * div;
  }
}

void launch_rhs_fast(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, const double *us,
                     const double *vs, const double *ws, int jacobi, const Stencil<double> &st, double *b) {
  k_rhs_fast<<<nblk, kBlock, 0, s>>>(g, dt, dtp, us, vs, ws, jacobi, st, b);
}

void launch_convdiff_f32(cudaStream_t s, int nblk, const Geo &g, const float *tab, const float *uni, double dt,
                         double nu, const double *u, const double *v, const double *w, const float *u32,
                         const float *v32, const float *w32, double *us, double *vs, double *ws, const StepCtl &sc) {
  FastArgs fa{};
  fa.L = (g.nx > g.ny ? (g.nx > g.nz ? g.nx : g.nz) : (g.ny > g.nz ? g.ny : g.nz)) + 1;
  fa.dt = (float)dt;
  fa.nu = (float)nu;
  if (uni) {
    for (int a = 0; a < 3; ++a)
      for (int r = 0; r < T_NROW; ++r) fa.uni[a][r] = uni[a * T_NROW + r];
    k_convdiff_f32<true><<<nblk, kBlock, 0, s>>>(g, fa, dt, tab, u, v, w, u32, v32, w32, us, vs, ws, sc);
  } else {
    k_convdiff_f32<false><<<nblk, kBlock, 0, s>>>(g, fa, dt, tab, u, v, w, u32, v32, w32, us, vs, ws, sc);
  }
}

void launch_mirror32(cudaStream_t s, const Geo &g, const double *u, const double *v, const double *w, float *u32,
                     float *v32, float *w32) {
  const long long n = (long long)g.nx * g.ny * g.nz;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = std::min<long long>((n + kBlock - 1) / kBlock, (long long)nsm * 8);
  k_mirror32<<<(int)blocks, kBlock, 0, s>>>(n, u, v, w, u32, v32, w32);
}

void launch_update_uf_fast(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, int step_mode,
                           double lz, const double *eta, const double *p, const double *us, const double *vs,
                           const double *ws, double *u3, double *v3, double *w3, const double *ui, const double *vi,
                           const double *wi, double *part, StepScal *ss) {
  if (g.uni)
    k_update_uf_fast<true><<<nblk, kBlock, 0, s>>>(g, dt, dtp, step_mode, lz, eta, p, us, vs, ws, u3, v3, w3, ui, vi,
                                                   wi, part, ss);
  else
    k_update_uf_fast<false><<<nblk, kBlock, 0, s>>>(g, dt, dtp, step_mode, lz, eta, p, us, vs, ws, u3, v3, w3, ui,
                                                    vi, wi, part, ss);
}

}  // namespace cfdgb
