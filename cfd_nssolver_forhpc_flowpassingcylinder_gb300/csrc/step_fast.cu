// MIXED precision stencil sweep: QUICK convection-diffusion (the same discretisation as
// inc/source/Convection_Difussion.hpp:174) computed in FP32 on the FP64 state.  All
// divisions by the metric arrays are replaced by per-axis FP32 coefficient tables, so
// the per-cell work is FP32 FMAs; only the final u* = u + increment is FP64.
#include "cfdgb_internal.cuh"
#include "kernels.h"

namespace cfdgb {

// Per-axis table rows (each of length L = tab_len): see host_tables_f32 in api.cu.
enum TabRow { T_ID = 0, T_IDS, T_IT, T_AP1, T_AP2, T_AN1, T_AN2, T_BP1, T_BP2, T_BN1, T_BN2, T_NROW };

struct FastArgs {
  int L;  // table row length
  float dt, nu;
};

__device__ __forceinline__ float tb(const float *__restrict__ tab, int L, int axis, int row, int I) {
  return __ldg(tab + ((axis * T_NROW + row) * L + I));
}

// QUICK along the component's own axis (QuickUnitA, :20-51)
__device__ __forceinline__ void qa(float Up, float Un, float pp, float p, float c, float n, float nn,
                                   const float *tab, int L, int ax, int I, float &P, float &N) {
  const float iDm1 = tb(tab, L, ax, T_ID, I - 1), iD0 = tb(tab, L, ax, T_ID, I), iD1 = tb(tab, L, ax, T_ID, I + 1),
              iD2 = tb(tab, L, ax, T_ID, I + 2);
  P = 0.5f * (c + p) - (Up > 0.0f ? tb(tab, L, ax, T_AP1, I) * ((p - c) * iD1 - (c - n) * iD0)
                                  : tb(tab, L, ax, T_AP2, I) * ((pp - p) * iD2 - (p - c) * iD1));
  N = 0.5f * (n + c) - (Un > 0.0f ? tb(tab, L, ax, T_AN1, I) * ((c - n) * iD0 - (n - nn) * iDm1)
                                  : tb(tab, L, ax, T_AN2, I) * ((p - c) * iD1 - (c - n) * iD0));
}
// QUICK across (QuickUnitB, :55-90)
__device__ __forceinline__ void qb(float Up, float Un, float pp, float p, float c, float n, float nn,
                                   const float *tab, int L, int ax, int I, float &P, float &N) {
  const float iSm2 = tb(tab, L, ax, T_IDS, I - 2), iSm1 = tb(tab, L, ax, T_IDS, I - 1),
              iS0 = tb(tab, L, ax, T_IDS, I), iS1 = tb(tab, L, ax, T_IDS, I + 1);
  P = 0.5f * (c + p) - (Up > 0.0f ? tb(tab, L, ax, T_BP1, I) * ((p - c) * iS0 - (c - n) * iSm1)
                                  : tb(tab, L, ax, T_BP2, I) * ((pp - p) * iS1 - (p - c) * iS0));
  N = 0.5f * (n + c) - (Un > 0.0f ? tb(tab, L, ax, T_BN1, I) * ((c - n) * iSm1 - (n - nn) * iSm2)
                                  : tb(tab, L, ax, T_BN2, I) * ((p - c) * iS0 - (c - n) * iSm1));
}

// One staggered component whose own axis is A.  vel[0..2] = u, v, w.
template <int A>
__device__ __forceinline__ double component(const Geo &g, const FastArgs &fa, const float *__restrict__ tab,
                                            const double *__restrict__ const *vel, long long ic, const int (&I)[3]) {
  const long long s[3] = {g.sx, g.sy, 1};
  const double *phi = vel[A];
  auto ld = [&](long long q) { return (float)__ldg(phi + q); };
  const float c = ld(ic);
  float conv = 0.0f, diff = 0.0f;
  const float IT = tb(tab, fa.L, A, T_IT, I[A]);
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const long long sb = s[b];
    const int Ib = I[b];
    const float p = ld(ic + sb), n = ld(ic - sb), pp = ld(ic + 2 * sb), nn = ld(ic - 2 * sb);
    float P, N;
    if (b == A) {
      const float Up = 0.5f * (p + c), Un = 0.5f * (n + c);
      qa(Up, Un, pp, p, c, n, nn, tab, fa.L, b, Ib, P, N);
      conv += (P - N) * (P + N) * tb(tab, fa.L, b, T_IDS, Ib);
      diff += ((p - c) * tb(tab, fa.L, b, T_ID, Ib + 1) - (c - n) * tb(tab, fa.L, b, T_ID, Ib)) *
              tb(tab, fa.L, b, T_IDS, Ib);
    } else {
      // velocity normal to the b-faces of this control volume, interpolated along A
      const double *vb = vel[b];
      const float b0 = (float)__ldg(vb + ic), bA = (float)__ldg(vb + ic + s[A]);
      const float bm = (float)__ldg(vb + ic - sb), bmA = (float)__ldg(vb + ic - sb + s[A]);
      const float Bp = b0 + (bA - b0) * IT, Bn = bm + (bmA - bm) * IT;
      qb(Bp, Bn, pp, p, c, n, nn, tab, fa.L, b, Ib, P, N);
      conv += (P * Bp - N * Bn) * tb(tab, fa.L, b, T_ID, Ib);
      diff += ((p - c) * tb(tab, fa.L, b, T_IDS, Ib) - (c - n) * tb(tab, fa.L, b, T_IDS, Ib - 1)) *
              tb(tab, fa.L, b, T_ID, Ib);
    }
  }
  return (double)(fa.nu * fa.dt * diff - fa.dt * conv);
}

__global__ void __launch_bounds__(kBlock) k_convdiff_f32(Geo g, FastArgs fa, const float *__restrict__ tab,
                                                         const double *__restrict__ u, const double *__restrict__ v,
                                                         const double *__restrict__ w, double *__restrict__ us,
                                                         double *__restrict__ vs, double *__restrict__ ws) {
  const double *vel[3] = {u, v, w};
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < g.ncell;
       row += (long long)gridDim.x * kBlock) {
    int i, j, k;
    row_ijk(g, row, i, j, k);
    const long long ic = pidx(g, i, j, k);
    const int I[3] = {i, j, k};
    if (i < g.nx - 3) us[ic] = u[ic] + component<0>(g, fa, tab, vel, ic, I);
    if (j < g.ny - 3) vs[ic] = v[ic] + component<1>(g, fa, tab, vel, ic, I);
    if (k < g.nz - 3) ws[ic] = w[ic] + component<2>(g, fa, tab, vel, ic, I);
  }
}

void launch_convdiff_f32(cudaStream_t s, int nblk, const Geo &g, const float *tab, double dt, double nu,
                         const double *u, const double *v, const double *w, double *us, double *vs, double *ws) {
  FastArgs fa;
  fa.L = (g.nx > g.ny ? (g.nx > g.nz ? g.nx : g.nz) : (g.ny > g.nz ? g.ny : g.nz)) + 1;
  fa.dt = (float)dt;
  fa.nu = (float)nu;
  k_convdiff_f32<<<nblk, kBlock, 0, s>>>(g, fa, tab, u, v, w, us, vs, ws);
}

}  // namespace cfdgb
