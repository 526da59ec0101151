// Pressure Poisson solvers on the 7-point Neumann operator.
//
// BiCGSTAB follows bicgstabRe2::solve (inc/solver/bicgstabRe2.hpp:84-180) step for step:
// warm start, relative-residual stop, rho restart, iteration cap and NaN recovery.  Every
// global dot product is a deterministic two-stage FP64 reduction (reduce.cuh) whose last
// block also makes the scalar decisions (alpha, omega, stop test, beta, restart), so no
// host round trip happens inside an iteration.  Every kernel returns at once when
// sc->done is set, which lets the host enqueue iterations in chunks (captured as CUDA
// graphs) and poll only between chunks.
//
// Launch geometry: 3-D blocks (bx along k, by along j) with the grid's z dimension
// striding over i, so each thread knows its (i, j, k) without a division.
//
// FP64 (the plain path, bound by the FP64 pipe): five kernels per iteration, no
// recomputation.  FP32 (inner solve of the mixed path, bound by HBM): three kernels per
// iteration; the p update is fused into the next SpMV and s into its SpMV by
// recomputing them at the stencil points (L1-resident), 17 instead of 19 words per cell.
#include <algorithm>

#include "cfdgb_internal.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace cfdgb {

// (ic, jc, kc) of this thread and the loop over the i planes it owns.
#define FOR_CELLS(g)                                               \
  const int kc = blockIdx.x * blockDim.x + threadIdx.x;            \
  const int jc = blockIdx.y * blockDim.y + threadIdx.y;            \
  const bool on_ = (kc < (g).nzc) && (jc < (g).nyc);               \
  for (int ic = blockIdx.z; on_ && ic < (g).nxc; ic += gridDim.z)

// the same, four planes of a thread's column in flight at once (short bodies that stream)
#define FOR_CELLS4(g)                                              \
  const int kc = blockIdx.x * blockDim.x + threadIdx.x;            \
  const int jc = blockIdx.y * blockDim.y + threadIdx.y;            \
  const bool on_ = (kc < (g).nzc) && (jc < (g).nyc);               \
  _Pragma("unroll 4") for (int ic = blockIdx.z; on_ && ic < (g).nxc; ic += gridDim.z)

#define ROW(g) ((((long long)ic * (g).nyc + jc) * (g).nzc) + kc)

__device__ __forceinline__ int cls_of(const Geo &g, int ic, int jc, int kc) { return row_class(g, ic, jc, kc); }

// y = (A f)(row) where f(q) is evaluated on demand at the stencil points
template <typename T, class F>
__device__ __forceinline__ T stencil_apply(const Geo &g, const Stencil<T> &st, int ic, int jc, int kc,
                                           long long row, F &&f, T &center) {
  const long long nyz = (long long)g.nyc * g.nzc;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (g.nonuni) {  // stretched grid (FP64 solvers only): the rows stored per context
      const double *__restrict__ cs = g.cof[st.jac] + row;
      const long long n = g.ncell, zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
      T sum = T(0);
      if (ic > 0) sum += cs[0] * f(row - nyz);
      if (jc > 0) sum += cs[n] * f(row - g.nzc);
      if (zm >= 0) sum += cs[2 * n] * f(zm);
      center = f(row);
      sum += cs[3 * n] * center;
      if (zp >= 0) sum += cs[4 * n] * f(zp);
      if (jc < g.nyc - 1) sum += cs[5 * n] * f(row + g.nzc);
      if (ic < g.nxc - 1) sum += cs[6 * n] * f(row + nyz);
      return sum;
    }
  }
  const T *c = st.c[cls_of(g, ic, jc, kc)];
  const long long zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
  T sum = T(0);
  if (ic > 0) sum += c[0] * f(row - nyz);
  if (jc > 0) sum += c[1] * f(row - g.nzc);
  if (zm >= 0) sum += c[2] * f(zm);
  center = f(row);
  sum += c[3] * center;
  if (zp >= 0) sum += c[4] * f(zp);
  if (jc < g.nyc - 1) sum += c[5] * f(row + g.nzc);
  if (ic < g.nxc - 1) sum += c[6] * f(row + nyz);
  return sum;
}

// FP32 form of the same operator: every row sums to zero (Neumann rows: the diagonal is
// minus the sum of the neighbour coefficients), so A f = sum_nb c_nb (f_nb - f_centre).
// Differencing first makes A exactly singular on constants in FP32 and keeps the rounding
// error proportional to the local differences rather than to |f|: on the smooth modes that
// dominate late in a solve, the plain 7-term sum would lose ~eps32 * cond(A) (~1e-2 at
// 512 cells per axis) and stall the iteration there.
template <class F>
__device__ __forceinline__ float stencil_apply_diff(const Geo &g, const Stencil<float> &st, int ic, int jc, int kc,
                                                    long long row, F &&f, float &center) {
  const long long nyz = (long long)g.nyc * g.nzc;
  const long long zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
  const float fc = f(row);
  center = fc;
  float sum = 0.0f;
  if (g.nonuni) {  // stretched grid (MIXED): its rows stored in FP32, [7][ncell]
    const float *__restrict__ cs = g.cof32[st.jac] + row;
    const long long n = g.ncell;
    if (ic > 0) sum = fmaf(cs[0], f(row - nyz) - fc, sum);
    if (jc > 0) sum = fmaf(cs[n], f(row - g.nzc) - fc, sum);
    if (zm >= 0) sum = fmaf(cs[2 * n], f(zm) - fc, sum);
    if (zp >= 0) sum = fmaf(cs[4 * n], f(zp) - fc, sum);
    if (jc < g.nyc - 1) sum = fmaf(cs[5 * n], f(row + g.nzc) - fc, sum);
    if (ic < g.nxc - 1) sum = fmaf(cs[6 * n], f(row + nyz) - fc, sum);
    return sum;
  }
  const float *c = st.c[cls_of(g, ic, jc, kc)];
  if (ic > 0) sum = fmaf(c[0], f(row - nyz) - fc, sum);
  if (jc > 0) sum = fmaf(c[1], f(row - g.nzc) - fc, sum);
  if (zm >= 0) sum = fmaf(c[2], f(zm) - fc, sum);
  if (zp >= 0) sum = fmaf(c[4], f(zp) - fc, sum);
  if (jc < g.nyc - 1) sum = fmaf(c[5], f(row + g.nzc) - fc, sum);
  if (ic < g.nxc - 1) sum = fmaf(c[6], f(row + nyz) - fc, sum);
  return sum;
}

// b - (A x)(row) as one FMA chain from b, the terms in stencil_apply's order (the MIXED
// refinement's residual: FP64-pipe-bound, so the subtraction folds into the chain)
__device__ __forceinline__ double resid_at(const Geo &g, const Stencil<double> &st, const double *__restrict__ x, int ic,
                                          int jc, int kc, long long row, double bb) {
  const long long nyz = (long long)g.nyc * g.nzc;
  const long long zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
  double r = bb;
  if (g.nonuni) {  // stretched grid: the rows stored per context
    const double *__restrict__ cs = g.cof[st.jac] + row;
    const long long n = g.ncell;
    if (ic > 0) r = fma(-cs[0], x[row - nyz], r);
    if (jc > 0) r = fma(-cs[n], x[row - g.nzc], r);
    if (zm >= 0) r = fma(-cs[2 * n], x[zm], r);
    r = fma(-cs[3 * n], x[row], r);
    if (zp >= 0) r = fma(-cs[4 * n], x[zp], r);
    if (jc < g.nyc - 1) r = fma(-cs[5 * n], x[row + g.nzc], r);
    if (ic < g.nxc - 1) r = fma(-cs[6 * n], x[row + nyz], r);
    return r;
  }
  const double *c = st.c[cls_of(g, ic, jc, kc)];
  if (ic > 0) r = fma(-c[0], x[row - nyz], r);
  if (jc > 0) r = fma(-c[1], x[row - g.nzc], r);
  if (zm >= 0) r = fma(-c[2], x[zm], r);
  r = fma(-c[3], x[row], r);
  if (zp >= 0) r = fma(-c[4], x[zp], r);
  if (jc < g.nyc - 1) r = fma(-c[5], x[row + g.nzc], r);
  if (ic < g.nxc - 1) r = fma(-c[6], x[row + nyz], r);
  return r;
}

template <typename T>
__device__ __forceinline__ T spmv_at(const Geo &g, const Stencil<T> &st, const T *__restrict__ x, int ic, int jc,
                                     int kc, long long row) {
  T c;
  return stencil_apply<T>(g, st, ic, jc, kc, row, [&](long long q) { return x[q]; }, c);
}

// ---- FP64 set-up: bicgstabRe2.hpp:86-106 ----
// restart: 1 for the preconditioned iteration, whose first p kernel then takes p = r0 = r1
__global__ void __launch_bounds__(kBlock) k_bicg_setup64(Geo g, Stencil<double> st, KrylovVecs<double> v,
                                                          const double *__restrict__ b, double *px1, double *px2,
                                                          double *part, SolverScal *sc, int restart) {
  double acc[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double bb = b[row];
    const double r = bb - spmv_at<double>(g, st, v.x, ic, jc, kc, row);
    v.r0[row] = r;
    v.r1[row] = r;
    v.p1[row] = r;
    px2[row] = px1[row];
    px1[row] = v.x[row];
    acc[0] += bb * bb;
    acc[1] += r * r;
  }
  double out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[0], out) && lin_tid() == 0) {
    sc->timestep += 1;
    sc->norm0 = sqrt(out[0]);
    sc->rho = out[1];
    sc->iter = 0;
    sc->done = 0;
    sc->status = 0;
    sc->restart = restart;
    sc->relres = 0.0;
  }
}

// ---- FP64 iteration: five kernels ----
// K1: ap = A p1, alpha = rho / <ap, r0>
__global__ void __launch_bounds__(kBlock) k64_ap(Geo g, Stencil<double> st, KrylovVecs<double> v, double *part,
                                                 SolverScal *sc) {
  if (sc->done) return;
  double a[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double y = spmv_at<double>(g, st, v.p1, ic, jc, kc, row);
    v.ap[row] = y;
    a[0] += y * v.r0[row];
  }
  double out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

// K2: s = r1 - alpha ap
__global__ void __launch_bounds__(kBlock) k64_s(Geo g, KrylovVecs<double> v, const SolverScal *sc) {
  if (sc->done) return;
  const double a = sc->alpha;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.s[row] = v.r1[row] - a * v.ap[row];
  }
}

// K3: as = A s, omega = <as, s> / <as, as>
__global__ void __launch_bounds__(kBlock) k64_as(Geo g, Stencil<double> st, KrylovVecs<double> v, double *part,
                                                 SolverScal *sc) {
  if (sc->done) return;
  double a[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double y = spmv_at<double>(g, st, v.s, ic, jc, kc, row);
    v.as[row] = y;
    a[0] += y * v.s[row];
    a[1] += y * y;
  }
  double out[2];
  if (grid_sum<2>(a, part, &sc->cnt[2], out) && lin_tid() == 0) sc->omega = out[0] / out[1];
}

// stop test, beta and restart decision of bicgstabRe2.hpp:128-176 (last block, thread 0);
// n2 = ||r1||^2, rr = <r1, r0>
template <bool FP32>
__device__ __forceinline__ void finish_iteration(SolverScal *sc, double n2, double rr) {
  const double relres = sqrt(n2) / sc->norm0;
  sc->relres = relres;
  if (FP32) {
    // MIXED sweep: hand over to the FP64 refinement once the residual has dropped by delta
    // below the sweep's start, or by peak below the sweep's largest one (BiCGSTAB's
    // residual can rise far above its start before it falls, and an FP32 recursion cannot
    // follow it down many decades below such a peak), or looks converged
    const double rn = sqrt(n2);
    if (relres < sc->best) sc->best = relres;
    // keep this iterate (the next x update copies it) once its residual has halved since
    // the last one kept: a few copies per sweep, and the sweep's correction is never worse
    // than that kept iterate, whatever the residual does afterwards
    sc->snap = relres <= 0.5 * sc->snap_rel;
    if (sc->snap) sc->snap_rel = relres;
    if (!isfinite(relres)) {
      sc->done = 1;
      sc->status = CFDGB_ENAN;
    } else if (sc->iter > 16 && relres > 1e3 * sc->best) {
      // runaway growth (BiCGSTAB's ordinary bumps stay far below this)
      sc->done = 1;
      sc->status = CFDGB_ENOCONV;
    } else if (sc->iter >= sc->maxit) {
      sc->done = 1;
      sc->status = CFDGB_ENOCONV;
      sc->iter += 1;
    } else if (relres < sc->tol || rn < sc->delta * sc->rstart || rn < sc->peak * sc->rmax) {
      sc->done = 1;
      sc->status = kStatusRefine;
      sc->iter += 1;
    } else {
      const double rho_old = sc->rho;
      sc->rho = rr;
      sc->beta = (sc->alpha / sc->omega) * (rr / rho_old);
      sc->restart = 0;
      if (!(isfinite(sc->beta) && sc->omega != 0.0 && rr != 0.0)) {  // Lanczos breakdown
        sc->restart = 1;
        sc->rho = n2;
      }
      sc->rmax = fmax(sc->rmax, rn);
      sc->iter += 1;
    }
    return;
  }
  if (relres < sc->tol) {  // :129
    sc->done = 1;
  } else if (sc->iter >= sc->maxit) {  // :133
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
  } else {  // :156-176
    const double rho_old = sc->rho;
    sc->rho = rr;
    sc->beta = (sc->alpha / sc->omega) * (sc->rho / rho_old);
    sc->restart = !(sc->timestep < 10 || fabs(rho_old) > sc->restart_thr);
    sc->iter += 1;
  }
}

// K4: x += alpha p1 + omega s; r1 = s - omega as; ||r1||^2, <r1, r0>
__global__ void __launch_bounds__(kBlock) k64_xr(Geo g, KrylovVecs<double> v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const double a = sc->alpha, w = sc->omega;
  double acc[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double s = v.s[row];
    v.x[row] = fma(w, s, fma(a, v.p1[row], v.x[row]));  // two FP64 ops instead of three
    const double r1 = fma(-w, v.as[row], s);
    v.r1[row] = r1;
    acc[0] += r1 * r1;
    acc[1] += r1 * v.r0[row];
  }
  double out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) finish_iteration<false>(sc, out[0], out[1]);
}

// K5: p1 = r1 + beta (p1 - omega ap), or restart r0 = p1 = r1
__global__ void __launch_bounds__(kBlock) k64_p(Geo g, KrylovVecs<double> v, const SolverScal *sc) {
  if (sc->done) return;
  const double b = sc->beta, w = sc->omega;
  const bool rst = sc->restart != 0;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double r1 = v.r1[row];
    if (rst) {
      v.r0[row] = r1;
      v.p1[row] = r1;
    } else {
      v.p1[row] = r1 + b * (v.p1[row] - w * v.ap[row]);
    }
  }
}

// ---- FP32 iteration: three fused kernels; p and ap are double-buffered by parity ----
struct Vec32 {
  float *x, *r0, *r1, *s, *as, *p[2], *ap[2];
  float *xb;  // best iterate of the BiCGSTAB sweep (xr kernels keep it)
};

// p_new = r1 + beta (p_old - omega ap_old) (or r1 on restart, which also sets r0 = r1),
// evaluated at the stencil points; ap_new = A p_new; alpha = rho / <ap_new, r0>
__global__ void __launch_bounds__(kBlock) k32_pap(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                  SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float b = (float)sc->beta, w = (float)sc->omega;
  const bool rst = sc->restart != 0;
  const float *__restrict__ po = (parity ? v.p[1] : v.p[0]);
  const float *__restrict__ apo = (parity ? v.ap[1] : v.ap[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  float *__restrict__ apn = (parity ? v.ap[0] : v.ap[1]);
  const float *__restrict__ r1 = v.r1;
  AccF acc;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    float pc;
    const float y = rst ? stencil_apply_diff(g, st, ic, jc, kc, row, [&](long long q) { return r1[q]; }, pc)
                        : stencil_apply_diff(g, st, ic, jc, kc, row,
                                               [&](long long q) { return r1[q] + b * (po[q] - w * apo[q]); }, pc);
    pn[row] = pc;
    apn[row] = y;
    float r0 = v.r0[row];
    if (rst) {
      r0 = r1[row];
      v.r0[row] = r0;
    }
    acc.add(y * r0);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

// s = r1 - alpha ap at the stencil points; as = A s; omega = <as, s> / <as, as>
__global__ void __launch_bounds__(kBlock) k32_sas(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                  SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float a = (float)sc->alpha;
  const float *__restrict__ ap = (parity ? v.ap[0] : v.ap[1]);
  const float *__restrict__ r1 = v.r1;
  AccF a0, a1;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    float sc_;
    const float y = stencil_apply_diff(g, st, ic, jc, kc, row, [&](long long q) { return r1[q] - a * ap[q]; }, sc_);
    v.s[row] = sc_;
    v.as[row] = y;
    a0.add(y * sc_);
    a1.add(y * y);
  }
  double acc[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    // s has vanished: the half step solved the system; omega = 0 makes the next kernel
    // take x += alpha p, r1 = s and stop instead of forming 0/0
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;
    sc->omega = wv;
  }
}

// x += alpha p + omega s; r1 = s - omega as; stop test, beta, restart
__global__ void __launch_bounds__(kBlock) k32_xr(Geo g, Vec32 v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float a = (float)sc->alpha, w = (float)sc->omega;
  const float *__restrict__ p = (parity ? v.p[0] : v.p[1]);
  const bool keep = sc->snap != 0;  // the current x is the iterate to keep
  AccF n2, rr;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const float s = v.s[row];
    const float x = v.x[row];
    if (keep) v.xb[row] = x;
    v.x[row] = fmaf(w, s, fmaf(a, p[row], x));
    const float r1 = fmaf(-w, v.as[row], s);
    v.r1[row] = r1;
    n2.add(r1 * r1);
    rr.add(r1 * v.r0[row]);
  }
  double acc[2] = {n2.get(), rr.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) {
    sc->par ^= 1;  // this iteration's p and ap become the previous ones
    finish_iteration<true>(sc, out[0], out[1]);
  }
}

// ---- FP32 BiCGSTAB with a right preconditioner (the multigrid V-cycle, multigrid.cu) ----
// The iteration of bicgstabRe2 on A M y = r with x = M y: p and s are preconditioned
// (ph = M p, sh = M s) before each operator application and the update of x, while r, s,
// and the stop test stay on the unpreconditioned residual.  Same device scalars and
// decisions as the plain FP32 sweep (finish_iteration<true>), counters 1-3 as there.

// p = r1 + beta (p - omega v), or p = r0 = r1 on restart
__global__ void __launch_bounds__(kBlock) k32p_p(Geo g, PrecVecs v, const SolverScal *sc) {
  if (sc->done) return;
  const float b = (float)sc->beta, w = (float)sc->omega;
  const bool rst = sc->restart != 0;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const float r1 = v.r1[row];
    if (rst) {
      v.r0[row] = r1;
      v.p[row] = r1;
    } else {
      v.p[row] = r1 + b * (v.p[row] - w * v.v[row]);
    }
  }
}

// v = A ph, alpha = rho / <v, r0>
__global__ void __launch_bounds__(kBlock) k32p_v(Geo g, Stencil<float> st, PrecVecs v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const float *__restrict__ ph = v.ph;
  AccF acc;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    float c;
    const float y = stencil_apply_diff(g, st, ic, jc, kc, row, [&](long long q) { return ph[q]; }, c);
    v.v[row] = y;
    acc.add(y * v.r0[row]);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

// s = r1 - alpha v
__global__ void __launch_bounds__(kBlock) k32p_s(Geo g, PrecVecs v, const SolverScal *sc) {
  if (sc->done) return;
  const float a = (float)sc->alpha;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.s[row] = fmaf(-a, v.v[row], v.r1[row]);
  }
}

// t = A sh, omega = <t, s> / <t, t> (0 when t vanishes, as in k32_sas)
__global__ void __launch_bounds__(kBlock) k32p_t(Geo g, Stencil<float> st, PrecVecs v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const float *__restrict__ sh = v.sh;
  AccF a0, a1;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    float c;
    const float y = stencil_apply_diff(g, st, ic, jc, kc, row, [&](long long q) { return sh[q]; }, c);
    v.t[row] = y;
    a0.add(y * v.s[row]);
    a1.add(y * y);
  }
  double acc[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;
    sc->omega = wv;
  }
}

// x += alpha ph + omega sh; r1 = s - omega t; stop test, beta, restart
__global__ void __launch_bounds__(kBlock) k32p_xr(Geo g, PrecVecs v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const float a = (float)sc->alpha, w = (float)sc->omega;
  const bool keep = sc->snap != 0;
  AccF n2, rr;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const float x = v.x[row];
    if (keep) v.xb[row] = x;
    v.x[row] = fmaf(w, v.sh[row], fmaf(a, v.ph[row], x));
    const float r1 = fmaf(-w, v.t[row], v.s[row]);
    v.r1[row] = r1;
    n2.add(r1 * r1);
    rr.add(r1 * v.r0[row]);
  }
  double acc[2] = {n2.get(), rr.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) finish_iteration<true>(sc, out[0], out[1]);
}

// ---- FP64 BiCGSTAB with the FP64 V-cycle as right preconditioner ----
// The FP32 preconditioned iteration above in FP64 (the like-for-like FP64 counterpart of
// the MIXED multigrid sweep): same kernels and order, FP64 vectors and dots.  Not the
// reference's iteration, so no rho-restart rule: it stops on the tolerance, the cap or a
// non-finite residual, and restarts only on a Lanczos breakdown.
__device__ __forceinline__ void finish_prec64(SolverScal *sc, double n2, double rr) {
  const double relres = sqrt(n2) / sc->norm0;
  sc->relres = relres;
  sc->iter += 1;
  if (!isfinite(relres)) {
    sc->done = 1;
    sc->status = CFDGB_ENAN;
  } else if (relres < sc->tol) {
    sc->done = 1;
  } else if (sc->iter >= sc->maxit) {
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
  } else {
    const double rho_old = sc->rho;
    sc->rho = rr;
    sc->beta = (sc->alpha / sc->omega) * (rr / rho_old);
    sc->restart = 0;
    if (!(isfinite(sc->beta) && sc->omega != 0.0 && rr != 0.0)) {
      sc->restart = 1;
      sc->rho = n2;
    }
  }
}

__global__ void __launch_bounds__(kBlock) k64p_p(Geo g, PrecVecsT<double> v, const SolverScal *sc) {
  if (sc->done) return;
  const double b = sc->beta, w = sc->omega;
  const bool rst = sc->restart != 0;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double r1 = v.r1[row];
    if (rst) {
      v.r0[row] = r1;
      v.p[row] = r1;
    } else {
      v.p[row] = fma(b, fma(-w, v.v[row], v.p[row]), r1);
    }
  }
}

__global__ void __launch_bounds__(kBlock) k64p_v(Geo g, Stencil<double> st, PrecVecsT<double> v, double *part,
                                                 SolverScal *sc) {
  if (sc->done) return;
  double a[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double y = spmv_at<double>(g, st, v.ph, ic, jc, kc, row);
    v.v[row] = y;
    a[0] = fma(y, v.r0[row], a[0]);
  }
  double out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

__global__ void __launch_bounds__(kBlock) k64p_s(Geo g, PrecVecsT<double> v, const SolverScal *sc) {
  if (sc->done) return;
  const double a = sc->alpha;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.s[row] = fma(-a, v.v[row], v.r1[row]);
  }
}

__global__ void __launch_bounds__(kBlock) k64p_t(Geo g, Stencil<double> st, PrecVecsT<double> v, double *part,
                                                 SolverScal *sc) {
  if (sc->done) return;
  double a[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double y = spmv_at<double>(g, st, v.sh, ic, jc, kc, row);
    v.t[row] = y;
    a[0] = fma(y, v.s[row], a[0]);
    a[1] = fma(y, y, a[1]);
  }
  double out[2];
  if (grid_sum<2>(a, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;
    sc->omega = wv;
  }
}

__global__ void __launch_bounds__(kBlock) k64p_xr(Geo g, PrecVecsT<double> v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const double a = sc->alpha, w = sc->omega;
  double acc[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.x[row] = fma(w, v.sh[row], fma(a, v.ph[row], v.x[row]));
    const double r1 = fma(-w, v.t[row], v.s[row]);
    v.r1[row] = r1;
    acc[0] = fma(r1, r1, acc[0]);
    acc[1] = fma(r1, v.r0[row], acc[1]);
  }
  double out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) finish_prec64(sc, out[0], out[1]);
}

// ---- FP32 iteration, vectorised: four consecutive k cells per thread (nzc % 4 == 0) ----
// One float4 load per vector and stencil point instead of four scalar loads; the k
// neighbours inside the quad come from registers.  Dot partials stay FP32 over the few
// dozen quads a thread owns and are added into the FP64 block/grid reduction once.
// k32v_xr is pointwise: a grid-stride loop over the planes.
#define FOR_QUADS(g)                                               \
  const int kc0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);     \
  const int kc = kc0; /* ROW(g) of the quad's first cell */        \
  const int jc = blockIdx.y * blockDim.y + threadIdx.y;            \
  const bool on_ = (kc0 < (g).nzc) && (jc < (g).nyc);              \
  for (int ic = blockIdx.z; on_ && ic < (g).nxc; ic += gridDim.z)

struct F4 {
  float v[4];
};
__device__ __forceinline__ F4 ld4(const float *p) {
  const float4 t = *reinterpret_cast<const float4 *>(p);
  return F4{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ void st4(float *p, const F4 &a) {
  *reinterpret_cast<float4 *>(p) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
}

// The two stencil kernels march along x.  A thread owns one quad of one j row and walks a
// chunk of consecutive i planes (the same chunk for the whole block, so every thread runs
// the same trip count).  The values of planes i-1, i, i+1 stay in registers: per plane a
// thread loads the next plane's quad (its first read from HBM) and the quads of rows j-1
// and j+1 (L1 hits, loaded one plane earlier by their owners); the cells left and right
// of the quad come from the neighbouring lanes by warp shuffle, from memory only at a
// block's k edge.  f4(q) evaluates the stencil's argument at the quad of row q, f1(q) at
// one cell; body(row, centre values, A-applied values) consumes the result.  (A shared-
// memory tile for the j neighbours, one barrier per plane, measured slower.)
template <class F4f, class F1f, class Body>
__device__ __forceinline__ void march_quads(const Geo &g, const Stencil<float> &st, F4f &&f4, F1f &&f1, Body &&body) {
  const int kc0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int jc = blockIdx.y * blockDim.y + threadIdx.y;
  const bool on = kc0 < g.nzc && jc < g.nyc;
  const int chunk = (g.nxc + gridDim.z - 1) / gridDim.z;
  const int i0 = min(g.nxc, (int)blockIdx.z * chunk), i1 = min(g.nxc, i0 + chunk);
  const long long nyz = (long long)g.nyc * g.nzc;
  const bool hy0 = jc > 0, hy1 = jc + 1 < g.nyc;
  // cells left / right exist (periodic z: always, across the wrap at the line's ends)...
  const bool kl = kc0 > 0 || g.pz, kr = kc0 + 4 < g.nzc || g.pz;
  // ... and are held by the neighbouring lane (within the line)
  const bool sl = threadIdx.x > 0 && kc0 > 0, sr = threadIdx.x + 1 < blockDim.x && kc0 + 4 < g.nzc;
  const long long wl = kc0 > 0 ? -1 : g.nzc - 1, wr = kc0 + 4 < g.nzc ? 4 : 4 - g.nzc;  // their offsets
  long long row = ((long long)i0 * g.nyc + jc) * g.nzc + kc0;
  F4 fm{}, fc{};
  if (on && i0 < i1) {
    if (i0 > 0) fm = f4(row - nyz);
    fc = f4(row);
  }
  for (int ic = i0; ic < i1; ++ic, row += nyz) {
    F4 fp{}, ym{}, yp{};
    if (on) {
      if (ic + 1 < g.nxc) fp = f4(row + nyz);
      if (hy0) ym = f4(row - g.nzc);
      if (hy1) yp = f4(row + g.nzc);
    }
    const float l = __shfl_up_sync(0xffffffffu, fc.v[3], 1);
    const float r = __shfl_down_sync(0xffffffffu, fc.v[0], 1);
    const float zl = !kl ? 0.0f : (sl ? l : (on ? f1(row + wl) : 0.0f));
    const float zr = !kr ? 0.0f : (sr ? r : (on ? f1(row + wr) : 0.0f));
    // difference form (stencil_apply_diff); a missing neighbour has coefficient 0
    const int cxy = axis_class(ic, g.nxc) * 9 + axis_class(jc, g.nyc) * 3;
    const float *cmid = st.c[cxy + 1], *cfirst = st.c[cxy + (kc0 == 0 && !g.pz ? 0 : 1)],
                *clast = st.c[cxy + (kc0 + 4 == g.nzc && !g.pz ? 2 : 1)];
    F4 y;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float *c = q == 0 ? cfirst : (q == 3 ? clast : cmid);
      const float f0 = fc.v[q];
      const float zm = q == 0 ? zl : fc.v[q - 1], zp = q == 3 ? zr : fc.v[q + 1];
      float t = c[0] * (fm.v[q] - f0);
      t = fmaf(c[1], ym.v[q] - f0, t);
      t = fmaf(c[2], zm - f0, t);
      t = fmaf(c[4], zp - f0, t);
      t = fmaf(c[5], yp.v[q] - f0, t);
      t = fmaf(c[6], fp.v[q] - f0, t);
      y.v[q] = t;
    }
    if (on) body(row, fc, y);
    fm = fc;
    fc = fp;
  }
}

// p_new = r1 + beta (p_old - omega ap_old) (restart: p_new = r0 = r1); ap_new = A p_new;
// alpha = rho / <ap_new, r0>
__global__ void __launch_bounds__(kBlock) k32v_pap(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                   SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float b = (float)sc->beta, w = (float)sc->omega;
  const bool rst = sc->restart != 0;
  const float *__restrict__ po = (parity ? v.p[1] : v.p[0]);
  const float *__restrict__ apo = (parity ? v.ap[1] : v.ap[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  float *__restrict__ apn = (parity ? v.ap[0] : v.ap[1]);
  const float *__restrict__ r1 = v.r1;
  float *__restrict__ r0 = v.r0;
  SumF acc;
  if (rst) {
    march_quads(
        g, st, [&](long long q) { return ld4(r1 + q); }, [&](long long q) { return r1[q]; },
        [&](long long row, const F4 &pc, const F4 &y) {
          st4(pn + row, pc);
          st4(apn + row, y);
          st4(r0 + row, pc);
#pragma unroll
          for (int t = 0; t < 4; ++t) acc.add(y.v[t], pc.v[t]);
        });
  } else {
    march_quads(
        g, st,
        [&](long long q) {
          const F4 r = ld4(r1 + q), p = ld4(po + q), a = ld4(apo + q);
          F4 o;
#pragma unroll
          for (int t = 0; t < 4; ++t) o.v[t] = fmaf(b, fmaf(-w, a.v[t], p.v[t]), r.v[t]);
          return o;
        },
        [&](long long q) { return fmaf(b, fmaf(-w, apo[q], po[q]), r1[q]); },
        [&](long long row, const F4 &pc, const F4 &y) {
          st4(pn + row, pc);
          st4(apn + row, y);
          const F4 z = ld4(r0 + row);
#pragma unroll
          for (int t = 0; t < 4; ++t) acc.add(y.v[t], z.v[t]);
        });
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

// s = r1 - alpha ap; as = A s; omega = <as, s> / <as, as>
__global__ void __launch_bounds__(kBlock) k32v_sas(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                   SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float a = (float)sc->alpha;
  const float *__restrict__ ap = (parity ? v.ap[0] : v.ap[1]);
  const float *__restrict__ r1 = v.r1;
  float *__restrict__ sv = v.s;
  float *__restrict__ asv = v.as;
  SumF a0, a1;
  march_quads(
      g, st,
      [&](long long q) {
        const F4 r = ld4(r1 + q), p = ld4(ap + q);
        F4 o;
#pragma unroll
        for (int t = 0; t < 4; ++t) o.v[t] = fmaf(-a, p.v[t], r.v[t]);
        return o;
      },
      [&](long long q) { return fmaf(-a, ap[q], r1[q]); },
      [&](long long row, const F4 &s4, const F4 &y) {
        st4(sv + row, s4);
        st4(asv + row, y);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          a0.add(y.v[t], s4.v[t]);
          a1.add(y.v[t], y.v[t]);
        }
      });
  double acc[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;  // see k32_sas
    sc->omega = wv;
  }
}

// ---- the preconditioned FP32 iteration on quads (nzc % 4 == 0): the operator kernels march
// along x as k32v_sas does, the pointwise ones stride over float4 quads as k32v_xr does ----
__global__ void __launch_bounds__(kBlock) k32pv_p(Geo g, PrecVecs v, const SolverScal *sc) {
  if (sc->done) return;
  const float b = (float)sc->beta, w = (float)sc->omega;
  const bool rst = sc->restart != 0;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const long long row = 4 * q;
    const F4 r1 = ld4(v.r1 + row);
    if (rst) {
      st4(v.r0 + row, r1);
      st4(v.p + row, r1);
      continue;
    }
    const F4 pp = ld4(v.p + row), vv = ld4(v.v + row);
    F4 o;
#pragma unroll
    for (int t = 0; t < 4; ++t) o.v[t] = r1.v[t] + b * (pp.v[t] - w * vv.v[t]);
    st4(v.p + row, o);
  }
}

__global__ void __launch_bounds__(kBlock) k32pv_v(Geo g, Stencil<float> st, PrecVecs v, double *part,
                                                  SolverScal *sc) {
  if (sc->done) return;
  const float *__restrict__ ph = v.ph;
  const float *__restrict__ r0 = v.r0;
  float *__restrict__ vv = v.v;
  SumF a0;
  march_quads(
      g, st, [&](long long q) { return ld4(ph + q); }, [&](long long q) { return ph[q]; },
      [&](long long row, const F4 &, const F4 &y) {
        st4(vv + row, y);
        const F4 r = ld4(r0 + row);
#pragma unroll
        for (int t = 0; t < 4; ++t) a0.add(y.v[t], r.v[t]);
      });
  double a[1] = {a0.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

__global__ void __launch_bounds__(kBlock) k32pv_s(Geo g, PrecVecs v, const SolverScal *sc) {
  if (sc->done) return;
  const float a = (float)sc->alpha;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const long long row = 4 * q;
    const F4 r1 = ld4(v.r1 + row), vv = ld4(v.v + row);
    F4 o;
#pragma unroll
    for (int t = 0; t < 4; ++t) o.v[t] = fmaf(-a, vv.v[t], r1.v[t]);
    st4(v.s + row, o);
  }
}

__global__ void __launch_bounds__(kBlock) k32pv_t(Geo g, Stencil<float> st, PrecVecs v, double *part,
                                                  SolverScal *sc) {
  if (sc->done) return;
  const float *__restrict__ sh = v.sh;
  const float *__restrict__ sv = v.s;
  float *__restrict__ tv = v.t;
  SumF a0, a1;
  march_quads(
      g, st, [&](long long q) { return ld4(sh + q); }, [&](long long q) { return sh[q]; },
      [&](long long row, const F4 &, const F4 &y) {
        st4(tv + row, y);
        const F4 s4 = ld4(sv + row);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          a0.add(y.v[t], s4.v[t]);
          a1.add(y.v[t], y.v[t]);
        }
      });
  double acc[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;
    sc->omega = wv;
  }
}

__global__ void __launch_bounds__(kBlock) k32pv_xr(Geo g, PrecVecs v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const float a = (float)sc->alpha, w = (float)sc->omega;
  const bool keep = sc->snap != 0;
  SumF n2, rr;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const long long row = 4 * q;
    const F4 ph = ld4(v.ph + row), sh = ld4(v.sh + row), s = ld4(v.s + row), t4 = ld4(v.t + row),
             r0 = ld4(v.r0 + row);
    F4 x = ld4(v.x + row), r1;
    if (keep) st4(v.xb + row, x);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      x.v[t] = fmaf(w, sh.v[t], fmaf(a, ph.v[t], x.v[t]));
      r1.v[t] = fmaf(-w, t4.v[t], s.v[t]);
      n2.add(r1.v[t], r1.v[t]);
      rr.add(r1.v[t], r0.v[t]);
    }
    st4(v.x + row, x);
    st4(v.r1 + row, r1);
  }
  double acc[2] = {n2.get(), rr.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) finish_iteration<true>(sc, out[0], out[1]);
}

// ---- FP32 stencil kernels on a bulk-copy (TMA) pipeline ----
// A block owns tj rows (all k) of the compact vectors and a chunk of consecutive i planes.
// Thread 0 streams each plane's rows jt-1 .. jt+tj (the halo rows included: one contiguous
// range per vector, since rows of a plane are contiguous) into one of kStages shared-memory
// stages with cp.async.bulk, signalling an mbarrier; every thread evaluates the stencil's
// argument from the stage, keeps its own quad's values of planes i-1, i, i+1 in registers
// and takes the j +- 1 values from the stage, the k +- 1 values by warp shuffle.  A stage is
// refilled once all warps have released it (a second mbarrier), one plane after its last
// use, so loads run up to kStages - 2 planes ahead of the computation.  Every wait is
// bounded: a wait that gives up sets sc->fault, the block stops, waits (bounded) for its
// own copies in flight and still joins the reduction.
constexpr int kStages = 4;
constexpr long long kWaitCycles = 1LL << 32;  // ~2 s at 2 GHz
constexpr long long kTestWaitCycles = 1LL << 20;  // ~0.5 ms: the wait limit of the test request

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase with the given parity to complete; false if it did not within `limit`
// cycles
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit = kWaitCycles) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void bulk_load(float *dst, const float *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// The vectors a stage holds: na with halo rows (the stencil's argument is built from them)
// and optionally one with the block's own rows only.
struct StageSrc {
  const float *a[3];
  int na;
  const float *own;
};

__host__ __device__ inline long long stage_floats(int tj, int nz, int na, bool own) {
  return (long long)na * (tj + 2) * nz + (own ? (long long)tj * nz : 0);
}

// fval(arrays of a stage, stage row, first cell) -> the argument's four values of a quad;
// f1(arrays, stage row, cell) -> one value; body(row, centre values, A-applied values,
// own-rows vector of the stage at this thread's row or nullptr)
template <class Fv, class F1, class Body>
__device__ __forceinline__ void tma_march(const Geo &g, const Stencil<float> &st, const StageSrc &src, SolverScal *sc,
                                          Fv &&fval, F1 &&f1, Body &&body) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int bad, test_wait;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + kStages;
  float *stage0 = reinterpret_cast<float *>(smem + 128);
  const int nz = g.nzc, nq = nz / 4, tj = g.tj;
  const long long SA = (long long)(tj + 2) * nz, SS = stage_floats(tj, nz, src.na, src.own != nullptr);
  const int tid = threadIdx.x, lane = tid & 31;
  const int tq = tid % nq, ty = tid / nq;
  const int jt = blockIdx.x * tj, jc = jt + ty, kc0 = 4 * tq;
  const bool on = ty < tj && jc < g.nyc;
  const int chunk = (g.nxc + gridDim.y - 1) / gridDim.y;
  const int i0 = min(g.nxc, (int)blockIdx.y * chunk), i1 = min(g.nxc, i0 + chunk);
  if (i0 >= i1) return;  // uniform per block
  const int lo = max(i0 - 1, 0), hi = min(i1, g.nxc - 1), khi = hi - lo;  // staged planes lo..hi
  const int jlo = max(jt - 1, 0), jhi = min(jt + tj, g.nyc - 1), ohi = min(jt + tj, g.nyc) - 1;
  const uint32_t hbytes = (uint32_t)((jhi - jlo + 1) * nz * 4), obytes = (uint32_t)((ohi - jt + 1) * nz * 4);
  const uint32_t txb = src.na * hbytes + (src.own ? obytes : 0u);
  const long long nyz = (long long)g.nyc * nz;
  int issued = -1;  // thread 0: highest plane index issued
  auto issue = [&](int k) {
    const int s = k % kStages;
    float *dst = stage0 + s * SS;
    const long long plane = (long long)(lo + k) * nyz;
    // the test request announces 16 bytes more than plane 0's copies bring, so that wait
    // runs out (every copy issued still lands; nothing is left in flight)
    mbar_expect_tx(&full[s], txb + (k == 0 && test_wait ? 16u : 0u));
    for (int a = 0; a < src.na; ++a)
      bulk_load(dst + a * SA + (long long)(jlo - (jt - 1)) * nz, src.a[a] + plane + (long long)jlo * nz, hbytes,
                &full[s]);
    if (src.own) bulk_load(dst + src.na * SA, src.own + plane + (long long)jt * nz, obytes, &full[s]);
    issued = k;
  };
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kBlock / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    bad = 0;
    // a one-shot request (SolverScal::test_wait, set only by the host's test switch):
    // block (0,0) of the next pipelined launch takes it
    test_wait = 0;
    if (blockIdx.x == 0 && blockIdx.y == 0 && sc->test_wait) {
      sc->test_wait = 0;
      test_wait = 1;
    }
  }
  __syncthreads();
  const long long wait_limit = test_wait ? kTestWaitCycles : kWaitCycles;
  if (tid == 0)
    for (int k = 0; k <= min(khi, kStages - 1); ++k) issue(k);
  auto fail = [&]() {
    *(volatile int *)&bad = 1;
    atomicExch(&sc->fault, 1);
  };
  auto wait_full = [&](int k) {
    if (mbar_wait(&full[k % kStages], (k / kStages) & 1, wait_limit)) return true;
    fail();
    return false;
  };
  auto arrays = [&](int k) { return stage0 + (k % kStages) * SS; };
  auto release = [&](int k) {
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[k % kStages]);
  };
  auto refill = [&](int k) {  // thread 0: plane k was released by every warp -> load plane k + kStages
    if (tid != 0 || k < 0 || k + kStages > khi) return;
    if (!mbar_wait(&empty[k % kStages], (k / kStages) & 1, wait_limit)) {
      fail();
      return;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    issue(k + kStages);
  };
  const int own = ty + 1;  // this thread's stage row
  int kc = i0 - lo;        // stage index of the centre plane
  int waited = -1;         // highest plane this thread waited for
  bool ok = wait_full(0);
  waited = 0;
  F4 fm{}, fc{};
  if (ok && kc == 1) {
    ok = wait_full(1);
    waited = 1;
  }
  if (ok) {
    if (kc == 1) {
      if (on) fm = fval(arrays(0), own, kc0);
      release(0);
    }
    if (on) fc = fval(arrays(kc), own, kc0);
  }
  long long row = ((long long)i0 * g.nyc + jc) * nz + kc0;
  for (int ic = i0; ok && ic < i1; ++ic, ++kc, row += nyz) {
    if (*(volatile int *)&bad) {
      ok = false;
      break;
    }
    F4 fp{}, ym{}, yp{};
    if (ic + 1 < g.nxc) {
      if (!wait_full(kc + 1)) {
        ok = false;
        break;
      }
      waited = kc + 1;
      if (on) fp = fval(arrays(kc + 1), own, kc0);
    }
    const float *arr = arrays(kc);
    if (on) {
      if (jc > 0) ym = fval(arr, own - 1, kc0);
      if (jc + 1 < g.nyc) yp = fval(arr, own + 1, kc0);
    }
    const float l = __shfl_up_sync(0xffffffffu, fc.v[3], 1);
    const float r = __shfl_down_sync(0xffffffffu, fc.v[0], 1);
    // the cells left and right of the quad: from the neighbouring lane within the row, from
    // the stage at a warp's edge, across the wrap at the row's ends (periodic z), else none
    const float zl = (tq == 0 && !g.pz) ? 0.0f
                                       : ((lane > 0 && tq > 0) ? l : (on ? f1(arr, own, tq > 0 ? kc0 - 1 : nz - 1) : 0.0f));
    const float zr = (tq == nq - 1 && !g.pz)
                         ? 0.0f
                         : ((lane < 31 && tq < nq - 1) ? r : (on ? f1(arr, own, tq < nq - 1 ? kc0 + 4 : 0) : 0.0f));
    const int cxy = axis_class(ic, g.nxc) * 9 + axis_class(jc, g.nyc) * 3;
    const float *cmid = st.c[cxy + 1], *cfirst = st.c[cxy + (kc0 == 0 && !g.pz ? 0 : 1)],
                *clast = st.c[cxy + (kc0 + 4 == nz && !g.pz ? 2 : 1)];
    F4 y;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float *c = q == 0 ? cfirst : (q == 3 ? clast : cmid);
      const float f0 = fc.v[q];
      const float zm = q == 0 ? zl : fc.v[q - 1], zp = q == 3 ? zr : fc.v[q + 1];
      float t = c[0] * (fm.v[q] - f0);
      t = fmaf(c[1], ym.v[q] - f0, t);
      t = fmaf(c[2], zm - f0, t);
      t = fmaf(c[4], zp - f0, t);
      t = fmaf(c[5], yp.v[q] - f0, t);
      t = fmaf(c[6], fp.v[q] - f0, t);
      y.v[q] = t;
    }
    if (on) body(row, fc, y, src.own ? arr + src.na * SA + (long long)ty * nz + kc0 : nullptr);
    release(kc);
    refill(kc - 1);
    fm = fc;
    fc = fp;
  }
  if (!ok && tid == 0)  // stopped early: let this block's copies land before it exits
    for (int k = waited + 1; k <= issued; ++k) mbar_wait(&full[k % kStages], (k / kStages) & 1, wait_limit);
}

__device__ __forceinline__ F4 lds4(const float *p) {
  const float4 t = *reinterpret_cast<const float4 *>(p);
  return F4{{t.x, t.y, t.z, t.w}};
}

__global__ void __launch_bounds__(kBlock) k32t_pap(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                   SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float b = (float)sc->beta, w = (float)sc->omega;
  const bool rst = sc->restart != 0;
  const float *po = (parity ? v.p[1] : v.p[0]);
  const float *apo = (parity ? v.ap[1] : v.ap[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  float *__restrict__ apn = (parity ? v.ap[0] : v.ap[1]);
  float *__restrict__ r0 = v.r0;
  const long long SA = (long long)(g.tj + 2) * g.nzc;
  const int nz = g.nzc;
  SumF acc;
  if (rst) {
    const StageSrc src{{v.r1, nullptr, nullptr}, 1, nullptr};
    tma_march(
        g, st, src, sc, [&](const float *a, int r, int k) { return lds4(a + r * nz + k); },
        [&](const float *a, int r, int k) { return a[r * nz + k]; },
        [&](long long row, const F4 &pc, const F4 &y, const float *) {
          st4(pn + row, pc);
          st4(apn + row, y);
          st4(r0 + row, pc);
#pragma unroll
          for (int t = 0; t < 4; ++t) acc.add(y.v[t], pc.v[t]);
        });
  } else {
    const StageSrc src{{v.r1, po, apo}, 3, r0};
    auto f4 = [&](const float *a, int r, int k) {
      const int o = r * nz + k;
      const F4 rr = lds4(a + o), pp = lds4(a + SA + o), aa = lds4(a + 2 * SA + o);
      F4 f;
#pragma unroll
      for (int t = 0; t < 4; ++t) f.v[t] = fmaf(b, fmaf(-w, aa.v[t], pp.v[t]), rr.v[t]);
      return f;
    };
    tma_march(
        g, st, src, sc, f4,
        [&](const float *a, int r, int k) {
          const int o = r * nz + k;
          return fmaf(b, fmaf(-w, a[2 * SA + o], a[SA + o]), a[o]);
        },
        [&](long long row, const F4 &pc, const F4 &y, const float *z0) {
          st4(pn + row, pc);
          st4(apn + row, y);
          const F4 z = lds4(z0);
#pragma unroll
          for (int t = 0; t < 4; ++t) acc.add(y.v[t], z.v[t]);
        });
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}

__global__ void __launch_bounds__(kBlock) k32t_sas(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                   SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float al = (float)sc->alpha;
  const float *ap = (parity ? v.ap[0] : v.ap[1]);
  float *__restrict__ sv = v.s;
  float *__restrict__ asv = v.as;
  const long long SA = (long long)(g.tj + 2) * g.nzc;
  const int nz = g.nzc;
  SumF a0, a1;
  const StageSrc src{{v.r1, ap, nullptr}, 2, nullptr};
  tma_march(
      g, st, src, sc,
      [&](const float *a, int r, int k) {
        const int o = r * nz + k;
        const F4 rr = lds4(a + o), pp = lds4(a + SA + o);
        F4 f;
#pragma unroll
        for (int t = 0; t < 4; ++t) f.v[t] = fmaf(-al, pp.v[t], rr.v[t]);
        return f;
      },
      [&](const float *a, int r, int k) { return fmaf(-al, a[SA + r * nz + k], a[r * nz + k]); },
      [&](long long row, const F4 &s4, const F4 &y, const float *) {
        st4(sv + row, s4);
        st4(asv + row, y);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          a0.add(y.v[t], s4.v[t]);
          a1.add(y.v[t], y.v[t]);
        }
      });
  double acc[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[2], out) && lin_tid() == 0) {
    double wv = out[0] / out[1];
    if (!(out[1] > 0.0 && isfinite(wv))) wv = 0.0;  // see k32_sas
    sc->omega = wv;
  }
}

// Shared memory of the bulk-copy kernels and their residency.  The pap kernel stages three
// vectors with halo rows and one without; the two-vector kernels (sas, CG pq) stage two, so
// they get their own, smaller size and more resident blocks.  0 when the grid does not fit
// the scheme (nz % 4 != 0 or more than 256 quads per row).
__global__ void k32cgt_pq(Geo g, Stencil<float> st, Vec32 v, double *part, SolverScal *sc);

int fp32_stage_plan(int nzc, int *tj, int *smem_bytes, int *blocks_per_sm, int *smem2_bytes, int *blocks2_per_sm) {
  if (nzc % 4 != 0 || nzc / 4 > kBlock) return 0;
  const int t = kBlock / (nzc / 4);
  const long long bytes = 128 + kStages * stage_floats(t, nzc, 3, true) * 4;
  const long long bytes2 = 128 + kStages * stage_floats(t, nzc, 2, false) * 4;
  if (bytes > 227 * 1024) return 0;
  *tj = t;
  *smem_bytes = (int)bytes;
  *smem2_bytes = (int)bytes2;
  if (cudaFuncSetAttribute(k32t_pap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess ||
      cudaFuncSetAttribute(k32t_sas, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes2) != cudaSuccess ||
      cudaFuncSetAttribute(k32cgt_pq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes2) != cudaSuccess)
    return 0;
  int n = 0, n2 = 0, n3 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k32t_pap, kBlock, (size_t)bytes) != cudaSuccess || n < 1 ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k32t_sas, kBlock, (size_t)bytes2) != cudaSuccess || n2 < 1 ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n3, k32cgt_pq, kBlock, (size_t)bytes2) != cudaSuccess || n3 < 1)
    return 0;
  *blocks_per_sm = n;
  *blocks2_per_sm = n2 < n3 ? n2 : n3;
  return 1;
}

// x += alpha p + omega s; r1 = s - omega as; ||r1||^2, <r1, r0>.  Pointwise, so a flat
// grid-stride loop over quads with a grid sized to fill every SM (g.xgrid blocks).
__global__ void __launch_bounds__(kBlock) k32v_xr(Geo g, Vec32 v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float a = (float)sc->alpha, w = (float)sc->omega;
  const float *__restrict__ p = (parity ? v.p[0] : v.p[1]);
  const float *__restrict__ sv = v.s;
  const float *__restrict__ asv = v.as;
  const float *__restrict__ r0v = v.r0;
  float *__restrict__ xv = v.x;
  float *__restrict__ r1v = v.r1;
  float *__restrict__ xb = v.xb;
  const bool keep = sc->snap != 0;  // the current x is the iterate to keep
  SumF n2, rr;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
    const long long row = 4 * q;
    const F4 s = ld4(sv + row), as = ld4(asv + row), pp = ld4(p + row), r0 = ld4(r0v + row);
    F4 x = ld4(xv + row), r1;
    if (keep) st4(xb + row, x);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      x.v[t] = fmaf(w, s.v[t], fmaf(a, pp.v[t], x.v[t]));
      r1.v[t] = fmaf(-w, as.v[t], s.v[t]);
      n2.add(r1.v[t], r1.v[t]);
      rr.add(r1.v[t], r0.v[t]);
    }
    st4(xv + row, x);
    st4(r1v + row, r1);
  }
  double acc[2] = {n2.get(), rr.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) {
    sc->par ^= 1;  // this iteration's p and ap become the previous ones
    finish_iteration<true>(sc, out[0], out[1]);
  }
}

__global__ void k32cg_xr(Geo g, Vec32 v, double *part, SolverScal *sc);

int fp32_pointwise_blocks_per_sm() {
  // the grid serves both pointwise kernels (BiCGSTAB and CG sweeps): the smaller residency
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k32v_xr, kBlock, 0) != cudaSuccess) a = 4;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k32cg_xr, kBlock, 0) != cudaSuccess) b = 4;
  const int n = a < b ? a : b;
  return n > 0 ? n : 1;
}

// ---- conjugate gradients on the SPE operator ----
// The reference's other Krylov solver, inc/solver/cg.hpp (selected by P_SOLVER_CG_ELL):
// unpreconditioned CG, x += alpha p, r -= alpha q, beta = <r, r>_new / <r, r>_old.  (That
// header does not compile as published; the method it spells out is followed, with
// bicgstabRe2's stop test ||r|| / ||b|| < tol and iteration cap.)  Three FP64 kernels per
// iteration; the FP32 sweeps of the MIXED mode fuse the p update into the SpMV (two
// kernels, 10 words per cell).
__device__ __forceinline__ void finish_cg64(SolverScal *sc, double n2) {
  const double relres = sqrt(n2) / sc->norm0;
  sc->relres = relres;
  if (relres < sc->tol) {
    sc->done = 1;
  } else if (!isfinite(relres)) {
    sc->done = 1;
    sc->status = CFDGB_ENAN;
  } else if (sc->iter >= sc->maxit) {
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
  } else {
    sc->beta = n2 / sc->rho;
    sc->rho = n2;
    sc->iter += 1;
  }
}

// r = b - A x, p = r; history px2 <- px1 <- x (the NaN recovery of the BiCGSTAB path)
__global__ void __launch_bounds__(kBlock) k64cg_setup(Geo g, Stencil<double> st, KrylovVecs<double> v,
                                                       const double *__restrict__ b, double *px1, double *px2,
                                                       double *part, SolverScal *sc) {
  double acc[2] = {0.0, 0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double bb = b[row];
    const double r = bb - spmv_at<double>(g, st, v.x, ic, jc, kc, row);
    v.r1[row] = r;
    v.p1[row] = r;
    px2[row] = px1[row];
    px1[row] = v.x[row];
    acc[0] += bb * bb;
    acc[1] += r * r;
  }
  double out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[0], out) && lin_tid() == 0) {
    sc->timestep += 1;
    sc->norm0 = sqrt(out[0]);
    sc->rho = out[1];
    sc->iter = 0;
    sc->status = 0;
    sc->relres = sqrt(out[1]) / sc->norm0;
    sc->done = (sc->relres < sc->tol) ? 1 : 0;
  }
}
// q = A p, alpha = rho / <p, q>
__global__ void __launch_bounds__(kBlock) k64cg_q(Geo g, Stencil<double> st, KrylovVecs<double> v, double *part,
                                                   SolverScal *sc) {
  if (sc->done) return;
  double a[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double q = spmv_at<double>(g, st, v.p1, ic, jc, kc, row);
    v.ap[row] = q;
    a[0] += q * v.p1[row];
  }
  double out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}
// x += alpha p, r -= alpha q, ||r||^2: stop test and beta
__global__ void __launch_bounds__(kBlock) k64cg_xr(Geo g, KrylovVecs<double> v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const double al = sc->alpha;
  double a[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.x[row] = fma(al, v.p1[row], v.x[row]);
    const double r = fma(-al, v.ap[row], v.r1[row]);
    v.r1[row] = r;
    a[0] += r * r;
  }
  double out[1];
  if (grid_sum<1>(a, part, &sc->cnt[3], out) && lin_tid() == 0) finish_cg64(sc, out[0]);
}
// p = r + beta p
__global__ void __launch_bounds__(kBlock) k64cg_p(Geo g, KrylovVecs<double> v, const SolverScal *sc) {
  if (sc->done) return;
  const double be = sc->beta;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    v.p1[row] = fma(be, v.p1[row], v.r1[row]);
  }
}

// FP32 sweep (MIXED): hand over to the FP64 refinement like the BiCGSTAB sweeps
__device__ __forceinline__ void finish_cg32(SolverScal *sc, double n2) {
  const double relres = sqrt(n2) / sc->norm0, rn = sqrt(n2);
  sc->relres = relres;
  if (relres < sc->best) sc->best = relres;
  if (!isfinite(relres)) {
    sc->done = 1;
    sc->status = CFDGB_ENAN;
  } else if (sc->iter > 16 && relres > 1e3 * sc->best) {
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
  } else if (sc->iter >= sc->maxit) {
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
    sc->iter += 1;
  } else if (relres < sc->tol || rn < sc->delta * sc->rmax) {
    sc->done = 1;
    sc->status = kStatusRefine;
    sc->iter += 1;
  } else {
    sc->beta = n2 / sc->rho;
    sc->rho = n2;
    sc->restart = 0;
    if (!isfinite(sc->beta)) {
      sc->restart = 1;
      sc->rho = n2;
    }
    sc->rmax = fmax(sc->rmax, rn);
    sc->iter += 1;
  }
}

// p_new = r + beta p_old (restart: r) at the stencil points; q = A p_new; alpha = rho / <p_new, q>
__global__ void __launch_bounds__(kBlock) k32cgt_pq(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                     SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float be = (float)sc->beta;
  const bool rst = sc->restart != 0;
  const float *po = (parity ? v.p[1] : v.p[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  float *__restrict__ q = v.ap[0];
  const long long SA = (long long)(g.tj + 2) * g.nzc;
  const int nz = g.nzc;
  SumF acc;
  auto body = [&](long long row, const F4 &pc, const F4 &y, const float *) {
    st4(pn + row, pc);
    st4(q + row, y);
#pragma unroll
    for (int t = 0; t < 4; ++t) acc.add(y.v[t], pc.v[t]);
  };
  if (rst) {
    const StageSrc src{{v.r1, nullptr, nullptr}, 1, nullptr};
    tma_march(
        g, st, src, sc, [&](const float *a, int r, int k) { return lds4(a + r * nz + k); },
        [&](const float *a, int r, int k) { return a[r * nz + k]; }, body);
  } else {
    const StageSrc src{{v.r1, po, nullptr}, 2, nullptr};
    tma_march(
        g, st, src, sc,
        [&](const float *a, int r, int k) {
          const int o = r * nz + k;
          const F4 rr = lds4(a + o), pp = lds4(a + SA + o);
          F4 f;
#pragma unroll
          for (int t = 0; t < 4; ++t) f.v[t] = fmaf(be, pp.v[t], rr.v[t]);
          return f;
        },
        [&](const float *a, int r, int k) { return fmaf(be, a[SA + r * nz + k], a[r * nz + k]); }, body);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}
__global__ void __launch_bounds__(kBlock) k32cgv_pq(Geo g, Stencil<float> st, Vec32 v, double *part,
                                                     SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float be = (float)sc->beta;
  const bool rst = sc->restart != 0;
  const float *__restrict__ po = (parity ? v.p[1] : v.p[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  float *__restrict__ q = v.ap[0];
  const float *__restrict__ r1 = v.r1;
  SumF acc;
  auto body = [&](long long row, const F4 &pc, const F4 &y) {
    st4(pn + row, pc);
    st4(q + row, y);
#pragma unroll
    for (int t = 0; t < 4; ++t) acc.add(y.v[t], pc.v[t]);
  };
  if (rst) {
    march_quads(
        g, st, [&](long long k) { return ld4(r1 + k); }, [&](long long k) { return r1[k]; }, body);
  } else {
    march_quads(
        g, st,
        [&](long long k) {
          const F4 rr = ld4(r1 + k), pp = ld4(po + k);
          F4 f;
#pragma unroll
          for (int t = 0; t < 4; ++t) f.v[t] = fmaf(be, pp.v[t], rr.v[t]);
          return f;
        },
        [&](long long k) { return fmaf(be, po[k], r1[k]); }, body);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}
__global__ void __launch_bounds__(kBlock) k32cg_pq(Geo g, Stencil<float> st, Vec32 v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float be = (float)sc->beta;
  const bool rst = sc->restart != 0;
  const float *__restrict__ po = (parity ? v.p[1] : v.p[0]);
  float *__restrict__ pn = (parity ? v.p[0] : v.p[1]);
  const float *__restrict__ r1 = v.r1;
  AccF acc;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    float pc;
    const float y = rst ? stencil_apply_diff(g, st, ic, jc, kc, row, [&](long long k) { return r1[k]; }, pc)
                        : stencil_apply_diff(g, st, ic, jc, kc, row,
                                             [&](long long k) { return fmaf(be, po[k], r1[k]); }, pc);
    pn[row] = pc;
    v.ap[0][row] = y;
    acc.add(y * pc);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && lin_tid() == 0) sc->alpha = sc->rho / out[0];
}
// x += alpha p_new; r -= alpha q; ||r||^2: refinement test and beta (flat: any cell count)
__global__ void __launch_bounds__(kBlock) k32cg_xr(Geo g, Vec32 v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const int parity = sc->par;
  const float al = (float)sc->alpha;
  const float *__restrict__ p = (parity ? v.p[0] : v.p[1]);
  const float *__restrict__ q = v.ap[0];
  float *__restrict__ xv = v.x;
  float *__restrict__ r1v = v.r1;
  SumF n2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g.ncell % 4 == 0) {
    for (long long k = t0; k < g.ncell / 4; k += stride) {
      const long long row = 4 * k;
      const F4 pp = ld4(p + row), qq = ld4(q + row);
      F4 x = ld4(xv + row), r = ld4(r1v + row);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        x.v[t] = fmaf(al, pp.v[t], x.v[t]);
        r.v[t] = fmaf(-al, qq.v[t], r.v[t]);
        n2.add(r.v[t], r.v[t]);
      }
      st4(xv + row, x);
      st4(r1v + row, r);
    }
  } else {
    for (long long row = t0; row < g.ncell; row += stride) {
      xv[row] = fmaf(al, p[row], xv[row]);
      const float r = fmaf(-al, q[row], r1v[row]);
      r1v[row] = r;
      n2.add(r, r);
    }
  }
  double acc[1] = {n2.get()}, out[1];
  if (grid_sum<1>(acc, part, &sc->cnt[3], out) && lin_tid() == 0) {
    sc->par ^= 1;
    finish_cg32(sc, out[0]);
  }
}

// bicgstabRe2.hpp:133-153: at the cap, NaN/Inf entries come from the previous solution;
// if more than 10 % were bad, the whole vector comes from the one before.
__global__ void __launch_bounds__(kBlock) k_nan_replace(Geo g, double *x, const double *px1, double *part,
                                                        SolverScal *sc) {
  if (sc->status != CFDGB_ENOCONV) return;
  double bad[1] = {0.0}, out[1];
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double xv = x[row];
    if (isnan(xv) || isinf(xv)) { x[row] = px1[row]; bad[0] += 1.0; }
  }
  if (grid_sum<1>(bad, part, &sc->cnt[4], out) && lin_tid() == 0)
    sc->restart = out[0] > (double)g.ncell * 0.1 ? 2 : 0;
}
__global__ void __launch_bounds__(kBlock) k_nan_restore(Geo g, double *x, const double *px2, const SolverScal *sc) {
  if (sc->status != CFDGB_ENOCONV || sc->restart != 2) return;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    x[row] = px2[row];
  }
}

// ---- mixed precision: FP32 BiCGSTAB inside FP64 iterative refinement ----
// Each sweep runs FP32 BiCGSTAB from a fresh start on r1 = (r - null-space part) / scale
// (scale fixed for the whole solve) until its residual has dropped by delta; its
// correction accumulates in the FP32 x.  The refinement adds scale * x to the FP64
// solution and recomputes r = b - A x in FP64, which starts the next sweep.  Keeping the
// Krylov space across refinements (reliable updates) was measured too: on the 512-cell
// axis the FP32 iteration then breaks down near 1e-3 (with compensated dot products as
// well: the FP32 vectors and stencil are the limit), while short restarted sweeps
// converge to the FP64 tolerance.

// r = b - A x in FP64, stored rounded to FP32 (rf); ||r||, ||b|| (flags & 1) and the sweep
// scale (flags & 2): the power of two at or below ||r||, so that scaling by it, here and in
// k_correct64, is exact.  jacobi: st holds the jp-scaled rows (st.c[.][7] = jp), whose
// unscaled residual is r / jp.  FIRST: also ||b|| (a solve's first residual).  The kernel
// is bound by the FP64 pipe, so only the residual (7 FMA from b) and the norms are FP64; the
// null-space sum (whose only use is to keep the FP32 system consistent) is summed in FP32
// per thread, and is left out on the stretched grid (whose residual is taken as it is).
template <bool FIRST>
__global__ void __launch_bounds__(kBlock) k_residual64(Geo g, Stencil<double> st, int jacobi,
                                                        const double *__restrict__ b, const double *__restrict__ x,
                                                        float *__restrict__ rf, double *part, StepScal *ss,
                                                        SolverScal *inner, int flags) {
  double acc[3] = {0.0, 0.0, 0.0};
  float ns = 0.0f;
  const bool nsum = !g.nonuni;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double bb = b[row];
    const double r = resid_at(g, st, x, ic, jc, kc, row, bb);
    const float r32 = d2f_int(r);
    rf[row] = r32;
    acc[0] += r * r;
    if (FIRST) acc[1] += bb * bb;
    // the unscaled residual's sum: its component along the operator's null space
    if (nsum) ns += jacobi ? r32 * d2f_int(row_diag(g, st, ic, jc, kc, row)) : r32;
  }
  acc[2] = f2d_int(ns);
  double out[3];
  if (grid_sum<3>(acc, part, &ss->cnt[1], out) && lin_tid() == 0) {
    if (flags & 1) ss->bnorm = sqrt(out[1]);
    ss->rnorm = sqrt(out[0]);
    ss->relres = ss->rnorm / ss->bnorm;
    ss->rsum = out[2];
    if (flags & 2) inner->scale = sweep_scale(ss->rnorm);
  }
}

// rf minus its null-space part (the mean of the unscaled residual; for the Jacobi rows its
// image jp * mean), divided by the sweep scale, in FP32 (the division by a power of two is
// exact).  Removing it keeps the FP32 system consistent, so the iteration cannot drift
// along the constant mode.
__device__ __forceinline__ float scaled_residual(const Geo &g, const Stencil<double> &st, int jacobi,
                                                 const float *__restrict__ rf, float mi, float inv, int ic, int jc,
                                                 int kc, long long row) {
  const float r = rf[row] * inv;
  return jacobi ? fmaf(-mi, d2f_int(row_jp(g, st, ic, jc, kc, row)), r) : r - mi;
}

// start of a sweep: x = 0, r0 = r1 = scaled residual, rho = <r1, r1>; restart = 1 makes the
// first k32_pap take p = r1 (the reference's p1 = r0); delta, peak: this sweep's residual
// reductions (against its start and its largest residual).  first: also the solve's set-up
// (iteration count, the FP32 estimate's normalisation).
__global__ void __launch_bounds__(kBlock) k_refine_start32(Geo g, Stencil<double> st, int jacobi, Vec32 v,
                                                            const float *__restrict__ rf, const StepScal *ss,
                                                            double delta, double peak, int first, double *part,
                                                            SolverScal *sc) {
  const double inv = sc->scale > 0.0 ? 1.0 / sc->scale : 0.0;  // a power of two
  // the null-space part is the mean on the uniform grid (a symmetric operator); on the
  // stretched grid the operator's left null vector is not constant, and the FP64 residual,
  // in range(A) for a consistent system, is taken as it is
  const double m = g.nonuni ? 0.0 : ss->rsum / (double)g.ncell;
  const float inv32 = d2f_int(inv), mi = d2f_int(m * inv);
  Dot2F acc;
  FOR_CELLS4(g) {
    const long long row = ROW(g);
    const float r = scaled_residual(g, st, jacobi, rf, mi, inv32, ic, jc, kc, row);
    v.x[row] = 0.0f;
    v.r0[row] = r;
    v.r1[row] = r;
    acc.add(r, r);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[0], out) && lin_tid() == 0) {
    if (first) {
      sc->fault = 0;
      sc->timestep += 1;
      sc->norm0 = ss->bnorm * inv;  // relres = ||r1|| scale / ||b||
      sc->best = ss->relres;
      sc->iter = 0;
    }
    sc->delta = delta;
    sc->peak = peak;
    sc->rho = out[0];
    sc->rmax = sqrt(out[0]);
    sc->rstart = sc->rmax;
    sc->relres = sqrt(out[0]) / sc->norm0;
    sc->rel0 = sc->relres;
    sc->snap_rel = sc->relres;  // x = 0, kept by the first x update
    sc->snap = 1;
    sc->done = 0;
    sc->status = 0;
    sc->restart = 1;
    sc->par = 0;
  }
}

// sum of e: FP32 per thread (its only use is the constant mode, which the operator
// annihilates, so its rounding changes x by a constant), FP64 over threads.  Pointwise on
// the compact vector: quads over a flat grid-stride loop (g.xgrid blocks), the tail cells
// of a cell count that is not a multiple of 4 by the first threads.
__global__ void __launch_bounds__(kBlock) k_sum32(Geo g, const float *__restrict__ e, double *part, StepScal *ss) {
  float f = 0.0f;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long q = t0; q < nq; q += stride) {
    const float4 v = *reinterpret_cast<const float4 *>(e + 4 * q);
    f += (v.x + v.y) + (v.z + v.w);
  }
  if (t0 < g.ncell - 4 * nq) f += e[4 * nq + t0];
  double acc[1] = {f2d_int(f)};
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[5], out) && lin_tid() == 0) ss->esum = out[0];
}

// x += factor (e - mean e): factor = +-2^k, the sweep scale, applies an inner correction
// (+) or takes it back (-); the mean (the constant mode, which the pressure leaves free) is
// dropped.  e - mean in FP32, widened exactly, scaled by 2^k and signed in its bits: one
// FP64 addition a cell.  Pointwise, quads as k_sum32.
__device__ __forceinline__ double correction(float e, float m, long long shift, long long sign) {
  const long long d = __double_as_longlong(f2d_int(e - m));
  // a zero stays zero; any other value is an FP32 normal, far from the FP64 limits
  return __longlong_as_double((d << 1) == 0 ? 0LL : (d + shift) ^ sign);
}
__global__ void __launch_bounds__(kBlock) k_correct64(Geo g, double *__restrict__ x, const float *__restrict__ e,
                                                       int k, int neg, const StepScal *ss) {
  const float m = d2f_int(ss->esum / (double)g.ncell);
  const long long shift = (long long)k << 52, sign = neg ? (long long)0x8000000000000000ULL : 0LL;
  const long long nq = g.ncell / 4, stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long q = t0; q < nq; q += stride) {
    const float4 v = *reinterpret_cast<const float4 *>(e + 4 * q);
    double2 *xp = reinterpret_cast<double2 *>(x + 4 * q);
    double2 a = xp[0], b = xp[1];
    a.x += correction(v.x, m, shift, sign);
    a.y += correction(v.y, m, shift, sign);
    b.x += correction(v.z, m, shift, sign);
    b.y += correction(v.w, m, shift, sign);
    xp[0] = a;
    xp[1] = b;
  }
  if (t0 < g.ncell - 4 * nq) x[4 * nq + t0] += correction(e[4 * nq + t0], m, shift, sign);
}

// ---- null-space projection of the right-hand side (project_rhs) ----
// The Neumann operator annihilates constants, so b must sum to zero (unscaled rows) for
// the system to have a solution.  rsum = sum of the unscaled b; b -= its mean, mapped
// back through jp for the Jacobi rows.
__global__ void __launch_bounds__(kBlock) k_rhs_sum(Geo g, Stencil<double> st, int jacobi,
                                                     const double *__restrict__ b, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    acc[0] += jacobi ? b[row] * row_diag(g, st, ic, jc, kc, row) : b[row];
  }
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[6], out) && lin_tid() == 0) ss->rsum = out[0];
}
__global__ void __launch_bounds__(kBlock) k_rhs_subtract(Geo g, Stencil<double> st, int jacobi,
                                                          double *__restrict__ b, const StepScal *ss) {
  const double m = ss->rsum / (double)g.ncell;
  FOR_CELLS(g) {
    const long long row = ROW(g);
    b[row] -= jacobi ? m * row_jp(g, st, ic, jc, kc, row) : m;
  }
}

// out = in scaled to the rows of the system: by jp (Jacobi-scaled rows) or unchanged
__global__ void __launch_bounds__(kBlock) k_scale_rows(Geo g, Stencil<double> st, int jacobi,
                                                        const double *__restrict__ in, double *__restrict__ out) {
  FOR_CELLS(g) {
    const long long row = ROW(g);
    out[row] = jacobi ? row_jp(g, st, ic, jc, kc, row) * in[row] : in[row];
  }
}

// ---- red-black SOR (FP64) on the exact Neumann rows ----
// One colour per launch: cells with (i+j+k) even, then odd, so each half-sweep updates
// cells whose neighbours all have the other colour (no race, order independent; periodic z
// needs an even nzc for the cells across the wrap to differ in colour).
__global__ void __launch_bounds__(kBlock) k_rbsor(Geo g, Stencil<double> st, const double *__restrict__ b,
                                                   double *__restrict__ x, double omega, int color) {
  const long long nyz = (long long)g.nyc * g.nzc;
  FOR_CELLS(g) {
    if (((ic + jc + kc) & 1) != color) continue;
    const long long row = ROW(g);
    const double *c = st.c[cls_of(g, ic, jc, kc)];
    double off = 0.0;
    if (ic > 0) off += c[0] * x[row - nyz];
    if (jc > 0) off += c[1] * x[row - g.nzc];
    const long long zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
    if (zm >= 0) off += c[2] * x[zm];
    if (zp >= 0) off += c[4] * x[zp];
    if (jc < g.nyc - 1) off += c[5] * x[row + g.nzc];
    if (ic < g.nxc - 1) off += c[6] * x[row + nyz];
    const double xn = (b[row] - off) * c[7];  // c[7] = 1/diag (no division in the sweep)
    x[row] += omega * (xn - x[row]);
  }
}

__global__ void __launch_bounds__(kBlock) k_residual_norm64(Geo g, Stencil<double> st, const double *__restrict__ b,
                                                             const double *__restrict__ x, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    const double r = b[row] - spmv_at<double>(g, st, x, ic, jc, kc, row);
    acc[0] += r * r;
  }
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[2], out) && lin_tid() == 0) {
    ss->rnorm = sqrt(out[0]);
    ss->relres = ss->rnorm / ss->bnorm;
  }
}

__global__ void __launch_bounds__(kBlock) k_vec_norm64(Geo g, const double *__restrict__ b, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  FOR_CELLS(g) {
    const long long row = ROW(g);
    acc[0] += b[row] * b[row];
  }
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[3], out) && lin_tid() == 0) ss->bnorm = sqrt(out[0]);
}

// ---- launchers ----
static inline dim3 cgrid(const Geo &g) { return dim3(g.lgx, g.lgy, g.lgz); }
static inline dim3 cblock(const Geo &g) { return dim3(g.lbx, g.lby, 1); }
static inline Vec32 v32(const KrylovVecs<float> &v, float *const p2[2], float *const ap2[2]) {
  Vec32 o;
  o.x = v.x; o.r0 = v.r0; o.r1 = v.r1; o.s = v.s; o.as = v.as;
  o.p[0] = p2[0]; o.p[1] = p2[1]; o.ap[0] = ap2[0]; o.ap[1] = ap2[1];
  o.xb = v.xb;
  return o;
}

// the stretched grid's rows, [7][ncell]: every column of nonuni_row, zeros included
__global__ void __launch_bounds__(kBlock) k_build_rows(Geo g, int jac, double *__restrict__ out) {
  FOR_CELLS(g) {
    const long long row = ROW(g);
    double c[8];
    nonuni_row(g, jac, ic, jc, kc, row, c);
#pragma unroll
    for (int q = 0; q < 7; ++q) out[q * g.ncell + row] = c[q];
  }
}

void launch_build_rows(cudaStream_t s, const Geo &g, int jac, double *out) {
  k_build_rows<<<cgrid(g), cblock(g), 0, s>>>(g, jac, out);
}

// the stored rows rounded to FP32 (MIXED on the stretched grid)
__global__ void __launch_bounds__(kBlock) k_rows_f32(long long n, const double *__restrict__ in,
                                                     float *__restrict__ out) {
  for (long long q = blockIdx.x * (long long)kBlock + threadIdx.x; q < n; q += (long long)gridDim.x * kBlock)
    out[q] = (float)in[q];
}
void launch_rows_f32(cudaStream_t s, long long n, const double *in, float *out) {
  k_rows_f32<<<(int)std::min<long long>((n + kBlock - 1) / kBlock, 4096), kBlock, 0, s>>>(n, in, out);
}

void launch_bicg_setup64(cudaStream_t s, int, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                         const double *b, double *px1, double *px2, double *part, SolverScal *sc, int restart) {
  k_bicg_setup64<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, b, px1, px2, part, sc, restart);
}

void launch_bicgp64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, PrecVecsT<double> v,
                         double *part_buf, SolverScal *sc) {
  switch (part) {
    case 0: k64p_p<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
    case 1: k64p_v<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    case 2: k64p_s<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
    case 3: k64p_t<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    default: k64p_xr<<<cgrid(g), cblock(g), 0, s>>>(g, v, part_buf, sc); break;
  }
}

void launch_bicg64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                        double *part_buf, SolverScal *sc) {
  switch (part) {
    case 0: k64_ap<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    case 1: k64_s<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
    case 2: k64_as<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    case 3: k64_xr<<<cgrid(g), cblock(g), 0, s>>>(g, v, part_buf, sc); break;
    default: k64_p<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
  }
}

void launch_bicg32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st,
                        KrylovVecs<float> v, float *const p2[2], float *const ap2[2], double *part_buf,
                        SolverScal *sc) {
  const Vec32 w = v32(v, p2, ap2);
  if (g.tma && part < 2) {  // stencil kernels on the bulk-copy pipeline
    if (part == 0)
      k32t_pap<<<dim3(g.tgx, g.tgy, 1), kBlock, g.tsmem, s>>>(g, st, w, part_buf, sc);
    else
      k32t_sas<<<dim3(g.tgx, g.tgy2, 1), kBlock, g.tsmem2, s>>>(g, st, w, part_buf, sc);
    return;
  }
  if (g.vbx > 0) {  // vectorised path
    const dim3 vg(g.vgx, g.vgy, g.vgz), vb(g.vbx, g.vby, 1);
    switch (part) {
      case 0: k32v_pap<<<vg, vb, 0, s>>>(g, st, w, part_buf, sc); break;
      case 1: k32v_sas<<<vg, vb, 0, s>>>(g, st, w, part_buf, sc); break;
      default: k32v_xr<<<g.xgrid, kBlock, 0, s>>>(g, w, part_buf, sc); break;
    }
    return;
  }
  switch (part) {
    case 0: k32_pap<<<cgrid(g), cblock(g), 0, s>>>(g, st, w, part_buf, sc); break;
    case 1: k32_sas<<<cgrid(g), cblock(g), 0, s>>>(g, st, w, part_buf, sc); break;
    default: k32_xr<<<cgrid(g), cblock(g), 0, s>>>(g, w, part_buf, sc); break;
  }
}

void launch_bicgp32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st, PrecVecs v,
                         double *part_buf, SolverScal *sc) {
  if (g.vbx > 0) {  // quads
    const dim3 vg(g.vgx, g.vgy, g.vgz), vb(g.vbx, g.vby, 1);
    switch (part) {
      case 0: k32pv_p<<<g.xgrid, kBlock, 0, s>>>(g, v, sc); break;
      case 1: k32pv_v<<<vg, vb, 0, s>>>(g, st, v, part_buf, sc); break;
      case 2: k32pv_s<<<g.xgrid, kBlock, 0, s>>>(g, v, sc); break;
      case 3: k32pv_t<<<vg, vb, 0, s>>>(g, st, v, part_buf, sc); break;
      default: k32pv_xr<<<g.xgrid, kBlock, 0, s>>>(g, v, part_buf, sc); break;
    }
    return;
  }
  switch (part) {
    case 0: k32p_p<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
    case 1: k32p_v<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    case 2: k32p_s<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
    case 3: k32p_t<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    default: k32p_xr<<<cgrid(g), cblock(g), 0, s>>>(g, v, part_buf, sc); break;
  }
}

void launch_cg_setup64(cudaStream_t s, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v, const double *b,
                       double *px1, double *px2, double *part, SolverScal *sc) {
  k64cg_setup<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, b, px1, px2, part, sc);
}
void launch_cg64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                      double *part_buf, SolverScal *sc) {
  switch (part) {
    case 0: k64cg_q<<<cgrid(g), cblock(g), 0, s>>>(g, st, v, part_buf, sc); break;
    case 1: k64cg_xr<<<cgrid(g), cblock(g), 0, s>>>(g, v, part_buf, sc); break;
    default: k64cg_p<<<cgrid(g), cblock(g), 0, s>>>(g, v, sc); break;
  }
}
void launch_cg32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st, KrylovVecs<float> v,
                      float *const p2[2], float *const ap2[2], double *part_buf, SolverScal *sc) {
  const Vec32 w = v32(v, p2, ap2);
  if (part == 1) {
    const int grid = g.xgrid > 0 ? g.xgrid : g.lgx * g.lgy * g.lgz;
    k32cg_xr<<<grid, kBlock, 0, s>>>(g, w, part_buf, sc);
  } else if (g.tma) {
    k32cgt_pq<<<dim3(g.tgx, g.tgy2, 1), kBlock, g.tsmem2, s>>>(g, st, w, part_buf, sc);
  } else if (g.vbx > 0) {
    k32cgv_pq<<<dim3(g.vgx, g.vgy, g.vgz), dim3(g.vbx, g.vby, 1), 0, s>>>(g, st, w, part_buf, sc);
  } else {
    k32cg_pq<<<cgrid(g), cblock(g), 0, s>>>(g, st, w, part_buf, sc);
  }
}
void launch_bicg_nan_reset(cudaStream_t s, int, const Geo &g, double *x, const double *px1, const double *px2,
                           double *part, SolverScal *sc) {
  k_nan_replace<<<cgrid(g), cblock(g), 0, s>>>(g, x, px1, part, sc);
  k_nan_restore<<<cgrid(g), cblock(g), 0, s>>>(g, x, px2, sc);
}

void launch_residual64(cudaStream_t s, int, const Geo &g, const Stencil<double> &st, int jacobi, const double *b,
                       const double *x, float *rf, double *part, StepScal *ss, SolverScal *inner, int flags) {
  if (flags & 1)
    k_residual64<true><<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, b, x, rf, part, ss, inner, flags);
  else
    k_residual64<false><<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, b, x, rf, part, ss, inner, flags);
}
void launch_refine_start32(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, KrylovVecs<float> v,
                           float *const p2[2], float *const ap2[2], const float *rf, const StepScal *ss,
                           double delta, double peak, int first, double *part, SolverScal *sc) {
  k_refine_start32<<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, v32(v, p2, ap2), rf, ss, delta, peak, first, part,
                                                   sc);
}
void launch_sum32(cudaStream_t s, const Geo &g, const float *e, double *part, StepScal *ss) {
  k_sum32<<<g.xgrid, kBlock, 0, s>>>(g, e, part, ss);
}
void launch_correct64(cudaStream_t s, int, const Geo &g, double *x, const float *e, double factor,
                      const StepScal *ss) {
  // factor = +-2^k (sweep_scale); a zero factor (a zero residual, never corrected) adds nothing
  if (!(std::fabs(factor) > 0.0) || !std::isfinite(factor)) return;
  k_correct64<<<g.xgrid, kBlock, 0, s>>>(g, x, e, std::ilogb(factor), factor < 0.0 ? 1 : 0, ss);
}
void launch_project_rhs(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, double *b, double *part,
                        StepScal *ss) {
  k_rhs_sum<<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, b, part, ss);
  k_rhs_subtract<<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, b, ss);
}
void launch_scale_rows(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, const double *in,
                       double *out) {
  k_scale_rows<<<cgrid(g), cblock(g), 0, s>>>(g, st, jacobi, in, out);
}
void launch_rbsor_sweep(cudaStream_t s, int, const Geo &g, const Stencil<double> &st, const double *b, double *x,
                        double omega) {
  k_rbsor<<<cgrid(g), cblock(g), 0, s>>>(g, st, b, x, omega, 0);
  k_rbsor<<<cgrid(g), cblock(g), 0, s>>>(g, st, b, x, omega, 1);
}
void launch_residual_norm64(cudaStream_t s, int, const Geo &g, const Stencil<double> &st, const double *b,
                            const double *x, double *part, StepScal *ss) {
  k_residual_norm64<<<cgrid(g), cblock(g), 0, s>>>(g, st, b, x, part, ss);
}
void launch_vec_norm64(cudaStream_t s, int, const Geo &g, const double *b, double *part, StepScal *ss) {
  k_vec_norm64<<<cgrid(g), cblock(g), 0, s>>>(g, b, part, ss);
}

}  // namespace cfdgb
