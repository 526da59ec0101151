// Pressure Poisson solvers on the 7-point Neumann operator.
//
// BiCGSTAB follows bicgstabRe2::solve (inc/solver/bicgstabRe2.hpp:84-180) step for step:
// warm start, relative-residual stop, rho restart, iteration cap and NaN recovery.  One
// iteration is five grid-stride kernels; every global dot product is a deterministic
// two-stage FP64 reduction (reduce.cuh) whose last block also computes the scalar
// update (alpha, omega, convergence, beta, restart), so no host round trip is needed
// inside an iteration.  Every kernel returns at once when sc->done is set, which lets
// the host enqueue iterations in chunks (or a CUDA graph) and poll only between chunks.
//
// Templated on the vector type: double for the FP64 path, float for the inner solve
// of the mixed-precision defect correction (dots still accumulate in FP64).
#include "cfdgb_internal.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace cfdgb {

#define GRID_STRIDE(row, n) \
  for (long long row = blockIdx.x * (long long)kBlock + threadIdx.x; row < (n); row += (long long)gridDim.x * kBlock)

template <typename T>
__device__ __forceinline__ T spmv(const Geo &g, const Stencil<T> &st, const T *__restrict__ x, long long row) {
  int ic, jc, kc;
  row_cijk(row, g.nyc, g.nzc, ic, jc, kc);
  return stencil_row<T>(st, x, row, ic, jc, kc, g.nxc, g.nyc, g.nzc);
}

// ---- FP64 set-up: bicgstabRe2.hpp:86-106 ----
__global__ void __launch_bounds__(kBlock) k_bicg_setup64(Geo g, Stencil<double> st, KrylovVecs<double> v,
                                                          const double *__restrict__ b, double *px1, double *px2,
                                                          double *part, SolverScal *sc) {
  double acc[2] = {0.0, 0.0};
  GRID_STRIDE(row, g.ncell) {
    const double bb = b[row];
    const double r = bb - spmv<double>(g, st, v.x, row);
    v.r0[row] = r;
    v.r1[row] = r;
    v.p1[row] = r;
    px2[row] = px1[row];
    px1[row] = v.x[row];
    acc[0] += bb * bb;
    acc[1] += r * r;
  }
  double out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[0], out) && threadIdx.x == 0) {
    sc->timestep += 1;
    sc->norm0 = sqrt(out[0]);
    sc->rho = out[1];
    sc->iter = 0;
    sc->done = 0;
    sc->status = 0;
    sc->restart = 0;
    sc->relres = 0.0;
  }
}

// ---- one iteration ----
// K1: ap = A p1, alpha = rho / <ap, r0>
template <typename T>
__global__ void __launch_bounds__(kBlock) k_bicg_ap(Geo g, Stencil<T> st, KrylovVecs<T> v, double *part,
                                                     SolverScal *sc) {
  if (sc->done) return;
  typename AccFor<T>::type acc;
  GRID_STRIDE(row, g.ncell) {
    const T y = spmv<T>(g, st, v.p1, row);
    v.ap[row] = y;
    acc.add(y * v.r0[row]);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[1], out) && threadIdx.x == 0) sc->alpha = sc->rho / out[0];
}

// K2: s = r1 - alpha ap
template <typename T>
__global__ void __launch_bounds__(kBlock) k_bicg_s(Geo g, KrylovVecs<T> v, const SolverScal *sc) {
  if (sc->done) return;
  const T a = (T)sc->alpha;
  GRID_STRIDE(row, g.ncell) v.s[row] = v.r1[row] - a * v.ap[row];
}

// K3: as = A s, omega = <as, s> / <as, as>
template <typename T>
__global__ void __launch_bounds__(kBlock) k_bicg_as(Geo g, Stencil<T> st, KrylovVecs<T> v, double *part,
                                                     SolverScal *sc) {
  if (sc->done) return;
  typename AccFor<T>::type a0, a1;
  GRID_STRIDE(row, g.ncell) {
    const T y = spmv<T>(g, st, v.s, row);
    v.as[row] = y;
    a0.add(y * v.s[row]);
    a1.add(y * y);
  }
  double a[2] = {a0.get(), a1.get()}, out[2];
  if (grid_sum<2>(a, part, &sc->cnt[2], out) && threadIdx.x == 0) {
    double w = out[0] / out[1];
    // FP32 inner solve only: when s has vanished (<as,as> = 0) the half step already
    // solved the system; omega = 0 makes K4 take x += alpha p1, r1 = s and stop, where
    // the unguarded formula would give 0/0.  The FP64 path keeps the reference's formula.
    if (sizeof(T) == 4 && !(out[1] > 0.0 && isfinite(w))) w = 0.0;
    sc->omega = w;
  }
}

// K4: x += alpha p1 + omega s; r1 = s - omega as; stop test; beta and restart decision
template <typename T>
__global__ void __launch_bounds__(kBlock) k_bicg_xr(Geo g, KrylovVecs<T> v, double *part, SolverScal *sc) {
  if (sc->done) return;
  const T a = (T)sc->alpha, w = (T)sc->omega;
  typename AccFor<T>::type n2, rr;
  GRID_STRIDE(row, g.ncell) {
    const T s = v.s[row];
    v.x[row] += a * v.p1[row] + w * s;
    const T r1 = s - w * v.as[row];
    v.r1[row] = r1;
    n2.add(r1 * r1);
    rr.add(r1 * v.r0[row]);
  }
  double acc[2] = {n2.get(), rr.get()}, out[2];
  if (grid_sum<2>(acc, part, &sc->cnt[3], out) && threadIdx.x == 0) {
    const double relres = sqrt(out[0]) / sc->norm0;
    sc->relres = relres;
    if (relres < sc->tol) {  // :129
      sc->done = 1;
    } else if (sizeof(T) == 4 && !isfinite(relres)) {  // FP32 inner solve broke down
      sc->done = 1;
      sc->status = CFDGB_ENAN;
    } else if (sc->iter >= sc->maxit) {  // :133
      sc->done = 1;
      sc->status = CFDGB_ENOCONV;
    } else {  // :156-176
      const double rho_old = sc->rho;
      sc->rho = out[1];
      sc->beta = (sc->alpha / sc->omega) * (sc->rho / rho_old);
      sc->restart = !(sc->timestep < 10 || fabs(rho_old) > sc->restart_thr);
      if (sizeof(T) == 4 && !(isfinite(sc->beta) && sc->omega != 0.0 && sc->rho != 0.0)) {
        // FP32 inner solve: Lanczos breakdown, restart from the current residual with a
        // fresh shadow vector r0 = r1, so rho = <r1, r1>
        sc->restart = 1;
        sc->rho = out[0];
      }
      sc->iter += 1;
    }
  }
}

// K5: p1 = r1 + beta (p1 - omega ap), or restart r0 = p1 = r1
template <typename T>
__global__ void __launch_bounds__(kBlock) k_bicg_p(Geo g, KrylovVecs<T> v, const SolverScal *sc) {
  if (sc->done) return;
  const T b = (T)sc->beta, w = (T)sc->omega;
  if (sc->restart) {
    GRID_STRIDE(row, g.ncell) {
      const T r1 = v.r1[row];
      v.r0[row] = r1;
      v.p1[row] = r1;
    }
  } else {
    GRID_STRIDE(row, g.ncell) v.p1[row] = v.r1[row] + b * (v.p1[row] - w * v.ap[row]);
  }
}

// bicgstabRe2.hpp:133-153: at the cap, NaN/Inf entries come from the previous solution;
// if more than 10 % were bad, the whole vector comes from the one before.
__global__ void __launch_bounds__(kBlock) k_nan_replace(Geo g, double *x, const double *px1, double *part,
                                                        SolverScal *sc) {
  if (sc->status != CFDGB_ENOCONV) return;
  double bad[1] = {0.0}, out[1];
  GRID_STRIDE(row, g.ncell) {
    const double xv = x[row];
    if (isnan(xv) || isinf(xv)) { x[row] = px1[row]; bad[0] += 1.0; }
  }
  if (grid_sum<1>(bad, part, &sc->cnt[4], out) && threadIdx.x == 0)
    sc->restart = out[0] > (double)g.ncell * 0.1 ? 2 : 0;
}
__global__ void __launch_bounds__(kBlock) k_nan_restore(Geo g, double *x, const double *px2, const SolverScal *sc) {
  if (sc->status != CFDGB_ENOCONV || sc->restart != 2) return;
  GRID_STRIDE(row, g.ncell) x[row] = px2[row];
}

// ---- mixed precision: FP64 outer residual, FP32 inner solve on the scaled residual ----
// r64 = b - A x (FP64); ||r||, and ||b|| on the first sweep; inner scale = ||r||.
__global__ void __launch_bounds__(kBlock) k_residual64(Geo g, Stencil<double> st, const double *__restrict__ b,
                                                        const double *__restrict__ x, double *__restrict__ r64,
                                                        double *part, StepScal *ss, SolverScal *inner, int first) {
  double acc[2] = {0.0, 0.0};
  GRID_STRIDE(row, g.ncell) {
    const double bb = b[row];
    const double r = bb - spmv<double>(g, st, x, row);
    r64[row] = r;
    acc[0] += r * r;
    acc[1] += bb * bb;
  }
  double out[2];
  if (grid_sum<2>(acc, part, &ss->cnt[1], out) && threadIdx.x == 0) {
    if (first) ss->bnorm = sqrt(out[1]);
    ss->rnorm = sqrt(out[0]);
    ss->relres = ss->rnorm / ss->bnorm;
    inner->scale = ss->rnorm;
  }
}

// inner set-up: e = 0, r0 = r1 = p1 = r64 / ||r|| in FP32, rho = <r0, r0>, norm0 = ||r0||
__global__ void __launch_bounds__(kBlock) k_inner_setup32(Geo g, KrylovVecs<float> v, const double *__restrict__ r64,
                                                           double *part, SolverScal *sc) {
  const double inv = sc->scale > 0.0 ? 1.0 / sc->scale : 0.0;
  AccF acc;
  GRID_STRIDE(row, g.ncell) {
    const float r = (float)(r64[row] * inv);
    v.x[row] = 0.0f;
    v.r0[row] = r;
    v.r1[row] = r;
    v.p1[row] = r;
    acc.add(r * r);
  }
  double a[1] = {acc.get()}, out[1];
  if (grid_sum<1>(a, part, &sc->cnt[0], out) && threadIdx.x == 0) {
    sc->timestep += 1;
    sc->norm0 = sqrt(out[0]);
    sc->rho = out[0];
    sc->iter = 0;
    sc->done = 0;
    sc->status = 0;
    sc->restart = 0;
    sc->relres = 0.0;
  }
}

// x += ||r|| e
__global__ void __launch_bounds__(kBlock) k_correct64(Geo g, double *__restrict__ x, const float *__restrict__ e,
                                                       const SolverScal *sc) {
  const double s = sc->scale;
  GRID_STRIDE(row, g.ncell) x[row] += s * (double)e[row];
}

// ---- red-black SOR (FP64) on the exact Neumann rows ----
// One colour per launch: cells with (i+j+k) even, then odd, so each half-sweep updates
// cells whose neighbours all have the other colour (no race, order independent).
__global__ void __launch_bounds__(kBlock) k_rbsor(Geo g, Stencil<double> st, const double *__restrict__ b,
                                                   double *__restrict__ x, double omega, int color) {
  const long long nyz = (long long)g.nyc * g.nzc;
  GRID_STRIDE(row, g.ncell) {
    int ic, jc, kc;
    row_cijk(row, g.nyc, g.nzc, ic, jc, kc);
    if (((ic + jc + kc) & 1) != color) continue;
    const double *c = st.c[axis_class(ic, g.nxc) * 9 + axis_class(jc, g.nyc) * 3 + axis_class(kc, g.nzc)];
    double off = 0.0;
    if (ic > 0) off += c[0] * x[row - nyz];
    if (jc > 0) off += c[1] * x[row - g.nzc];
    if (kc > 0) off += c[2] * x[row - 1];
    if (kc < g.nzc - 1) off += c[4] * x[row + 1];
    if (jc < g.nyc - 1) off += c[5] * x[row + g.nzc];
    if (ic < g.nxc - 1) off += c[6] * x[row + nyz];
    const double xn = (b[row] - off) / c[3];
    x[row] += omega * (xn - x[row]);
  }
}

__global__ void __launch_bounds__(kBlock) k_residual_norm64(Geo g, Stencil<double> st, const double *__restrict__ b,
                                                             const double *__restrict__ x, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  GRID_STRIDE(row, g.ncell) {
    const double r = b[row] - spmv<double>(g, st, x, row);
    acc[0] += r * r;
  }
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[2], out) && threadIdx.x == 0) {
    ss->rnorm = sqrt(out[0]);
    ss->relres = ss->rnorm / ss->bnorm;
  }
}

__global__ void __launch_bounds__(kBlock) k_vec_norm64(Geo g, const double *__restrict__ b, double *part, StepScal *ss) {
  double acc[1] = {0.0};
  GRID_STRIDE(row, g.ncell) acc[0] += b[row] * b[row];
  double out[1];
  if (grid_sum<1>(acc, part, &ss->cnt[3], out) && threadIdx.x == 0) ss->bnorm = sqrt(out[0]);
}

// ---- launchers ----
void launch_bicg_setup64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                         const double *b, double *px1, double *px2, double *part, SolverScal *sc) {
  k_bicg_setup64<<<nblk, kBlock, 0, s>>>(g, st, v, b, px1, px2, part, sc);
}

template <typename T>
void launch_bicg_part(cudaStream_t s, int part, int nblk, const Geo &g, const Stencil<T> &st, KrylovVecs<T> v,
                      double *part_buf, SolverScal *sc) {
  switch (part) {
    case 0: k_bicg_ap<T><<<nblk, kBlock, 0, s>>>(g, st, v, part_buf, sc); break;
    case 1: k_bicg_s<T><<<nblk, kBlock, 0, s>>>(g, v, sc); break;
    case 2: k_bicg_as<T><<<nblk, kBlock, 0, s>>>(g, st, v, part_buf, sc); break;
    case 3: k_bicg_xr<T><<<nblk, kBlock, 0, s>>>(g, v, part_buf, sc); break;
    default: k_bicg_p<T><<<nblk, kBlock, 0, s>>>(g, v, sc); break;
  }
}
template void launch_bicg_part<double>(cudaStream_t, int, int, const Geo &, const Stencil<double> &,
                                       KrylovVecs<double>, double *, SolverScal *);
template void launch_bicg_part<float>(cudaStream_t, int, int, const Geo &, const Stencil<float> &,
                                      KrylovVecs<float>, double *, SolverScal *);

template <typename T>
void launch_bicg_iter(cudaStream_t s, int nblk, const Geo &g, const Stencil<T> &st, KrylovVecs<T> v, double *part,
                      SolverScal *sc) {
  for (int q = 0; q < 5; ++q) launch_bicg_part<T>(s, q, nblk, g, st, v, part, sc);
}
template void launch_bicg_iter<double>(cudaStream_t, int, const Geo &, const Stencil<double> &, KrylovVecs<double>,
                                       double *, SolverScal *);
template void launch_bicg_iter<float>(cudaStream_t, int, const Geo &, const Stencil<float> &, KrylovVecs<float>,
                                      double *, SolverScal *);

void launch_bicg_nan_reset(cudaStream_t s, int nblk, const Geo &g, double *x, const double *px1, const double *px2,
                           double *part, SolverScal *sc) {
  k_nan_replace<<<nblk, kBlock, 0, s>>>(g, x, px1, part, sc);
  k_nan_restore<<<nblk, kBlock, 0, s>>>(g, x, px2, sc);
}

void launch_residual64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *b,
                       const double *x, double *r64, double *part, StepScal *ss, SolverScal *inner, int first) {
  k_residual64<<<nblk, kBlock, 0, s>>>(g, st, b, x, r64, part, ss, inner, first);
}
void launch_inner_setup32(cudaStream_t s, int nblk, const Geo &g, KrylovVecs<float> v, const double *r64,
                          double *part, SolverScal *sc) {
  k_inner_setup32<<<nblk, kBlock, 0, s>>>(g, v, r64, part, sc);
}
void launch_correct64(cudaStream_t s, int nblk, const Geo &g, double *x, const float *e, const SolverScal *sc) {
  k_correct64<<<nblk, kBlock, 0, s>>>(g, x, e, sc);
}
void launch_rbsor_sweep(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *b,
                        double *x, double omega) {
  k_rbsor<<<nblk, kBlock, 0, s>>>(g, st, b, x, omega, 0);
  k_rbsor<<<nblk, kBlock, 0, s>>>(g, st, b, x, omega, 1);
}
void launch_residual_norm64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *b,
                            const double *x, double *part, StepScal *ss) {
  k_residual_norm64<<<nblk, kBlock, 0, s>>>(g, st, b, x, part, ss);
}
void launch_vec_norm64(cudaStream_t s, int nblk, const Geo &g, const double *b, double *part, StepScal *ss) {
  k_vec_norm64<<<nblk, kBlock, 0, s>>>(g, b, part, ss);
}

}  // namespace cfdgb
