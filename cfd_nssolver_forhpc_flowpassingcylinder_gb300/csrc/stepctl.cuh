// The CFL reduction that the convection-diffusion kernels make over u*, and the time-step
// rules it feeds (shared by the exact FP64 and the MIXED kernels).
#pragma once

#include "cfdgb_internal.cuh"
#include "reduce.cuh"

namespace cfdgb {

// dt of the running step: from the step scalars when the step driver passes them
__device__ __forceinline__ double step_dt(const StepCtl &sc, double dt_arg) { return sc.dtp ? *sc.dtp : dt_arg; }

// Per-thread CFL state (get_Cfl, inc/analyses/cfl.hpp:3-78): m[0] the largest per-cell sum
// u/Dxs + v/Dys + w/Dzs, m[1..3] the largest u, v, w, m[4..6] the largest -u, -v, -w.
struct CflAcc {
  double m[7] = {-1e300, -1e10, -1e10, -1e10, -1e10, -1e10, -1e10};
  __device__ __forceinline__ void comp(int a, double x) {
    m[1 + a] = fmax(m[1 + a], x);
    m[4 + a] = fmax(m[4 + a], -x);
  }
  __device__ __forceinline__ void cell(double c) { m[0] = fmax(m[0], c); }
};

// The next dt from this step's CFL extremes (thread 0 of the last block).
//  CFDGB_DT_REFERENCE: timestepper (inc/0_1_SimulationVariable.hpp:172-185) with its factors
//  cflFactor 0.05, gridFoFactor 0.15, dtMin 1e-12 (:270-272), on U_max / U_min kept since
//  init, each product in the reference's left-to-right order.
//  CFDGB_DT_CFL: cfl_target over the largest per-cell sum, at most dt_max.
__device__ __forceinline__ double next_dt(const StepCtl &sc, const StepScal *ss, double cmax, double dt) {
  if (sc.dt_mode == CFDGB_DT_REFERENCE) {
    double d = 1e10;
    for (int a = 0; a < 3; ++a) {
      const double x = ss->urun[a];
      const double lim = 0.05 / (sc.Re * x * x);
      d = lim < d ? lim : d;  // std::min(d, lim)
    }
    for (int a = 0; a < 3; ++a) {
      const double x = -ss->urun[3 + a];
      const double lim = 0.15 * 0.5 * sc.Re * x * x;
      d = lim < d ? lim : d;
    }
    return d < 1e-12 ? 1e-12 : d;
  }
  if (sc.dt_mode == CFDGB_DT_CFL) {
    const double d = cmax > 0.0 ? sc.cfl_target / cmax : sc.dt_max;
    return d < sc.dt_max ? d : sc.dt_max;
  }
  return dt;
}

// Block and grid maxima of the CFL state; the last block stores the CFL number and the
// extremes (ss->cfl) and, in a time step, the running extremes and the next dt.
__device__ __forceinline__ void cfl_finish(CflAcc &acc, double dt, const StepCtl &sc) {
  double out[7];
  if (grid_max<7>(acc.m, sc.part, &sc.ss->cnt[7], out) && lin_tid() == 0) {
    StepScal *ss = sc.ss;
    ss->cfl[0] = out[0] * dt;
    for (int a = 0; a < 3; ++a) {
      ss->cfl[1 + a] = out[1 + a];
      ss->cfl[4 + a] = -out[4 + a];
    }
    if (sc.in_step) {
      for (int q = 0; q < 6; ++q) ss->urun[q] = fmax(ss->urun[q], out[1 + q]);
      ss->dt_next = next_dt(sc, ss, out[0], dt);
      if (sc.time_order > 1) {  // this step's increment is stored: the history grows
        if (ss->hist < 2) ss->hist += 1;
        if (sc.time_order == 3) ss->hslot ^= 1;
      }
    }
  }
}

// End of a time step (finishloop, inc/0_1_SimulationVariable.hpp:139-155): time += dt,
// then, with an adaptive rule (mode 2), dt = dt_next.  Written by the last block of the
// velocity correction, after every block of the step has read dt.  mode 0: not a step.
__device__ __forceinline__ void step_end(StepScal *ss, double dt, int mode) {
  if (mode == 0) return;
  ss->time += dt;
  ss->dt_step = dt;
  if (mode == 2) ss->dt = ss->dt_next;
}

// The new value of a velocity component from this step's convection and diffusion terms:
// the reference's Euler step u + convection + diffusion (Convection_Difussion.hpp:269), or
// with Adams-Bashforth (not in the reference) inc = convection + diffusion and
//   order 2: u + (inc + (r/2) (inc - r h1)),  r = dt_n / dt_(n-1) (variable step);
//   order 3: u + ((23 inc - 16 h1) + 5 h2) / 12 (constant step);
// h1, h2 the increments of the two steps before; the order in effect grows from 1 as the
// history fills after init.  inc is stored for the next steps.
struct AbStep {
  int ord;   // order in effect this step (1: Euler)
  double r;  // dt_n / dt_(n-1)
  double *h1[3], *h2[3], *hn[3];
  __device__ __forceinline__ void init(const StepCtl &sc, double dt) {
    const int hist = sc.ss ? sc.ss->hist : 0;
    ord = sc.time_order > 1 ? (hist + 1 < sc.time_order ? hist + 1 : sc.time_order) : 1;
    r = ord == 2 ? dt / sc.ss->dt_step : 1.0;
    const int s = sc.ss ? sc.ss->hslot : 0;
    for (int c = 0; c < 3; ++c) {
      h1[c] = sc.hb[s][c];
      h2[c] = sc.hb[1 - s][c];
      hn[c] = sc.time_order == 2 ? sc.hb[s][c] : sc.hb[1 - s][c];
    }
  }
  __device__ __forceinline__ double value(int c, long long ic, double uc, double convection, double difussion) const {
    const double inc = convection + difussion;
    double out;
    if (ord <= 1)
      out = uc + convection + difussion;
    else if (ord == 2)
      out = uc + (inc + (0.5 * r) * (inc - r * h1[c][ic]));
    else
      out = uc + ((23.0 * inc - 16.0 * h1[c][ic]) + 5.0 * h2[c][ic]) / 12.0;
    hn[c][ic] = inc;
    return out;
  }
};

}  // namespace cfdgb
