// Internal types shared by the cfdgb translation units.
//
// Device data layout (all in HBM, one context = one grid):
//   padded FP64 fields  (nx+4)(ny+4)(nz+4), k fastest: u,v,w (T0 = u^n), us,vs,ws
//                       (T1 = u*), ui,vi,wi (initial T0, read only on the three
//                       last-face planes), p, eta;
//   compact Poisson vectors of nx*ny*nz (row = icelCal): b, x and the Krylov vectors,
//   FP64 and (MIXED) FP32 copies;
//   block partial sums [NV][nblk] for the deterministic two-stage reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cfdgb.h"

namespace cfdgb {

constexpr int kBlock = 256;  // threads per block of every grid-stride kernel

// Geometry as the kernels see it.  Padded indices i,j,k run over [0, nx+4); interior
// cells are [2, n+2).  Compact rows enumerate the interior with k fastest.
struct Geo {
  int nxc, nyc, nzc;    // interior cells
  int nx, ny, nz;       // padded extents
  long long sx, sy;     // padded strides: sx = ny*nz, sy = nz
  long long ncell;      // nxc*nyc*nzc
  const double *Dx, *Dy, *Dz, *Dxs, *Dys, *Dzs;  // metric arrays (padded lengths)
  // 3-D launch geometry of the solver kernels: blocks of (lbx along k) x (lby along j)
  // threads, grid (lgx, lgy) covering a (j, k) plane and lgz blocks striding over i
  int lbx, lby, lgx, lgy, lgz;
  // geometry of the vectorised FP32 kernels (four consecutive k cells per thread; used
  // when nzc % 4 == 0, else vbx = 0): vbx quads along k, vby rows along j, vgz over i
  int vbx, vby, vgx, vgy, vgz;
  int xgrid;  // blocks of the flat pointwise FP32 kernel (every SM filled)
  // bulk-copy (TMA) pipeline of the FP32 stencil kernels (nzc % 4 == 0, nzc <= 1024):
  // blocks of tj rows x all k, tgx row tiles x tgy chunks of planes, dynamic shared memory;
  // tgy2, tsmem2: the same for the kernels that stage two vectors (sas, CG pq)
  int tma, tj, tgx, tgy, tsmem, tgy2, tsmem2;
  // stretched grid (the reference's non_uniform-SML): the operator rows come from per-axis
  // factors 1/(D Ds) (fxm[i] = 1/Dx[i+2]/Dxs[i+1], fxp[i] = 1/Dx[i+2]/Dxs[i+2], compact
  // index; SPE_sparseMatrix.hpp:52-58) and jpv, the Jacobi scale of every row
  int nonuni;
  const double *fxm, *fxp, *fym, *fyp, *fzm, *fzp, *jpv;
  // the same rows stored once per context, [7][ncell] (column q of row r at q*ncell + r),
  // cof[0] the SPE rows and cof[1] the Jacobi-scaled CSR rows: built by nonuni_row, so the
  // solver kernels read the bits they would otherwise recompute at every application
  const double *cof[2];
  // MIXED on the stretched grid: the same rows rounded to FP32 (the FP32 sweeps' operator)
  const float *cof32[2];
  int walls;  // a cfdgb_walls value (the boundary table's y-wall rows)
  // periodic z (cfdgb_config.bc_z): z ghosts wrap, the top w face nz-3 is an unknown (face 1
  // its image), every Poisson row keeps both z terms and rows k = 0, nzc-1 couple
  int pz;
  // convective outflow (cfdgb_config.outflow) and its convective velocity: the
  // area-weighted mean inlet u
  int outflow;
  double uconv;
  // per-index reciprocals RN(1/D), RN(1/Ds) of the metrics (padded lengths) for div_by, and
  // the DFIB face-fraction factors (Ds * 0.5) / D of updateUandF.hpp, each one IEEE division
  const double *rDx, *rDy, *rDz, *rDxs, *rDys, *rDzs, *hfx, *hfy, *hfz;
  int div2;  // 1: div_by applies its correction twice (a divisor lacks the certificate)
  int uni;   // 1: every metric array holds one value (a uniform grid): per-axis factors hoist
};

// Width along k of the 3-D solver blocks (host side; the context driver and the
// allocation-free solve share it, so both launch the same shape and reduce in the same
// order): the next power of two up to a warp, then, from 8 k cells up, the width among
// 8, 16 and 32 that leaves the fewest idle lanes at the end of a k line (40 cells: 8 wide,
// where 32 would idle 24 of every 64 lanes).
inline int k_block_width(int nz) {
  int w = 1;
  while (w < nz && w < 32) w *= 2;
  auto idle = [](int n, int b) { return (n + b - 1) / b * b - n; };
  for (int c = 16; c >= 8 && nz >= 8; c /= 2)
    if (idle(nz, c) < idle(nz, w)) w = c;
  return w;
}

// a / b correctly rounded, given y = RN(1/b), by Markstein's FMA correction.  Markstein's
// theorem (P. Markstein, IBM J. Res. Develop. 34(1), 1990; J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, the chapter on division by FMA): if y is within half an ulp of
// 1/b and q within one ulp of a/b, then r = a - b q is exact and RN(q + r y) = RN(a/b),
// while a/b and the intermediates are normal numbers.  q = RN(a y) is within
// 1/2 ulp + |a/b| |b y - 1| of a/b: within one ulp for every a when the divisor's
// certificate |b y - 1| < 2^-54 holds (div_certified, checked on the host for every
// divisor a context uploads), but only within 1.5 ulp in general.  two = true (some
// divisor of the context lacks the certificate) applies the correction twice: the first
// brings q within 1/2 ulp plus a few 2^-53 of an ulp of a/b (its r is exact or nearly so),
// after which the theorem applies to the second.  a = +-0 returns the zero of IEEE
// division's sign.
__device__ __forceinline__ double div_by(double a, double b, double y, bool two) {
  const double q = __dmul_rn(a, y);
  double r = fma(-q, b, a);
  double q1 = fma(r, y, q);
  if (two) {
    r = fma(-q1, b, a);
    q1 = fma(r, y, q1);
  }
  return a == 0.0 ? q : q1;
}

// Host: whether b's reciprocal y = RN(1/b) carries Markstein's certificate |b y - 1| < 2^-54
// (the product b y - 1 is computed exactly by one FMA: its 106-bit product lies within
// 2^-52 of 1, so the difference fits a double).
inline bool div_certified(double b) {
  const double y = 1.0 / b;
  const double e = __builtin_fma(b, y, -1.0);
  return __builtin_fabs(e) < 0x1.0p-54;
}

// FP64 <-> FP32 conversions by integer operations: on this GPU the FP64 pipe, ~1/70 of the
// FP32 rate, also executes the conversion instructions, so the MIXED kernels convert with
// the integer pipes instead.
// double -> float, rounded to nearest (ties to even), by integer operations.  Results
// below the normal FP32 range flush to a signed zero, above it to infinity; NaN stays NaN.
// the scale of a MIXED solve's FP32 sweeps for a residual norm r: the power of two at or
// below r (a multiplication by it, or by its inverse, is exact)
__host__ __device__ __forceinline__ double sweep_scale(double r) {
  return r > 0.0 && r <= 1.7e308 ? ldexp(1.0, ilogb(r)) : r;
}

__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long a = b & 0x7fffffffffffffffULL;
  if ((a >> 52) == 0x7ffULL) return __uint_as_float(sign | 0x7f800000u | ((a << 12) ? 0x400000u : 0u));
  const unsigned long long r = a + 0x0fffffffULL + ((a >> 29) & 1ULL);  // drop 29 bits: nearest, even
  const int e = (int)(r >> 52) - 896;                                     // FP32 exponent field
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((r >> 29) & 0x7fffffULL));
}

// float -> double, exact, by integer operations (FP32 subnormals, never met here, read as zero)
__device__ __forceinline__ double f2d_int(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned e = (b >> 23) & 0xffu;
  if (e == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
  const unsigned eh = e == 0xffu ? 0x7ffu : e + 896u;
  return __hiloint2double((int)((b & 0x80000000u) | (eh << 20) | ((b >> 3) & 0xfffffu)), (int)(b << 29));
}

// compact row -> padded (i,j,k).  Grids below 2^31 cells divide in 32 bits: a 64-bit
// division is a long software sequence on the GPU, twice per cell in every grid-stride kernel.
__device__ __forceinline__ void row_ijk(const Geo &g, long long row, int &i, int &j, int &k) {
  if (g.ncell < (1LL << 31)) {
    const unsigned r = (unsigned)row, nz = (unsigned)g.nzc, nyz = (unsigned)g.nyc * nz;
    const unsigned ic = r / nyz, rem = r - ic * nyz, jc = rem / nz;
    i = (int)ic + 2;
    j = (int)jc + 2;
    k = (int)(rem - jc * nz) + 2;
    return;
  }
  const long long nyz = (long long)g.nyc * g.nzc;
  const int ic = (int)(row / nyz);
  const long long rem = row - (long long)ic * nyz;
  const int jc = (int)(rem / g.nzc);
  k = (int)(rem - (long long)jc * g.nzc) + 2;
  j = jc + 2;
  i = ic + 2;
}

__device__ __forceinline__ long long pidx(const Geo &g, int i, int j, int k) {
  return (long long)i * g.sx + (long long)j * g.sy + k;
}

// 7-point Neumann operator of the pressure Poisson problem, uniform grid.  A row's
// coefficients depend only on whether the cell is first / inner / last along each axis
// (27 classes).  c[cls][0..6] multiply x at -x,-y,-z,0,+z,+y,+x (the SPE column order,
// inc/matrix/SPE_sparseMatrix.hpp:119-125); c[cls][7] = 1/diag of the unscaled operator.
template <typename T>
struct Stencil {
  T c[27][8];
  T dg[27];  // the unscaled diagonal of each class (1/jp up to rounding)
  int jac;   // 1: the rows are scaled by jp (CSR / Jacobi)
};

__device__ __forceinline__ int axis_class(int a, int n) { return a == 0 ? 0 : (a == n - 1 ? 2 : 1); }
// the class of a row: periodic z has no first or last cell along z
__device__ __forceinline__ int row_class(const Geo &g, int ic, int jc, int kc) {
  return axis_class(ic, g.nxc) * 9 + axis_class(jc, g.nyc) * 3 + (g.pz ? 1 : axis_class(kc, g.nzc));
}
// compact rows of the z neighbours: across the ends of a periodic z the wrapped cell;
// -1 where a Neumann row has none
__device__ __forceinline__ long long z_minus(const Geo &g, int kc, long long row) {
  return kc > 0 ? row - 1 : (g.pz ? row + g.nzc - 1 : -1);
}
__device__ __forceinline__ long long z_plus(const Geo &g, int kc, long long row) {
  return kc < g.nzc - 1 ? row + 1 : (g.pz ? row - (g.nzc - 1) : -1);
}

// Coefficients of row (ic, jc, kc) on a stretched grid, computed from the per-axis factors
// with the reference's arithmetic: SPE_sparseMatrix.hpp:66-85 (c[1] the j-1 neighbour with
// the j+1 factor and c[5] the reverse, as there) or, scaled, the CSR rows of
// structureGrid.hpp:583-645 (not swapped); c[7] = jp (CSR) or 1/diag (SPE).
__device__ __forceinline__ void nonuni_row(const Geo &g, int jac, int ic, int jc, int kc, long long row,
                                           double (&c)[8]) {
  const double xm = g.fxm[ic], xp = g.fxp[ic], ym = g.fym[jc], yp = g.fyp[jc], zm = g.fzm[kc], zp = g.fzp[kc];
  const bool i0 = ic == 0, i1 = ic == g.nxc - 1, j0 = jc == 0, j1 = jc == g.nyc - 1, k0 = kc == 0 && !g.pz,
             k1 = kc == g.nzc - 1 && !g.pz;
  if (!jac) {
    double ijk = xm + ym + zm + xp + yp + zp;
    if (i0) ijk -= xm;
    if (i1) ijk -= xp;
    if (j0) ijk -= ym;
    if (j1) ijk -= yp;
    if (k0) ijk -= zm;
    if (k1) ijk -= zp;
    c[0] = i0 ? 0.0 : -xm;
    c[1] = j0 ? 0.0 : -yp;
    c[2] = k0 ? 0.0 : -zm;
    c[3] = ijk;
    c[4] = k1 ? 0.0 : -zp;
    c[5] = j1 ? 0.0 : -ym;
    c[6] = i1 ? 0.0 : -xp;
    c[7] = 1.0 / ijk;
    return;
  }
  const double aa = i0 ? -xm : (i1 ? -xp : 0.0), bb = j0 ? -ym : (j1 ? -yp : 0.0), cc = k0 ? -zm : (k1 ? -zp : 0.0);
  const double dj = xm + ym + zm + xp + yp + zp + aa + bb + cc;
  const double jp = g.jpv[row];
  c[0] = i0 ? 0.0 : -xm * jp;
  c[1] = j0 ? 0.0 : -ym * jp;
  c[2] = k0 ? 0.0 : -zm * jp;
  c[3] = dj * jp;
  c[4] = k1 ? 0.0 : -zp * jp;
  c[5] = j1 ? 0.0 : -yp * jp;
  c[6] = i1 ? 0.0 : -xp * jp;
  c[7] = jp;
}

// y = (A x)[row] for compact row with compact coordinates (ic,jc,kc); bounds on the
// coordinates, terms accumulated in SPE column order; pz: periodic z (the z terms wrap)
template <typename T>
__device__ __forceinline__ T stencil_row(const Stencil<T> &st, const T *__restrict__ x, long long row,
                                         int ic, int jc, int kc, int nxc, int nyc, int nzc, bool pz = false) {
  const long long nyz = (long long)nyc * nzc;
  const T *c = st.c[axis_class(ic, nxc) * 9 + axis_class(jc, nyc) * 3 + (pz ? 1 : axis_class(kc, nzc))];
  T sum = T(0);
  if (ic > 0) sum += c[0] * x[row - nyz];
  if (jc > 0) sum += c[1] * x[row - nzc];
  if (kc > 0) sum += c[2] * x[row - 1];
  else if (pz) sum += c[2] * x[row + nzc - 1];
  sum += c[3] * x[row];
  if (kc < nzc - 1) sum += c[4] * x[row + 1];
  else if (pz) sum += c[4] * x[row - (nzc - 1)];
  if (jc < nyc - 1) sum += c[5] * x[row + nzc];
  if (ic < nxc - 1) sum += c[6] * x[row + nyz];
  return sum;
}

// the same on any grid (the class table on a uniform one)
__device__ __forceinline__ double stencil_row_g(const Geo &g, const Stencil<double> &st, const double *__restrict__ x,
                                                long long row, int ic, int jc, int kc) {
  if (!g.nonuni) return stencil_row<double>(st, x, row, ic, jc, kc, g.nxc, g.nyc, g.nzc, g.pz != 0);
  const double *__restrict__ c = g.cof[st.jac] + row;
  const long long n = g.ncell, nyz = (long long)g.nyc * g.nzc;
  const long long zm = z_minus(g, kc, row), zp = z_plus(g, kc, row);
  double sum = 0.0;
  if (ic > 0) sum += c[0] * x[row - nyz];
  if (jc > 0) sum += c[n] * x[row - g.nzc];
  if (zm >= 0) sum += c[2 * n] * x[zm];
  sum += c[3 * n] * x[row];
  if (zp >= 0) sum += c[4 * n] * x[zp];
  if (jc < g.nyc - 1) sum += c[5 * n] * x[row + g.nzc];
  if (ic < g.nxc - 1) sum += c[6 * n] * x[row + nyz];
  return sum;
}
// jp of a row (the Jacobi scale): class table or the stretched grid's per-row vector
__device__ __forceinline__ double row_jp(const Geo &g, const Stencil<double> &st, int ic, int jc, int kc,
                                         long long row) {
  if (g.nonuni) return g.jpv[row];
  return st.c[row_class(g, ic, jc, kc)][7];
}

// the unscaled diagonal of a row (class table, or column 3 of the stored SPE rows): maps a
// Jacobi-scaled residual back to the unscaled one by a multiplication (r / jp ~ r * diag)
__device__ __forceinline__ double row_diag(const Geo &g, const Stencil<double> &st, int ic, int jc, int kc,
                                           long long row) {
  if (g.nonuni) return g.cof[0][3 * g.ncell + row];
  return st.dg[row_class(g, ic, jc, kc)];
}

__device__ __forceinline__ void row_cijk(long long row, int nyc, int nzc, int &ic, int &jc, int &kc) {
  if (row < (1LL << 31) && (long long)nyc * nzc < (1LL << 31)) {  // 32-bit division, as row_ijk
    const unsigned r = (unsigned)row, nz = (unsigned)nzc, nyz = (unsigned)nyc * nz;
    const unsigned a = r / nyz, rem = r - a * nyz, b = rem / nz;
    ic = (int)a;
    jc = (int)b;
    kc = (int)(rem - b * nz);
    return;
  }
  const long long nyz = (long long)nyc * nzc;
  ic = (int)(row / nyz);
  const long long rem = row - (long long)ic * nyz;
  jc = (int)(rem / nzc);
  kc = (int)(rem - (long long)jc * nzc);
}

// Device-resident scalars of one Krylov solve.  Written by the last block of a kernel,
// read by the next kernel in stream order.
struct SolverScal {
  double rho, alpha, omega, beta, norm0, relres, tol, restart_thr;
  double scale;              // MIXED: fixed scale of the FP32 residual (FP64 ||r|| at the start)
  double best;               // FP32: smallest estimated relative residual seen
  double rmax;               // MIXED: largest FP32 residual norm since the last refinement
  double rstart;             // MIXED: FP32 residual norm at the start of the sweep
  double delta;              // MIXED: refine once ||r1|| < delta * rstart (CG: delta * rmax)
  double peak;               // MIXED BiCGSTAB: or once ||r1|| < peak * rmax
  double rel0;               // MIXED: relres at the start of the sweep
  double snap_rel;           // MIXED BiCGSTAB: relres of the best iterate kept so far
  int snap;                  // MIXED BiCGSTAB: 1 = the current iterate is the new one to keep
  int iter, maxit, done, status, timestep, restart;
  int par;                   // FP32: p[par], ap[par] hold the previous iteration's vectors
  int fault;                 // FP32: a pipeline wait of a stencil kernel gave up (never expected)
  int test_wait;             // FP32: one-shot test request: the next pipelined launch makes
                             // one of its waits run out (CFDGB_TEST_WAIT_FAULT; tests only)
  unsigned cnt[8];           // last-block counters, one per kernel kind
};
// status of an FP32 solve that stopped for an FP64 refinement (never returned to callers)
constexpr int kStatusRefine = 1;

// Per-step scalars (drag, lift, outer residual of the mixed solve)
struct StepScal {
  double cd, cl, fsum[2];
  double bnorm, rnorm, relres;
  double rsum;  // MIXED: sum of the raw residual (its component along the operator's null space)
  double esum;  // MIXED: sum of the inner correction e
  double cfl[7];  // get_Cfl on u*: cfl, U_max[3], U_min[3]
  // time step: dt of the current step (read by the step kernels), the next step's dt (set
  // with the CFL reduction), the simulated time at the end of the last step, and the
  // running extremes U_max[3], -U_min[3] since init (the reference's simu.U_max / U_min
  // keep their values from step to step: cfl.hpp:12-13 resizes, it does not reset)
  double dt, dt_next, time;
  double urun[6];
  double dt_step;  // dt of the last step (set with time at its end)
  double oflux;    // convective outflow: the outlet correction (net boundary flux / outlet area)
  int hist;        // Adams-Bashforth: increments stored by the steps since init (at most 2)
  int hslot;       // Adams-Bashforth order 3: the history slot that holds the last increment
  int nan_flag, pad;
  unsigned cnt[10];
};

// What the step kernels need beside their fields: where dt lives (device memory, so an
// adaptive step needs no host round trip), where the CFL reduction goes and how the next
// dt is chosen (cfdgb_dt_mode: fixed, the reference's timestepper, or a CFL target).
struct StepCtl {
  const double *dtp;  // current dt on the device; null: the kernel's dt argument
  StepScal *ss;       // CFL extremes, dt_next, running extremes
  double *part;       // block partials of the CFL reduction
  int in_step;        // 1: a time step (running extremes and dt_next are kept); 0: a single call
  int dt_mode;        // a cfdgb_dt_mode value
  double Re, cfl_target, dt_max;
  // Adams-Bashforth time stepping (cfdgb_config.time_order 2 or 3; 1: the reference's Euler
  // step): increments convection + diffusion of the last two steps, in slots hb[0], hb[1]
  int time_order;
  double *hb[2][3];
};

// Dir/Num boundary table of inc/BoundaryCondition/FLOWpassing.hpp:6-40 as
// dir[face][component], num[face][component]; faces 0..5 = x-, x+, y-, y+, z-, z+.
// Face 0 is the inlet (u = 1, reflected v and w); every other face is zero-gradient, or,
// with free-slip walls (the rows left commented out at :14-21), v = 0 on faces 2 and 3.
struct BcTable {
  double dir[6][3], num[6][3];
};
inline BcTable flowpassing_table(int walls) {
  BcTable t{};
  for (int f = 0; f < 6; ++f)
    for (int c = 0; c < 3; ++c) { t.dir[f][c] = 0.0; t.num[f][c] = 1.0; }
  t.dir[0][0] = 1.0;
  t.num[0][0] = t.num[0][1] = t.num[0][2] = 0.0;
  if (walls == CFDGB_WALLS_FREE_SLIP) t.num[2][1] = t.num[3][1] = 0.0;
  return t;
}

}  // namespace cfdgb
