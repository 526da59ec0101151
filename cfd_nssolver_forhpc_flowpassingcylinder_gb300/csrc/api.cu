// Host side of the C ABI (include/cfdgb.h): context set-up, the time-step driver and the
// per-function entry points.  The driver enqueues everything on the context's stream;
// the only host synchronisations are the Poisson solver's convergence polls (one per
// chunk of iterations, each chunk a captured CUDA graph) and the per-step read-back of
// the step scalars (iterations, residual, drag, lift).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cfdgb_internal.cuh"
#include "kernels.h"

using namespace cfdgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(e_ == cudaErrorMemoryAllocation ? CFDGB_ENOMEM : CFDGB_ECUDA, "%s: %s (%s:%d)", #call, \
                  cudaGetErrorString(e_), __FILE__, __LINE__);                                \
  } while (0)

#define TRY(expr)            \
  do {                       \
    int rc_ = (expr);        \
    if (rc_ < 0) return rc_; \
  } while (0)

uint64_t splitmix64(uint64_t &s) {
  s += 0x9E3779B97F4A7C15ULL;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Kernels the instrumentation tells apart (cfdgb_kernel_stat).
enum KId {
  K_CONVDIFF, K_RHS, K_SETUP64, K_AP64, K_S64, K_AS64, K_XR64, K_P64, K_PAP32, K_SAS32, K_XR32,
  K_RESID64, K_SETUP32, K_CORRECT64, K_TRANSFORM, K_UPDATE, K_BC, K_RBSOR, K_RNORM, K_NANRESET, K_ETA,
  K_CGQ64, K_CGXR64, K_CGP64, K_CGPQ32, K_CGXR32, K_CFL, K_LES,
  K_PP32, K_MG, K_PV32, K_PS32, K_PT32, K_PXR32, K_MIRROR,
  K_PP64, K_MG64, K_PV64, K_PS64, K_PT64, K_PXR64, K_COUNT
};
const char *const kKernelNames[K_COUNT] = {
    "convection_diffusion", "rhs", "bicg_setup64", "bicg_ap64", "bicg_s64", "bicg_as64", "bicg_xr64",
    "bicg_p64", "bicg_pap32", "bicg_sas32", "bicg_xr32", "residual64", "refine32",
    "correct64", "transform", "update_uf", "bc", "rbsor_sweep", "residual_norm64", "nan_reset", "solid_fraction",
    "cg_q64", "cg_xr64", "cg_p64", "cg_pq32", "cg_xr32", "cfl", "smagorinsky",
    "bicgp_p32", "mg_vcycle", "bicgp_v32", "bicgp_s32", "bicgp_t32", "bicgp_xr32", "mirror32",
    "bicgp_p64", "mg_vcycle64", "bicgp_v64", "bicgp_s64", "bicgp_t64", "bicgp_xr64"};

// Scalars of one time step run as a graph, appended on the device (k_step_record)
struct StepRec {
  double relres, cd, cl, cfl, dt, time;
  int iters, status, nan, bodies;
};
constexpr int kRing = 1024;  // steps per read-back
struct StepRing {
  int n;       // records written since the last read-back
  int bodies;  // WHILE-body executions of the running step
  StepRec rec[kRing];
};

struct PendingEv {
  int id;
  cudaEvent_t a, b;
};

}  // namespace

struct cfdgb_ctx {
  cfdgb_config cfg{};
  int device = 0, nsm = 0, nblk = 0;
  cudaStream_t stream = nullptr;
  Geo g{};
  long long npad = 0, ncell = 0;
  // host grid (inc/grid/structureGrid.hpp:336-367)
  std::vector<double> X, Y, Z, Dx, Dy, Dz, Dxs, Dys, Dzs;
  Stencil<double> spe64{}, jac64{};
  Stencil<float> spe32{}, jac32{};
  // device buffers
  double *metric = nullptr, *Xd = nullptr, *Yd = nullptr;
  float *tab32 = nullptr;
  std::vector<float> tab32_uni;  // a uniform grid's table rows, one value each (3 x 11); empty otherwise
  double *u = nullptr, *v = nullptr, *w = nullptr, *us = nullptr, *vs = nullptr, *ws = nullptr;
  double *ui = nullptr, *vi = nullptr, *wi = nullptr, *p = nullptr, *eta = nullptr;
  double *b = nullptr, *x = nullptr, *px1 = nullptr, *px2 = nullptr;
  float *rf = nullptr;  // MIXED: the FP64 residual rounded to FP32
  KrylovVecs<double> k64{};
  KrylovVecs<float> k32{};
  float *p32[2] = {nullptr, nullptr}, *ap32[2] = {nullptr, nullptr};  // FP32 double buffers
  // multigrid preconditioner of the FP32 BiCGSTAB sweeps: levels and the two
  // preconditioned vectors M p, M s
  bool use_mg = false;
  MgPlan mg{};
  float *ph32 = nullptr, *sh32 = nullptr;
  // the same preconditioner in FP64 for the FP64 BiCGSTAB (precision FP64, precond multigrid)
  bool use_mg64 = false;
  MgPlanT<double> mg64{};
  double *ph64 = nullptr, *sh64 = nullptr;
  // MIXED QUICK: FP32 copies of the padded u, v, w that the FP32 stencil sweep reads
  float *u32 = nullptr, *v32 = nullptr, *w32 = nullptr;
  // Adams-Bashforth history (time_order 2, 3): increments of the last two steps
  double *hb[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  double *part = nullptr;
  SolverScal *sc = nullptr, *sc32 = nullptr;
  StepScal *ss = nullptr;
  // pinned host mirrors of the scalars
  SolverScal *h_sc = nullptr;
  StepScal *h_ss = nullptr;
  // chunk graphs of solver iterations
  cudaGraphExec_t chunk64 = nullptr, chunk32 = nullptr;
  int chunk_len = 16;
  double omega = 0.0;  // SOR relaxation in use (cfg.omega, or the optimal one when that is 0)
  // test switch (environment CFDGB_TEST_WAIT_FAULT at create): the next MIXED solve makes one
  // bounded wait of the FP32 bulk-copy pipeline run out, to exercise that failure path
  bool test_wait_fault = false;
  // one CUDA graph per time step (FP64 Krylov solvers, after the first step, kernel timing
  // off): the whole step with its convergence loop as a conditional WHILE node; each step
  // appends its scalars to a device ring read back once per cfdgb_step call
  cudaGraphExec_t step_graph = nullptr;
  bool no_step_graph = false;   // CFDGB_NO_STEP_GRAPH at create: the host-driven step instead
  cudaStream_t side = nullptr;  // the WHILE body is captured on it
  bool capturing = false;       // L() neither counts nor times while a graph is captured
  long long graph_fixed = 0;    // kernels of one step graph outside the WHILE body
  long long graph_fixed_kn[64] = {0};
  StepRing *ring = nullptr, *h_ring = nullptr;
  // scratch for the per-function entry points (allocated on first use)
  double *op[10] = {nullptr};
  // Plot3D staging: five float32 arrays on the device and a pinned host copy
  float *p3d = nullptr, *h_p3d = nullptr;
  // Smagorinsky model: (CS delta)^2 per compact row and the eddy viscosity of T0
  double *les_l2 = nullptr, *nut = nullptr;
  double *opc[3] = {nullptr};
  std::vector<void *> allocs;
  int loop = 0;  // steps taken since the last init_fields
  bool have_fields = false;
  // instrumentation
  long long launches = 0;
  bool timing = false;
  double kms[K_COUNT] = {0};
  long long kn[K_COUNT] = {0};
  std::vector<cudaEvent_t> ev_free;
  std::vector<PendingEv> ev_pending;
  // inlet u profile (nyc*nzc) replacing Dir[0][0]; NULL = the reference's constant 1
  double *inlet = nullptr, *inlet_buf = nullptr;
  // discrete adjoint: checkpoints (T0, p, warm start x, solver scalars, step counter)
  // every ckpt_every steps, a recompute window of ckpt_every steps, adjoint fields
  cfdgb_objective obj{};
  bool fwd_done = false;
  std::vector<double *> ck_f;  // 5 buffers per checkpoint: u, v, w, p (padded), x (compact)
  std::vector<SolverScal> ck_sc;
  std::vector<int> ck_loop;
  std::vector<double *> win;  // 3 padded buffers per window step: u, v, w
  std::vector<float *> winp;  // the window steps' pressure, padded, rounded to FP32
  // the adjoint's transposed solve preconditioned by an FP64 V-cycle (contexts with the
  // multigrid preconditioner; built on the first backward)
  bool adj_mg = false;
  double *lA[3] = {nullptr}, *lB[3] = {nullptr}, *lus[3] = {nullptr}, *le[3] = {nullptr};
  double *leta = nullptr, *lx = nullptr, *linlet = nullptr;
  KrylovVecs<double> ka{};
  double *kapx[2] = {nullptr, nullptr};
  SolverScal *sca = nullptr;
  double J = 0.0;
};

namespace {

template <typename T>
int dalloc(cfdgb_ctx *c, T **p, size_t n) {
  void *q = nullptr;
  CK(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
  c->allocs.push_back(q);
  *p = (T *)q;
  return 0;
}

// Resolve recorded event pairs (the stream must have passed them).
void resolve_events(cfdgb_ctx *c) {
  for (auto &e : c->ev_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) c->kms[e.id] += ms;
    c->ev_free.push_back(e.a);
    c->ev_free.push_back(e.b);
  }
  c->ev_pending.clear();
}

// Every kernel launch of the driver goes through here: counts launches and, with timing
// on, brackets the launch with a CUDA-event pair on the context's stream.
template <class F>
void L(cfdgb_ctx *c, int id, int nkernels, F &&launch) {
  if (c->capturing) {  // counted per replay instead (run_step_graphs)
    c->graph_fixed += nkernels;
    c->graph_fixed_kn[id] += nkernels;
    launch();
    return;
  }
  c->launches += nkernels;
  c->kn[id] += nkernels;
  if (!c->timing) {
    launch();
    return;
  }
  if (c->ev_free.size() < 2) {
    if (c->ev_pending.size() >= 2048) {
      cudaStreamSynchronize(c->stream);
      resolve_events(c);
    }
    for (int q = 0; q < 64; ++q) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) == cudaSuccess) c->ev_free.push_back(e);
    }
  }
  PendingEv pe{id, c->ev_free.back(), nullptr};
  c->ev_free.pop_back();
  pe.b = c->ev_free.back();
  c->ev_free.pop_back();
  cudaEventRecord(pe.a, c->stream);
  launch();
  cudaEventRecord(pe.b, c->stream);
  c->ev_pending.push_back(pe);
}

// Reference coefficient helpers (structureGrid.hpp:560-566, SPE_sparseMatrix.hpp:93-99),
// compact index a.
struct Coef {
  const cfdgb_ctx *c;
  double xp(int i) const { return 1.0 / c->Dx[i + 2] / c->Dxs[i + 2]; }
  double yp(int j) const { return 1.0 / c->Dy[j + 2] / c->Dys[j + 2]; }
  double zp(int k) const { return 1.0 / c->Dz[k + 2] / c->Dzs[k + 2]; }
  double xm(int i) const { return 1.0 / c->Dx[i + 2] / c->Dxs[i + 1]; }
  double ym(int j) const { return 1.0 / c->Dy[j + 2] / c->Dys[j + 1]; }
  double zm(int k) const { return 1.0 / c->Dz[k + 2] / c->Dzs[k + 1]; }
};

// init_nonuniform_SML's axis (structureGrid.hpp:250-310, unit_SML): three uniform parts,
// ns fine cells over lsml shifted by off cells, then init_gC_dx (:433-487): ghost nodes by
// linear extrapolation, widths and centre spacings, ghost widths from the nearest interior
void sml_axis(std::vector<double> &a, std::vector<double> &D, std::vector<double> &Ds, double lsml, int ns, int off,
              double l, int n) {
  const int gc = 2, ncal = n - 2 * gc;
  a[gc] = 0.0;
  if (ns != 0) {
    const double dS = lsml / ns, d = (l - lsml) / (ncal - ns);
    int nl0 = (ncal - ns) / 2, ns0 = nl0 + ns;
    const int nl1 = ns0 + nl0;
    nl0 += off;
    ns0 += off;
    for (int i = 0; i < nl0; i++) a[i + gc + 1] = a[i + gc] + d;
    for (int i = nl0; i < ns0; ++i) a[i + gc + 1] = a[i + gc] + dS;
    for (int i = ns0; i < nl1; i++) a[i + gc + 1] = a[i + gc] + d;
  } else {
    for (int i = gc; i < n - gc; i++) a[i + 1] = a[i] + l / ncal;
  }
  a[1] = 2 * a[2] - a[3];
  a[0] = 2 * a[1] - a[2];
  a[n - 1] = 2 * a[n - 2] - a[n - 3];
  a[n] = 2 * a[n - 1] - a[n - 2];
  for (int i = gc; i < n - gc - 1; ++i) Ds[i] = (a[i + 2] - a[i]) / 2.0;
  for (int i = gc; i < n - gc - 1; ++i) D[i] = (a[i + 1] - a[i]);
  D[0] = D[1] = D[2];
  Ds[0] = Ds[1] = Ds[2];
  D[n - 1] = D[n - 2] = D[n - 3] = a[n - 2] - a[n - 3];
  Ds[n - 1] = Ds[n - 2] = Ds[n - 3] = Ds[n - 4];
}

// 27 boundary classes: a representative compact index per class along each axis.
int class_rep(int cls, int n) { return cls == 0 ? 0 : (cls == 2 ? n - 1 : 1); }

void build_stencils(cfdgb_ctx *c) {
  const Coef C{c};
  const int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
  for (int bx = 0; bx < 3; ++bx)
    for (int by = 0; by < 3; ++by)
      for (int bz = 0; bz < 3; ++bz) {
        const int cls = bx * 9 + by * 3 + bz;
        const int i = class_rep(bx, nx), j = class_rep(by, ny), k = class_rep(bz, nz);
        // SPE values, SPE_sparseMatrix.hpp:101-126 (y coefficients swapped as there)
        double ijk = C.xm(i) + C.ym(j) + C.zm(k) + C.xp(i) + C.yp(j) + C.zp(k);
        if (i == 0) ijk -= C.xm(i);
        if (i == nx - 1) ijk -= C.xp(i);
        if (j == 0) ijk -= C.ym(j);
        if (j == ny - 1) ijk -= C.yp(j);
        if (k == 0) ijk -= C.zm(k);
        if (k == nz - 1) ijk -= C.zp(k);
        double *s = c->spe64.c[cls];
        s[0] = i != 0 ? -C.xm(i) : 0.0;
        s[1] = j != 0 ? -C.yp(j) : 0.0;
        s[2] = k != 0 ? -C.zm(k) : 0.0;
        s[3] = ijk;
        s[4] = k != nz - 1 ? -C.zp(k) : 0.0;
        s[5] = j != ny - 1 ? -C.ym(j) : 0.0;
        s[6] = i != nx - 1 ? -C.xp(i) : 0.0;
        // CSR rows scaled by jp, structureGrid.hpp:583-645
        double aa = 0.0, bb = 0.0, cc = 0.0;
        if (i == 0) aa = -C.xm(i);
        if (i == nx - 1) aa = -C.xp(i);
        if (j == 0) bb = -C.ym(j);
        if (j == ny - 1) bb = -C.yp(j);
        if (k == 0) cc = -C.zm(k);
        if (k == nz - 1) cc = -C.zp(k);
        const double dj = C.xm(i) + C.ym(j) + C.zm(k) + C.xp(i) + C.yp(j) + C.zp(k) + aa + bb + cc;
        const double jp = 1.0 / dj;
        double *q = c->jac64.c[cls];
        q[0] = i != 0 ? -C.xm(i) * jp : 0.0;
        q[1] = j != 0 ? -C.ym(j) * jp : 0.0;
        q[2] = k != 0 ? -C.zm(k) * jp : 0.0;
        q[3] = dj * jp;
        q[4] = k != nz - 1 ? -C.zp(k) * jp : 0.0;
        q[5] = j != ny - 1 ? -C.yp(j) * jp : 0.0;
        q[6] = i != nx - 1 ? -C.xp(i) * jp : 0.0;
        q[7] = jp;
        s[7] = 1.0 / ijk;
        c->spe64.dg[cls] = c->jac64.dg[cls] = ijk;
        c->spe32.dg[cls] = c->jac32.dg[cls] = (float)ijk;
        for (int e = 0; e < 8; ++e) {
          c->spe32.c[cls][e] = (float)s[e];
          c->jac32.c[cls][e] = (float)q[e];
        }
      }
  c->spe64.jac = c->spe32.jac = 0;
  c->jac64.jac = c->jac32.jac = 1;
}

// FP32 per-axis tables for step_fast.cu (rows: 1/D, 1/Ds, interpolation factor, QUICK
// coefficients of QuickUnitA and QuickUnitB for both upwind directions).
std::vector<float> build_tab32(const cfdgb_ctx *c, int L) {
  std::vector<float> t(3 * 11 * (size_t)L, 0.0f);
  const std::vector<double> *D[3] = {&c->Dx, &c->Dy, &c->Dz}, *S[3] = {&c->Dxs, &c->Dys, &c->Dzs};
  for (int a = 0; a < 3; ++a) {
    const auto &d = *D[a], &s = *S[a];
    const int n = (int)d.size();
    auto at = [&](const std::vector<double> &v, int I) { return v[std::min(std::max(I, 0), n - 1)]; };
    for (int I = 0; I < n; ++I) {
      float *r = t.data() + (size_t)a * 11 * L;
      r[0 * L + I] = (float)(1.0 / d[I]);
      r[1 * L + I] = (float)(1.0 / s[I]);
      r[2 * L + I] = (float)((s[I] * 0.5) / d[I]);
      r[3 * L + I] = (float)(0.125 * at(d, I + 1) * at(d, I + 1) / s[I]);
      r[4 * L + I] = (float)(0.125 * at(d, I + 1) * at(d, I + 1) / at(s, I + 1));
      r[5 * L + I] = (float)(0.125 * d[I] * d[I] / at(s, I - 1));
      r[6 * L + I] = (float)(0.125 * d[I] * d[I] / s[I]);
      r[7 * L + I] = (float)(0.125 * s[I] * s[I] / d[I]);
      r[8 * L + I] = (float)(0.125 * s[I] * s[I] / at(d, I + 1));
      r[9 * L + I] = (float)(0.125 * at(s, I - 1) * at(s, I - 1) / at(d, I - 1));
      r[10 * L + I] = (float)(0.125 * at(s, I - 1) * at(s, I - 1) / d[I]);
    }
  }
  return t;
}

// The convective outflow's velocity: the area-weighted mean of the inlet u over the inlet
// face (in NULL: the reference's constant 1.0, whose mean is exactly 1)
double inlet_mean(const cfdgb_ctx *c, const double *in) {
  double q = 0.0, a = 0.0;
  for (int j = 2; j < c->cfg.ny + 2; ++j)
    for (int k = 2; k < c->cfg.nz + 2; ++k) {
      const double da = c->Dy[j] * c->Dz[k];
      q += (in ? in[(size_t)(j - 2) * c->cfg.nz + (k - 2)] : 1.0) * da;
      a += da;
    }
  return q / a;
}

// The optimal SOR relaxation for the uniform-grid Neumann operator: 2 / (1 + sqrt(1 - mu^2))
// with mu the spectral radius of the Jacobi iteration on the non-constant modes, the mode
// with one half-wave along the axis where c_a (1 - cos(pi / n_a)) is least (c_a = 1/h_a^2):
// mu = 1 - min_a c_a (1 - cos(pi / n_a)) / (c_x + c_y + c_z)  (Young's theorem for red-black
// ordering, which is consistently ordered).
double sor_omega_opt(const cfdgb_config *c) {
  const double h[3] = {c->lx / c->nx, c->ly / c->ny, c->lz / c->nz};
  const int n[3] = {c->nx, c->ny, c->nz};
  double sum = 0.0, low = 1e300;
  for (int a = 0; a < 3; ++a) {
    const double w = 1.0 / (h[a] * h[a]);
    sum += w;
    if (n[a] > 1) low = std::min(low, w * (1.0 - std::cos(3.14159265358979323846 / n[a])));
  }
  const double mu = 1.0 - low / sum;
  return 2.0 / (1.0 + std::sqrt(std::max(0.0, 1.0 - mu * mu)));
}

// The step kernels' divisors are the metric arrays and dt: the single correction of div_by
// is proven only for certified divisors (div_certified); any other one, or a dt that an
// adaptive rule chooses on the device, selects the double correction
bool division_twice(const cfdgb_ctx *c) {
  if (c->cfg.dt_mode != CFDGB_DT_FIXED || !div_certified(c->cfg.dt)) return true;
  for (auto *v : {&c->Dx, &c->Dy, &c->Dz, &c->Dxs, &c->Dys, &c->Dzs})
    for (double d : *v)
      if (!div_certified(d)) return true;
  return false;
}

int validate(const cfdgb_config *c) {
  if (!c) return fail(CFDGB_EINVAL, "null config");
  if (c->nx < 3 || c->ny < 3 || c->nz < 3) return fail(CFDGB_EINVAL, "grid must be at least 3x3x3 interior cells");
  const double cells = (double)(c->nx + 4) * (c->ny + 4) * (c->nz + 4);
  if (cells > 4.0e9) return fail(CFDGB_EINVAL, "padded grid above 4e9 cells");
  if (!(c->lx > 0 && c->ly > 0 && c->lz > 0)) return fail(CFDGB_EINVAL, "domain lengths must be positive");
  if (!(c->Re > 0) || !(c->dt > 0)) return fail(CFDGB_EINVAL, "Re and dt must be positive");
  if (c->solver < 0 || c->solver > 3) return fail(CFDGB_EINVAL, "unknown solver %d", c->solver);
  if (c->precision < 0 || c->precision > 1) return fail(CFDGB_EINVAL, "unknown precision %d", c->precision);
  if (!(c->tol > 0)) return fail(CFDGB_EINVAL, "tol must be positive");
  if (c->maxit < 1) return fail(CFDGB_EINVAL, "maxit must be >= 1");
  if (c->solver == CFDGB_RBSOR && !(c->omega >= 0 && c->omega < 2)) return fail(CFDGB_EINVAL, "omega outside [0,2)");
  if (c->precision == CFDGB_MIXED && c->solver == CFDGB_RBSOR)
    return fail(CFDGB_EINVAL, "MIXED precision is implemented for the Krylov solvers");
  if (c->precision == CFDGB_MIXED && !(c->inner_tol >= 0 && c->inner_tol < 1))
    return fail(CFDGB_EINVAL, "inner_tol outside [0,1)");
  if (c->dfib && !(c->radius > 0)) return fail(CFDGB_EINVAL, "radius must be positive");
  if (c->grid < 0 || c->grid > 1) return fail(CFDGB_EINVAL, "unknown grid %d", c->grid);
  if (c->scheme < CFDGB_QUICK || c->scheme > CFDGB_UD) return fail(CFDGB_EINVAL, "unknown scheme %d", c->scheme);
  if (c->les != 0 && c->les != 1) return fail(CFDGB_EINVAL, "les must be 0 or 1");
  if (c->walls != CFDGB_WALLS_ZERO_GRADIENT && c->walls != CFDGB_WALLS_FREE_SLIP)
    return fail(CFDGB_EINVAL, "unknown walls %d", c->walls);
  if (c->precond != CFDGB_PRECOND_NONE && c->precond != CFDGB_PRECOND_MULTIGRID)
    return fail(CFDGB_EINVAL, "unknown precond %d", c->precond);
  if (c->precond == CFDGB_PRECOND_MULTIGRID) {
    if ((c->solver != CFDGB_BICGSTAB && c->solver != CFDGB_BICGSTAB_JACOBI) || c->grid != CFDGB_GRID_UNIFORM)
      return fail(CFDGB_EINVAL, "the multigrid preconditioner is for the BiCGSTAB solvers on a uniform grid");
    MgPlan mg;
    if (!mg_plan(c->nx, c->ny, c->nz, c->lx / c->nx, c->ly / c->ny, c->lz / c->nz, 1, false, &mg,
                 c->bc_z == CFDGB_Z_PERIODIC))
      return fail(CFDGB_EINVAL,
                  "multigrid: %dx%dx%d does not coarsen to %d cells by halving even extents (periodic z: with an "
                  "even nz on every level)",
                  c->nx, c->ny, c->nz, kMgSharedCells);
  }
  if (c->bc_z != CFDGB_Z_ZERO_GRADIENT && c->bc_z != CFDGB_Z_PERIODIC)
    return fail(CFDGB_EINVAL, "unknown bc_z %d", c->bc_z);
  if (c->outflow != CFDGB_OUTFLOW_ZERO_GRADIENT && c->outflow != CFDGB_OUTFLOW_CONVECTIVE)
    return fail(CFDGB_EINVAL, "unknown outflow %d", c->outflow);
  if (c->bc_z == CFDGB_Z_PERIODIC && c->solver == CFDGB_RBSOR && c->nz % 2)  // the cells across the wrap
    return fail(CFDGB_EINVAL, "red-black SOR with periodic z needs nz even");  // must differ in colour
  if (c->dt_mode < CFDGB_DT_FIXED || c->dt_mode > CFDGB_DT_CFL) return fail(CFDGB_EINVAL, "unknown dt_mode %d", c->dt_mode);
  if (c->time_order < 0 || c->time_order > 3) return fail(CFDGB_EINVAL, "time_order must be 1, 2 or 3");
  if (c->time_order == 3 && c->dt_mode != CFDGB_DT_FIXED)
    return fail(CFDGB_EINVAL, "third-order Adams-Bashforth is the constant-step form: it needs CFDGB_DT_FIXED");
  if (c->dt_mode == CFDGB_DT_CFL && !(c->cfl_target > 0 && c->dt_max >= 0))
    return fail(CFDGB_EINVAL, "CFDGB_DT_CFL needs cfl_target > 0 and dt_max >= 0");
  if (c->grid == CFDGB_GRID_SML) {
    // unit_SML's own conditions (structureGrid.hpp:269,283): 100 fine cells in x (shifted 4
    // cells) and in y, an even number of coarse ones on both sides
    if (c->nx % 2 || c->nx <= 108 || c->ny % 2 || c->ny <= 100)
      return fail(CFDGB_EINVAL, "the SML grid needs nx even > 108 and ny even > 100");
    if (c->solver != CFDGB_BICGSTAB && c->solver != CFDGB_BICGSTAB_JACOBI)
      return fail(CFDGB_EINVAL, "the SML grid is implemented for the BiCGSTAB solvers (its operator is not symmetric)");
    if (c->project_rhs)
      return fail(CFDGB_EINVAL, "project_rhs removes the mean, not the stretched operator's null-space part");
  }
  return 0;
}

// The kernels of one Krylov iteration: BiCGSTAB 5 (FP64) / 3 (FP32), CG 3 / 2.
// The multigrid-preconditioned FP32 iteration: p, M p, v = A M p, s, M s, t = A M s, x/r
constexpr int kPrecParts = 7;
const int kPrecKid[kPrecParts] = {K_PP32, K_MG, K_PV32, K_PS32, K_MG, K_PT32, K_PXR32};
const int kPrecKid64[kPrecParts] = {K_PP64, K_MG64, K_PV64, K_PS64, K_MG64, K_PT64, K_PXR64};

// the iteration of this precision is the multigrid-preconditioned one
bool prec_iter(const cfdgb_ctx *c, bool fp32) { return fp32 ? c->use_mg : c->use_mg64; }

int iter_kernels(const cfdgb_ctx *c, bool fp32) {
  if (prec_iter(c, fp32)) return kPrecParts;
  if (c->cfg.solver == CFDGB_CG) return fp32 ? 2 : 3;
  return fp32 ? 3 : 5;
}
int iter_kid(const cfdgb_ctx *c, bool fp32, int part) {
  if (prec_iter(c, fp32)) return (fp32 ? kPrecKid : kPrecKid64)[part];
  if (c->cfg.solver == CFDGB_CG) return (fp32 ? K_CGPQ32 : K_CGQ64) + part;
  return (fp32 ? K_PAP32 : K_AP64) + part;
}
// kernels one part launches (a V-cycle is many)
int iter_part_launches(const cfdgb_ctx *c, bool fp32, int part) {
  const int k = iter_kid(c, fp32, part);
  return k == K_MG ? mg_vcycle_launches(c->mg) : k == K_MG64 ? mg_vcycle_launches(c->mg64) : 1;
}
// iterations per captured chunk: the preconditioned iteration is long and needs few
int chunk_iters(const cfdgb_ctx *c, bool fp32) { return prec_iter(c, fp32) ? 2 : c->chunk_len; }
void launch_iter_kernel(cfdgb_ctx *c, bool fp32, int part) {
  const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
  if (!fp32 && c->use_mg64) {
    PrecVecsT<double> v{c->k64.x, c->k64.r0, c->k64.r1, c->k64.p1, c->k64.ap, c->k64.s, c->k64.as, c->ph64, c->sh64,
                        nullptr};
    const int jf = jac ? 1 : 0;
    switch (part) {
      case 1: launch_mg_vcycle(c->stream, c->mg64, jf, (const double *)v.p, v.ph, c->sc); break;
      case 4: launch_mg_vcycle(c->stream, c->mg64, jf, (const double *)v.s, v.sh, c->sc); break;
      default:
        launch_bicgp64_part(c->stream, part == 0 ? 0 : part == 2 ? 1 : part == 3 ? 2 : part == 5 ? 3 : 4, c->g,
                            jac ? c->jac64 : c->spe64, v, c->part, c->sc);
    }
    return;
  }
  if (fp32 && c->use_mg) {
    PrecVecs v{c->k32.x, c->k32.r0, c->k32.r1, c->p32[0], c->ap32[0], c->k32.s, c->k32.as, c->ph32, c->sh32,
               c->k32.xb};
    const int jf = jac ? 1 : 0;
    switch (part) {
      case 1: launch_mg_vcycle(c->stream, c->mg, jf, (const float *)v.p, v.ph, c->sc32); break;
      case 4: launch_mg_vcycle(c->stream, c->mg, jf, (const float *)v.s, v.sh, c->sc32); break;
      default:
        launch_bicgp32_part(c->stream, part == 0 ? 0 : part == 2 ? 1 : part == 3 ? 2 : part == 5 ? 3 : 4, c->g,
                            jac ? c->jac32 : c->spe32, v, c->part, c->sc32);
    }
    return;
  }
  if (c->cfg.solver == CFDGB_CG) {
    if (fp32)
      launch_cg32_part(c->stream, part, c->g, c->spe32, c->k32, c->p32, c->ap32, c->part, c->sc32);
    else
      launch_cg64_part(c->stream, part, c->g, c->spe64, c->k64, c->part, c->sc);
  } else if (fp32) {
    launch_bicg32_part(c->stream, part, c->g, jac ? c->jac32 : c->spe32, c->k32, c->p32, c->ap32, c->part, c->sc32);
  } else {
    launch_bicg64_part(c->stream, part, c->g, jac ? c->jac64 : c->spe64, c->k64, c->part, c->sc);
  }
}

int capture_chunk(cfdgb_ctx *c, bool fp32) {
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int m = 0; m < chunk_iters(c, fp32); ++m)
    for (int part = 0; part < iter_kernels(c, fp32); ++part) launch_iter_kernel(c, fp32, part);
  CK(cudaStreamEndCapture(c->stream, &graph));
  cudaGraphExec_t exec;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  (fp32 ? c->chunk32 : c->chunk64) = exec;
  return 0;
}

// Set the solve parameters in the device scalars (read by the set-up kernels' successors).
int set_solver_params(cfdgb_ctx *c, SolverScal *dsc, double tol, int maxit) {
  // tol, restart_thr, maxit live at fixed offsets; write them with small async copies
  struct {
    double tol, thr;
  } t{tol, tol * 1e-7};  // bicgstabRe2.hpp:53 (pRestartFactor_)
  CK(cudaMemcpyAsync(&dsc->tol, &t, sizeof(t), cudaMemcpyHostToDevice, c->stream));
  // restart_thr follows tol in SolverScal
  static_assert(offsetof(SolverScal, restart_thr) == offsetof(SolverScal, tol) + sizeof(double), "layout");
  CK(cudaMemcpyAsync(&dsc->maxit, &maxit, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  return 0;
}

// Iterate chunks until the device says done.  Returns the scalars in *out.  Each chunk
// is a captured graph of chunk_len iterations; with kernel timing on, the same kernels
// are launched one by one between event pairs instead, one iteration per poll, so that no
// launch after the stop (which returns at once) enters the per-kernel averages.
int run_chunks(cfdgb_ctx *c, bool fp32, SolverScal *out) {
  SolverScal *dsc = fp32 ? c->sc32 : c->sc;
  if (!c->timing && !(fp32 ? c->chunk32 : c->chunk64)) TRY(capture_chunk(c, fp32));
  const int len = c->timing ? 1 : chunk_iters(c, fp32);
  const long long max_chunks = (long long)c->cfg.maxit / len + 3;
  const int nk = iter_kernels(c, fp32);
  for (long long q = 0; q < max_chunks; ++q) {
    if (c->timing) {
      for (int m = 0; m < len; ++m)
        for (int part = 0; part < nk; ++part)
          L(c, iter_kid(c, fp32, part), iter_part_launches(c, fp32, part), [&] { launch_iter_kernel(c, fp32, part); });
    } else {
      for (int part = 0; part < nk; ++part) {
        const int n = iter_part_launches(c, fp32, part);
        c->launches += (long long)n * len;
        c->kn[iter_kid(c, fp32, part)] += (long long)n * len;
      }
      CK(cudaGraphLaunch(fp32 ? c->chunk32 : c->chunk64, c->stream));
    }
    CK(cudaMemcpyAsync(c->h_sc, dsc, sizeof(SolverScal), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    resolve_events(c);
    static const int trace = std::getenv("CFDGB_TRACE") ? std::atoi(std::getenv("CFDGB_TRACE")) : 0;
    if (trace >= 2)
      std::fprintf(stderr, "[cfdgb]     %s it %d relres %.4e\n", fp32 ? "fp32" : "fp64", c->h_sc->iter,
                   c->h_sc->relres);
    if (fp32 && c->h_sc->fault)
      return fail(CFDGB_ECUDA, "FP32 stencil pipeline: a bounded wait gave up (block stopped early)");
    if (c->h_sc->done) {
      *out = *c->h_sc;
      return 0;
    }
  }
  return fail(CFDGB_ECUDA, "solver did not report completion");
}

// Residual reduction of one FP32 sweep against its start (cfg.inner_tol, or 0 for the
// solver's own, measured on the 512x256x64 and 1024x512x128 workloads): BiCGSTAB in FP32
// loses track of its residual a few decades into one Krylov run, so its sweeps stay short
// (0.3); CG has no such breakdown and gains from long sweeps (iterations per solve on
// 512x256x64: 0.3 ~4000, 1e-3 ~2400 in 3 refinements, 3e-4 ~2250 in 3; on 1024x512x128
// 3e-4 saves the fourth refinement that 1e-3 needs, and 1e-4 restarts no less often).
// The multigrid-preconditioned sweep converges in a few dozen iterations, far too few for
// the FP32 recursion to drift, and runs 1e-3 deep.
double sweep_reduction(const cfdgb_ctx *c) {
  if (c->cfg.inner_tol > 0.0) return c->cfg.inner_tol;
  if (c->use_mg) return 1e-3;
  return c->cfg.solver == CFDGB_CG ? 3e-4 : 0.3;
}

// A BiCGSTAB sweep also ends once its residual is this fraction of its largest one: its
// residual can rise far above the sweep's start before it falls, and the FP32 recursion
// cannot follow it down much more than two decades below such a peak (the kept iterate
// bounds what the sweep gives back).  0.3 ended sweeps right after every bump and cost
// ~15 % on 512x256x64; the two were even on 1024x512x128.
// The multigrid-preconditioned sweep has no such bumps (its residual falls ~30x an
// iteration): the rule stays off there and only the reduction ends it (0 never fires).
double sweep_peak(const cfdgb_ctx *c) { return c->use_mg ? 0.0 : 1e-2; }

// FP64 Krylov set-up on the current b and warm start x
void launch_setup64(cfdgb_ctx *c, const Stencil<double> &st64) {
  if (c->cfg.solver == CFDGB_CG)
    launch_cg_setup64(c->stream, c->g, st64, c->k64, c->b, c->px1, c->px2, c->part, c->sc);
  else
    launch_bicg_setup64(c->stream, c->nblk, c->g, st64, c->k64, c->b, c->px1, c->px2, c->part, c->sc,
                        c->use_mg64 ? 1 : 0);
}

// createBMatrix + solve + (caller) transform, on the current u*.  Fills iters/relres.
// createBMatrix_omp on u* (and, project_rhs, the null-space projection)
void enqueue_rhs(cfdgb_ctx *c) {
  const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
  const Stencil<double> &st64 = jac ? c->jac64 : c->spe64;
  L(c, K_RHS, 1, [&] {
    if (c->cfg.precision == CFDGB_MIXED)
      launch_rhs_fast(c->stream, c->nblk, c->g, c->cfg.dt, &c->ss->dt, c->us, c->vs, c->ws, jac, c->jac64, c->b);
    else
      launch_rhs_exact(c->stream, c->nblk, c->g, c->cfg.dt, &c->ss->dt, c->us, c->vs, c->ws, jac, c->jac64, c->b);
  });
  if (c->cfg.project_rhs)
    L(c, K_RHS, 2, [&] { launch_project_rhs(c->stream, c->g, st64, jac ? 1 : 0, c->b, c->part, c->ss); });
}

int solve_mixed(cfdgb_ctx *c, double tol, int *iters, int *outer, double *relres, int *status);

int solve_pressure(cfdgb_ctx *c, int *iters, int *outer, double *relres, int *status) {
  const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
  const Stencil<double> &st64 = jac ? c->jac64 : c->spe64;
  enqueue_rhs(c);
  *iters = 0;
  *outer = 0;
  *status = 0;
  if (c->cfg.solver == CFDGB_RBSOR) {
    L(c, K_RNORM, 1, [&] { launch_vec_norm64(c->stream, c->nblk, c->g, c->b, c->part, c->ss); });
    int sweeps = 0;
    for (;;) {
      L(c, K_RNORM, 1, [&] { launch_residual_norm64(c->stream, c->nblk, c->g, c->spe64, c->b, c->x, c->part, c->ss); });
      CK(cudaMemcpyAsync(c->h_ss, c->ss, sizeof(StepScal), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      *relres = c->h_ss->relres;
      if (c->h_ss->relres < c->cfg.tol) break;
      if (sweeps >= c->cfg.maxit || !std::isfinite(c->h_ss->relres)) {
        *status = std::isfinite(c->h_ss->relres) ? CFDGB_ENOCONV : CFDGB_ENAN;
        break;
      }
      for (int q = 0; q < c->cfg.check_every; ++q)
        L(c, K_RBSOR, 2, [&] { launch_rbsor_sweep(c->stream, c->nblk, c->g, c->spe64, c->b, c->x, c->omega); });
      sweeps += c->cfg.check_every;
    }
    *iters = sweeps;
    return 0;
  }
  if (c->cfg.precision == CFDGB_FP64) {
    TRY(set_solver_params(c, c->sc, c->cfg.tol, c->cfg.maxit));
    L(c, K_SETUP64, 1, [&] { launch_setup64(c, st64); });
    SolverScal r;
    TRY(run_chunks(c, false, &r));
    if (r.status == CFDGB_ENOCONV)
      L(c, K_NANRESET, 2, [&] { launch_bicg_nan_reset(c->stream, c->nblk, c->g, c->x, c->px1, c->px2, c->part, c->sc); });
    *iters = r.iter;
    *relres = r.relres;
    *status = r.status;
    return 0;
  }
  return solve_mixed(c, c->cfg.tol, iters, outer, relres, status);
}

// MIXED solve of the context's system on b (rows of the context's solver) from the warm
// start x, to relative residual tol; iters, outer, relres and status as solve_pressure's
int solve_mixed(cfdgb_ctx *c, double tol, int *iters, int *outer, double *relres, int *status) {
  const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
  const Stencil<double> &st64 = jac ? c->jac64 : c->spe64;
  *iters = 0;
  *outer = 0;
  *status = 0;
  // MIXED: FP32 BiCGSTAB sweeps inside FP64 iterative refinement (defect correction).
  // Each sweep starts afresh from the FP64 residual and stops once its own residual has
  // dropped by inner_tol (or looks converged); the refinement adds its correction to the
  // FP64 solution and recomputes the residual in FP64.  The FP64 residual is the
  // convergence and divergence test: when a sweep's FP32 residual has drifted from it, or
  // it runs away, the last correction is taken back if it raised the residual and the FP64
  // BiCGSTAB finishes from the current solution, so the mode always ends at the FP64
  // tolerance.
  static const bool trace = std::getenv("CFDGB_TRACE") != nullptr;
  const int jacf = jac ? 1 : 0;
  auto residual = [&](int flags, double *rel) -> int {
    L(c, K_RESID64, 1, [&] {
      launch_residual64(c->stream, c->nblk, c->g, st64, jacf, c->b, c->x, c->rf, c->part, c->ss, c->sc32, flags);
    });
    CK(cudaMemcpyAsync(c->h_ss, c->ss, sizeof(StepScal), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *rel = c->h_ss->relres;
    return 0;
  };
  double rel = 0.0;
  TRY(residual(3, &rel));
  const double scale = sweep_scale(c->h_ss->rnorm);  // as the residual kernel set it
  *relres = rel;
  if (trace) std::fprintf(stderr, "[cfdgb] step %d relres %.3e\n", c->loop, rel);
  if (!std::isfinite(rel)) {
    *status = CFDGB_ENAN;
    return 0;
  }
  if (rel < tol) return 0;
  TRY(set_solver_params(c, c->sc32, tol, c->cfg.maxit));
  if (c->test_wait_fault) {  // one shot
    static const int one = 1;
    CK(cudaMemcpyAsync(&c->sc32->test_wait, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->test_wait_fault = false;
  }
  L(c, K_SETUP32, 1, [&] {
    launch_refine_start32(c->stream, c->g, st64, jacf, c->k32, c->p32, c->ap32, c->rf, c->ss, sweep_reduction(c), sweep_peak(c), 1,
                          c->part, c->sc32);
  });
  bool finish64 = false;
  double best = rel;
  for (int o = 0;; ++o) {
    SolverScal r;
    TRY(run_chunks(c, true, &r));
    *iters = r.iter;
    // the sweep's correction: its last iterate, or (BiCGSTAB) the best one it kept when the
    // last is worse, as after a residual peak or a breakdown; CG keeps none.  A kept iterate
    // counts only beyond the sweep's start (its residual at least halved): a zero correction
    // would start the next sweep from the same residual, and that sweep would repeat this one
    const bool broke = r.status == CFDGB_ENAN || (r.status == CFDGB_ENOCONV && r.iter < c->cfg.maxit);
    const bool bicg = c->cfg.solver != CFDGB_CG;
    const bool kept = bicg && r.snap_rel < r.rel0;
    const bool last = !kept || (!broke && r.relres <= r.snap_rel);
    const float *e = last ? c->k32.x : c->k32.xb;
    const double est = last ? r.relres : r.snap_rel;
    if (broke && !kept) {
      // the FP32 iteration broke down or diverged before it kept any progress
      if (trace) std::fprintf(stderr, "[cfdgb]   FP32 stopped: status %d at %d\n", r.status, r.iter);
      finish64 = true;
      break;
    }
    L(c, K_CORRECT64, 2, [&] {
      launch_sum32(c->stream, c->g, e, c->part, c->ss);
      launch_correct64(c->stream, c->nblk, c->g, c->x, e, scale, c->ss);
    });
    double rn = 0.0;
    TRY(residual(0, &rn));
    *outer = o + 1;
    if (trace)
      std::fprintf(stderr, "[cfdgb]   refinement %d after %d FP32 iterations: relres %.3e (FP32 estimate %.3e%s)\n",
                   o + 1, r.iter, rn, est, last ? "" : ", kept iterate");
    // the FP32 recursion must still track the true residual (BiCGSTAB's residual is not
    // monotone, so a larger one alone is no failure).  A sweep whose estimate has drifted
    // still counts when the true residual at least halved (a long CG sweep on a fine grid
    // ends a little short of its FP32 estimate); otherwise, or when the residual runs away,
    // the correction is taken back when it made things worse and FP64 finishes
    const bool drifted = !(std::fabs(rn - est) <= 0.5 * rn);
    if (!std::isfinite(rn) || (drifted && !(rn <= 0.5 * rel)) || rn > 1e3 * best) {
      if (!(rn <= rel))
        L(c, K_CORRECT64, 1, [&] { launch_correct64(c->stream, c->nblk, c->g, c->x, e, -scale, c->ss); });
      else
        *relres = rn;
      finish64 = true;
      break;
    }
    rel = rn;
    best = std::min(best, rn);
    *relres = rn;
    if (rn < tol) break;
    if (r.status == CFDGB_ENOCONV && !broke) {  // iteration cap
      *status = CFDGB_ENOCONV;
      break;
    }
    if (o + 1 >= c->cfg.max_outer) {
      finish64 = true;
      break;
    }
    L(c, K_SETUP32, 1, [&] {
      launch_refine_start32(c->stream, c->g, st64, jacf, c->k32, c->p32, c->ap32, c->rf, c->ss, sweep_reduction(c), sweep_peak(c), 0,
                            c->part, c->sc32);
    });
  }
  if (finish64) {
    TRY(set_solver_params(c, c->sc, tol, c->cfg.maxit));
    L(c, K_SETUP64, 1, [&] { launch_setup64(c, st64); });
    SolverScal r;
    TRY(run_chunks(c, false, &r));
    if (trace) std::fprintf(stderr, "[cfdgb]   FP64 finish iters %d status %d relres %.3e\n", r.iter, r.status, r.relres);
    *iters += r.iter;
    *relres = r.relres;
    *status = r.status;
  }
  return 0;
}

// time-step scalars at init: dt as configured, time 0, running extremes at get_Cfl's
// starting values (U_max = -1e10, U_min = 1e10, cfl.hpp:12-13)
int reset_time(cfdgb_ctx *c) {
  double h[9];
  h[0] = c->cfg.dt;
  h[1] = c->cfg.dt;
  h[2] = 0.0;
  for (int q = 0; q < 6; ++q) h[3 + q] = -1e10;
  static_assert(offsetof(StepScal, dt_next) == offsetof(StepScal, dt) + 8 &&
                    offsetof(StepScal, time) == offsetof(StepScal, dt) + 16 &&
                    offsetof(StepScal, urun) == offsetof(StepScal, dt) + 24,
                "StepScal time-step fields are contiguous");
  CK(cudaMemcpyAsync(&c->ss->dt, h, 9 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(&c->ss->hist, 0, 2 * sizeof(int), c->stream));  // Adams-Bashforth history empty
  static_assert(offsetof(StepScal, hslot) == offsetof(StepScal, hist) + sizeof(int), "hist, hslot adjacent");
  CK(cudaStreamSynchronize(c->stream));  // h is reused by the next call
  return 0;
}

int apply_init_bc(cfdgb_ctx *c) {
  // src/RUN_CPU.cpp:104-109: T1 = T3 = T0, then the first ghost fill and copy
  const size_t bytes = c->npad * sizeof(double);
  CK(cudaMemcpyAsync(c->ui, c->u, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->vi, c->v, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->wi, c->w, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->us, c->u, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->vs, c->v, bytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->ws, c->w, bytes, cudaMemcpyDeviceToDevice, c->stream));
  launch_bc(c->stream, c->g, c->u, c->v, c->w, c->p, c->us, c->vs, c->ws, 1, c->inlet, 0, c->part, c->ss, c->nblk);
  CK(cudaMemsetAsync(c->x, 0, c->ncell * sizeof(double), c->stream));  // X_result = 0
  CK(cudaMemsetAsync(c->px1, 0, c->ncell * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->px2, 0, c->ncell * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->sc, 0, sizeof(SolverScal), c->stream));
  CK(cudaMemsetAsync(c->sc32, 0, sizeof(SolverScal), c->stream));
  TRY(reset_time(c));
  CK(cudaGetLastError());
  c->loop = 0;
  c->have_fields = true;
  return 0;
}

// Plot3D staging: five float32 arrays on the device and their pinned host copy
int ensure_p3d(cfdgb_ctx *c) {
  if (c->p3d) return 0;
  const size_t n = (size_t)c->ncell;
  TRY(dalloc(c, &c->p3d, 5 * n));
  CK(cudaMallocHost(&c->h_p3d, 5 * n * sizeof(float)));
  return 0;
}

// Smagorinsky model: the length scale (CS delta)^2, delta = pow(Dx Dy Dz, 1/3) as
// SmagorinskyModel.hpp:74-76 computes it, per compact row (on the host, with the same pow),
// and the eddy viscosity buffer
int ensure_les(cfdgb_ctx *c) {
  if (c->nut) return 0;
  const int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
  std::vector<double> l2((size_t)c->ncell);
  const double CS = 0.18;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        const double delta = std::pow(c->Dx[i + 2] * c->Dy[j + 2] * c->Dz[k + 2], 1.0 / 3.0);
        const double l = CS * delta;
        l2[((size_t)i * ny + j) * nz + k] = l * l;
      }
  TRY(dalloc(c, &c->les_l2, l2.size()));
  TRY(dalloc(c, &c->nut, l2.size()));
  CK(cudaMemcpy(c->les_l2, l2.data(), l2.size() * sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

// The step kernels' time-step control: in a time step dt comes from the step scalars (so an
// adaptive rule needs no host round trip) and the CFL reduction keeps the running extremes
// and the next dt; a single call uses the configured dt and only reports the CFL number.
StepCtl step_ctl(const cfdgb_ctx *c, bool in_step) {
  StepCtl sc{};
  sc.dtp = in_step ? &c->ss->dt : nullptr;
  sc.ss = c->ss;
  sc.part = c->part;
  sc.in_step = in_step ? 1 : 0;
  sc.dt_mode = c->cfg.dt_mode;
  sc.Re = c->cfg.Re;
  sc.cfl_target = c->cfg.cfl_target;
  sc.dt_max = c->cfg.dt_max > 0.0 ? c->cfg.dt_max : c->cfg.dt;
  sc.time_order = in_step && c->cfg.time_order > 1 ? c->cfg.time_order : 1;
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) sc.hb[q][a] = c->hb[q][a];
  return sc;
}
// step_end mode of the velocity correction (launch_update_uf_exact)
int step_mode(const cfdgb_ctx *c) { return c->cfg.dt_mode == CFDGB_DT_FIXED ? 1 : 2; }

bool fast_convdiff(const cfdgb_ctx *c) {
  return c->cfg.precision == CFDGB_MIXED && c->cfg.scheme == CFDGB_QUICK && !c->cfg.les && c->cfg.time_order <= 1;
}

// u* of the step, with the CFL number of u* (get_Cfl, src/RUN_CPU.cpp:274) from the same
// kernel: Smagorinsky first when on; the FP32 stencil sweep for MIXED QUICK, on FP32
// copies of u, v, w made first
void convdiff(cfdgb_ctx *c, const double *u, const double *v, const double *w, double *us, double *vs, double *ws,
              bool in_step) {
  const double nu = 1.0 / c->cfg.Re;  // 0_1_SimulationVariable.hpp:26-31
  const StepCtl sc = step_ctl(c, in_step);
  if (c->cfg.les)
    L(c, K_LES, 1, [&] { launch_smagorinsky(c->stream, c->nblk, c->g, c->les_l2, u, v, w, c->nut); });
  if (fast_convdiff(c)) {
    L(c, K_MIRROR, 1, [&] { launch_mirror32(c->stream, c->g, u, v, w, c->u32, c->v32, c->w32); });
    L(c, K_CONVDIFF, 1, [&] {
      launch_convdiff_f32(c->stream, c->nblk, c->g, c->tab32, c->tab32_uni.empty() ? nullptr : c->tab32_uni.data(),
                          c->cfg.dt, nu, u, v, w, c->u32, c->v32, c->w32, us, vs,
                          ws, sc);
    });
  } else {
    L(c, K_CONVDIFF, 1, [&] {
      launch_convdiff_exact(c->stream, c->nblk, c->g, c->cfg.scheme, c->cfg.dt, nu, c->cfg.les ? c->nut : nullptr,
                            u, v, w, us, vs, ws, sc);
    });
  }
}

// 3. correction + DFIB + drag, written straight into T0 (copyVel, RUN_CPU.cpp:369-391);
// 4. ghost fill of T0 and p, copy into T1 (RUN_CPU.cpp:399-400)
void enqueue_update_bc(cfdgb_ctx *c) {
  L(c, K_UPDATE, 1, [&] {
    if (c->cfg.precision == CFDGB_MIXED)
      launch_update_uf_fast(c->stream, c->nblk, c->g, c->cfg.dt, &c->ss->dt, step_mode(c), c->cfg.lz, c->eta, c->p,
                            c->us, c->vs, c->ws, c->u, c->v, c->w, c->ui, c->vi, c->wi, c->part, c->ss);
    else
      launch_update_uf_exact(c->stream, c->nblk, c->g, c->cfg.dt, &c->ss->dt, step_mode(c), c->cfg.lz, c->eta,
                             c->p, c->us, c->vs, c->ws, c->u, c->v, c->w, nullptr, c->ui, c->vi, c->wi, c->part,
                             c->ss);
  });
  L(c, K_BC, 3 + c->g.outflow, [&] {
    launch_bc(c->stream, c->g, c->u, c->v, c->w, c->p, c->us, c->vs, c->ws, 1, c->inlet, 1, c->part, c->ss, c->nblk);
  });
}

// ---- one CUDA graph per time step ----
// The WHILE node's condition: another chunk of iterations while the solver has not decided.
// Bounded twice over: the solver decides at its iteration cap, and the body count stops
// the loop (with ENOCONV) a few chunks past the cap should that ever fail.
__global__ void k_loop_cond(cudaGraphConditionalHandle h, SolverScal *sc, StepRing *ring, int max_bodies) {
  const int b = ++ring->bodies;
  bool more = !sc->done;
  if (more && b >= max_bodies) {
    sc->done = 1;
    sc->status = CFDGB_ENOCONV;
    more = false;
  }
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// The solve parameters (bicgstabRe2's tol, restart threshold tol * 1e-7, cap) at the start
// of every graph step: cfdgb_init_fields clears the solver scalars
__global__ void k_solver_params(SolverScal *sc, double tol, int maxit) {
  sc->tol = tol;
  sc->restart_thr = tol * 1e-7;  // bicgstabRe2.hpp:53 (pRestartFactor_)
  sc->maxit = maxit;
}

// The step's scalars into the ring (what the host path reads back after each step)
__global__ void k_step_record(StepRing *ring, const SolverScal *sc, const StepScal *ss) {
  const int n = ring->n;
  if (n >= kRing) return;  // the host reads back before the ring fills
  StepRec &r = ring->rec[n];
  r.relres = sc->relres;
  r.iters = sc->iter;
  r.status = sc->status;
  r.cd = ss->cd;
  r.cl = ss->cl;
  r.cfl = ss->cfl[0];
  r.dt = ss->dt_step;
  r.time = ss->time;
  r.nan = ss->nan_flag;
  r.bodies = ring->bodies;
  ring->bodies = 0;
  ring->n = n + 1;
}

// the steps after the first run as one graph each: FP64 Krylov solvers (their loop is the
// device's own decision), kernel timing off (it times launches one by one)
bool use_step_graph(const cfdgb_ctx *c) {
  return !c->no_step_graph && !c->timing && c->cfg.precision == CFDGB_FP64 && c->cfg.solver != CFDGB_RBSOR;
}

void drop_step_graph(cfdgb_ctx *c) {
  if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
  c->step_graph = nullptr;
}

int capture_step_graph(cfdgb_ctx *c) {
  const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
  const Stencil<double> &st64 = jac ? c->jac64 : c->spe64;
  if (!c->side) CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  if (!c->ring) {
    TRY(dalloc(c, &c->ring, 1));
    CK(cudaMallocHost(&c->h_ring, sizeof(StepRing)));
    CK(cudaMemsetAsync(c->ring, 0, sizeof(StepRing), c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  c->graph_fixed = 0;
  std::fill(std::begin(c->graph_fixed_kn), std::end(c->graph_fixed_kn), 0LL);
  const int len = chunk_iters(c, false), nk = iter_kernels(c, false);
  cudaGraph_t graph = nullptr;
  c->capturing = true;
  auto done = [&](cudaError_t e) -> int {
    c->capturing = false;
    if (e != cudaSuccess) {
      cudaGraph_t g2 = nullptr;
      cudaStreamEndCapture(c->stream, &g2);  // leave no capture open on an error
      if (g2) cudaGraphDestroy(g2);
      cudaGetLastError();
      return fail(CFDGB_ECUDA, "step graph capture: %s", cudaGetErrorString(e));
    }
    return 0;
  };
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return done(e);
  convdiff(c, c->u, c->v, c->w, c->us, c->vs, c->ws, true);
  enqueue_rhs(c);
  L(c, K_SETUP64, 1, [&] { k_solver_params<<<1, 1, 0, c->stream>>>(c->sc, c->cfg.tol, c->cfg.maxit); });
  L(c, K_SETUP64, 1, [&] { launch_setup64(c, st64); });
  // the convergence loop: a WHILE node whose body is a chunk of iterations and k_loop_cond
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return done(e);
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return done(e);
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t loop_node;
  e = cudaGraphAddNode(&loop_node, g, deps, nullptr, nd, &np);
  if (e != cudaSuccess) return done(e);
  cudaGraph_t body = np.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(c->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return done(e);
  std::swap(c->stream, c->side);  // the iteration launchers enqueue on c->stream
  for (int m = 0; m < len; ++m)
    for (int part = 0; part < nk; ++part) launch_iter_kernel(c, false, part);
  const int max_bodies = c->cfg.maxit / len + 4;
  k_loop_cond<<<1, 1, 0, c->stream>>>(h, c->sc, c->ring, max_bodies);
  std::swap(c->stream, c->side);
  cudaGraph_t body_out = nullptr;
  e = cudaStreamEndCapture(c->side, &body_out);
  if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(c->stream, &loop_node, nullptr, 1,
                                                                cudaStreamSetCaptureDependencies);
  if (e != cudaSuccess) return done(e);
  // bicgstabRe2's NaN recovery after a capped solve (the kernels check the status)
  L(c, K_NANRESET, 2, [&] { launch_bicg_nan_reset(c->stream, c->nblk, c->g, c->x, c->px1, c->px2, c->part, c->sc); });
  L(c, K_TRANSFORM, 1, [&] { launch_transform(c->stream, c->nblk, c->g, c->x, c->p); });
  enqueue_update_bc(c);
  k_step_record<<<1, 1, 0, c->stream>>>(c->ring, c->sc, c->ss);
  e = cudaStreamEndCapture(c->stream, &graph);
  c->capturing = false;
  if (e != cudaSuccess) return fail(CFDGB_ECUDA, "step graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&c->step_graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    c->step_graph = nullptr;
    return fail(CFDGB_ECUDA, "step graph instantiate: %s", cudaGetErrorString(e));
  }
  return 0;
}

// n steps (each after the first of the run) as graph launches, one read-back per kRing
// steps; fills stats[0..n) and returns the worst status
int run_step_graphs(cfdgb_ctx *c, int n, cfdgb_step_stats *stats, int *worst) {
  if (!c->step_graph) TRY(capture_step_graph(c));
  const int len = chunk_iters(c, false), nk = iter_kernels(c, false);
  long long per_body = 1;  // k_loop_cond
  for (int part = 0; part < nk; ++part) per_body += (long long)iter_part_launches(c, false, part) * len;
  for (int done = 0; done < n;) {
    const int b = std::min(n - done, kRing);
    CK(cudaMemsetAsync(&c->ring->n, 0, sizeof(int), c->stream));
    for (int q = 0; q < b; ++q) CK(cudaGraphLaunch(c->step_graph, c->stream));
    CK(cudaMemcpyAsync(c->h_ring, c->ring, offsetof(StepRing, rec) + b * sizeof(StepRec), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    if (c->h_ring->n != b) return fail(CFDGB_ECUDA, "step graph: %d of %d step records", c->h_ring->n, b);
    for (int q = 0; q < b; ++q) {
      const StepRec &r = c->h_ring->rec[q];
      const int loop = ++c->loop;
      int status = r.status;
      if (r.nan && status == 0) status = CFDGB_ENAN;
      c->launches += c->graph_fixed + 1 + r.bodies * per_body;
      for (int k = 0; k < K_COUNT; ++k) c->kn[k] += c->graph_fixed_kn[k];
      for (int part = 0; part < nk; ++part)
        c->kn[iter_kid(c, false, part)] += (long long)r.bodies * len * iter_part_launches(c, false, part);
      if (stats) {
        cfdgb_step_stats &st = stats[done + q];
        st.step = loop;
        st.iters = r.iters;
        st.outer = 0;
        st.status = status;
        st.relres = r.relres;
        st.cd = r.cd;
        st.cl = r.cl;
        st.cfl = r.cfl;
        st.dt = r.dt;
        st.time = r.time;
      }
      if (status < *worst) *worst = status;
    }
    done += b;
  }
  return 0;
}

int ensure_op_buffers(cfdgb_ctx *c) {
  if (c->op[0]) return 0;
  for (int q = 0; q < 7; ++q) TRY(dalloc(c, &c->op[q], c->npad));
  TRY(dalloc(c, &c->op[7], 3 * c->npad));
  TRY(dalloc(c, &c->op[8], c->npad));
  for (int q = 0; q < 3; ++q) TRY(dalloc(c, &c->opc[q], c->ncell));
  return 0;
}

// the coarsest level's dense pseudo-inverse, when it is small enough
template <typename T>
int upload_dense_coarse(cfdgb_ctx *c, MgPlanT<T> &mg) {
  std::vector<T> M;
  mg.cinv = nullptr;
  if (!mg_dense_inverse(mg, M)) return 0;
  T *d = nullptr;
  TRY(dalloc(c, &d, M.size()));
  CK(cudaMemcpy(d, M.data(), M.size() * sizeof(T), cudaMemcpyHostToDevice));
  mg.cinv = d;
  return 0;
}

int h2d(cfdgb_ctx *c, double *d, const double *h, size_t n) {
  CK(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return 0;
}
int d2h(cfdgb_ctx *c, double *h, const double *d, size_t n) {
  CK(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return 0;
}
int sync(cfdgb_ctx *c) {
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

}  // namespace

extern "C" {

int cfdgb_abi_version(void) { return CFDGB_ABI_VERSION; }
static_assert(K_COUNT <= 64, "graph_fixed_kn holds every kernel id");
const char *cfdgb_last_error(void) { return g_last_error.c_str(); }

int cfdgb_config_default(cfdgb_config *c) {
  if (!c) return fail(CFDGB_EINVAL, "null config");
  std::memset(c, 0, sizeof(*c));
  c->nx = 96; c->ny = 48; c->nz = 4;
  c->lx = 24.0; c->ly = 12.0; c->lz = 1.0;
  c->cx = 6.0; c->cy = 6.0; c->radius = 0.5;
  c->Re = 100.0; c->dt = 0.005;
  c->solver = CFDGB_BICGSTAB;
  c->precision = CFDGB_FP64;
  c->tol = 1e-8;
  c->maxit = 5000;
  c->omega = 1.7;
  c->inner_tol = 0.0;  // each solver's own sweep reduction (sweep_reduction)
  c->max_outer = 400;
  c->check_every = 10;
  c->dfib = 1;
  c->seed = 0;
  c->amp = 0.0;
  c->dt_mode = CFDGB_DT_FIXED;
  c->cfl_target = 0.5;
  c->dt_max = 0.0;  // 0: the configured dt
  c->time_order = 1;
  return 0;
}

int cfdgb_create(const cfdgb_config *cfg, cfdgb_ctx **out) {
  if (!out) return fail(CFDGB_EINVAL, "null output pointer");
  *out = nullptr;
  TRY(validate(cfg));
  cfdgb_ctx *c = new cfdgb_ctx();
  c->cfg = *cfg;
  auto bail = [&](int rc) { cfdgb_destroy(c); return rc; };
  if (cudaGetDevice(&c->device) != cudaSuccess) return bail(fail(CFDGB_ECUDA, "no CUDA device"));
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) return bail(fail(CFDGB_ECUDA, "device query"));
  c->nsm = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(CFDGB_ECUDA, "stream create"));
  // grid (structureGrid.hpp:336-367): uniform, X[0] = -2 dx, running sums
  const int nx = cfg->nx + 4, ny = cfg->ny + 4, nz = cfg->nz + 4;
  auto axis = [](std::vector<double> &Xa, std::vector<double> &D, std::vector<double> &Ds, int n, double l) {
    const double d = l / (n - 2.0 * 2);
    Xa.assign(n + 1, 0.0);
    Xa[0] = 0.0 - 2.0 * d;
    for (int q = 1; q < n + 1; ++q) Xa[q] = Xa[q - 1] + d;
    D.assign(n, d);
    Ds.assign(n, d);
  };
  axis(c->X, c->Dx, c->Dxs, nx, cfg->lx);
  axis(c->Y, c->Dy, c->Dys, ny, cfg->ly);
  axis(c->Z, c->Dz, c->Dzs, nz, cfg->lz);
  if (cfg->grid == CFDGB_GRID_SML) {  // init_nonuniform_SML, structureGrid.hpp:312-329
    sml_axis(c->X, c->Dx, c->Dxs, 0.3 * cfg->lx, 100, -4, cfg->lx, nx);
    sml_axis(c->Y, c->Dy, c->Dys, 0.3 * cfg->ly, 100, 0, cfg->ly, ny);
    sml_axis(c->Z, c->Dz, c->Dzs, 0.5 * cfg->lz, 0, 0, cfg->lz, nz);
  }
  c->npad = (long long)nx * ny * nz;
  c->ncell = (long long)cfg->nx * cfg->ny * cfg->nz;
  build_stencils(c);
  // reduction grid: a fixed number of resident blocks
  c->nblk = (int)std::min<long long>((c->ncell + kBlock - 1) / kBlock, (long long)c->nsm * 8);
  c->chunk_len = c->ncell > (1LL << 22) ? 8 : 32;
  c->omega = cfg->omega > 0.0 ? cfg->omega : sor_omega_opt(cfg);
  c->test_wait_fault = std::getenv("CFDGB_TEST_WAIT_FAULT") != nullptr;
  c->no_step_graph = std::getenv("CFDGB_NO_STEP_GRAPH") != nullptr;
  int rc = 0;
  const int nmet = nx + ny + nz;
  if ((rc = dalloc(c, &c->metric, 2 * (size_t)nmet))) return bail(rc);
  std::vector<double> met;
  for (auto *v : {&c->Dx, &c->Dy, &c->Dz, &c->Dxs, &c->Dys, &c->Dzs}) met.insert(met.end(), v->begin(), v->end());
  if (cudaMemcpy(c->metric, met.data(), met.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(CFDGB_ECUDA, "metric upload"));
  if ((rc = dalloc(c, &c->Xd, nx + 1)) || (rc = dalloc(c, &c->Yd, ny + 1))) return bail(rc);
  cudaMemcpy(c->Xd, c->X.data(), (nx + 1) * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(c->Yd, c->Y.data(), (ny + 1) * sizeof(double), cudaMemcpyHostToDevice);
  const int L = std::max(nx, std::max(ny, nz)) + 1;
  std::vector<float> tab = build_tab32(c, L);
  if ((rc = dalloc(c, &c->tab32, tab.size()))) return bail(rc);
  cudaMemcpy(c->tab32, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice);
  {  // every row one value along its axis (a uniform grid): the kernel takes them as parameters
    const int ext[3] = {nx, ny, nz};
    bool uni = true;
    std::vector<float> u1(3 * 11);
    for (int a = 0; a < 3 && uni; ++a)
      for (int r = 0; r < 11 && uni; ++r) {
        const float *row = tab.data() + ((size_t)a * 11 + r) * L;
        u1[a * 11 + r] = row[0];
        for (int q = 1; q < ext[a]; ++q)
          if (row[q] != row[0]) uni = false;
      }
    if (uni) c->tab32_uni = u1;
  }
  Geo &g = c->g;
  g.nxc = cfg->nx; g.nyc = cfg->ny; g.nzc = cfg->nz;
  g.walls = cfg->walls;
  g.pz = cfg->bc_z == CFDGB_Z_PERIODIC ? 1 : 0;
  g.outflow = cfg->outflow == CFDGB_OUTFLOW_CONVECTIVE ? 1 : 0;
  g.uconv = inlet_mean(c, nullptr);
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.sx = (long long)ny * nz; g.sy = nz;
  g.ncell = c->ncell;
  g.Dx = c->metric; g.Dy = g.Dx + nx; g.Dz = g.Dy + ny;
  g.Dxs = g.Dz + nz; g.Dys = g.Dxs + nx; g.Dzs = g.Dys + ny;
  {  // reciprocals of the metrics and the DFIB face factors, one IEEE division each
    std::vector<double> rm;
    for (auto *v : {&c->Dx, &c->Dy, &c->Dz, &c->Dxs, &c->Dys, &c->Dzs})
      for (double d : *v) rm.push_back(1.0 / d);
    const std::vector<double> *DD[3] = {&c->Dx, &c->Dy, &c->Dz}, *DS[3] = {&c->Dxs, &c->Dys, &c->Dzs};
    for (int a = 0; a < 3; ++a)
      for (size_t q = 0; q < DD[a]->size(); ++q) rm.push_back(((*DS[a])[q] * 0.5) / (*DD[a])[q]);
    double *drm = nullptr;
    if ((rc = dalloc(c, &drm, rm.size()))) return bail(rc);
    if (cudaMemcpy(drm, rm.data(), rm.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(CFDGB_ECUDA, "metric reciprocal upload"));
    g.rDx = drm; g.rDy = g.rDx + nx; g.rDz = g.rDy + ny;
    g.rDxs = g.rDz + nz; g.rDys = g.rDxs + nx; g.rDzs = g.rDys + ny;
    g.hfx = g.rDzs + nz; g.hfy = g.hfx + nx; g.hfz = g.hfy + ny;
  }
  g.div2 = division_twice(c) ? 1 : 0;
  g.uni = 1;
  for (auto *v : {&c->Dx, &c->Dy, &c->Dz, &c->Dxs, &c->Dys, &c->Dzs})
    for (double d : *v)
      if (d != v->front()) g.uni = 0;
  if (cfg->grid == CFDGB_GRID_SML) {
    // per-axis operator factors and the Jacobi scale of every row (createPressureMatrixCSR)
    const Coef C{c};
    std::vector<double> fac;
    for (int q = 0; q < cfg->nx; ++q) fac.push_back(C.xm(q));
    for (int q = 0; q < cfg->nx; ++q) fac.push_back(C.xp(q));
    for (int q = 0; q < cfg->ny; ++q) fac.push_back(C.ym(q));
    for (int q = 0; q < cfg->ny; ++q) fac.push_back(C.yp(q));
    for (int q = 0; q < cfg->nz; ++q) fac.push_back(C.zm(q));
    for (int q = 0; q < cfg->nz; ++q) fac.push_back(C.zp(q));
    std::vector<double> jp((size_t)c->ncell);
    for (int i = 0; i < cfg->nx; ++i)
      for (int j = 0; j < cfg->ny; ++j)
        for (int k = 0; k < cfg->nz; ++k) {
          double aa = 0.0, bb = 0.0, cc = 0.0;
          if (i == 0) aa = -C.xm(i);
          if (i == cfg->nx - 1) aa = -C.xp(i);
          if (j == 0) bb = -C.ym(j);
          if (j == cfg->ny - 1) bb = -C.yp(j);
          if (k == 0 && !g.pz) cc = -C.zm(k);
          if (k == cfg->nz - 1 && !g.pz) cc = -C.zp(k);
          const double dj = C.xm(i) + C.ym(j) + C.zm(k) + C.xp(i) + C.yp(j) + C.zp(k) + aa + bb + cc;
          jp[((size_t)i * cfg->ny + j) * cfg->nz + k] = 1.0 / dj;
        }
    double *dfac = nullptr, *djp = nullptr;
    if ((rc = dalloc(c, &dfac, fac.size())) || (rc = dalloc(c, &djp, jp.size()))) return bail(rc);
    if (cudaMemcpy(dfac, fac.data(), fac.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(djp, jp.data(), jp.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(CFDGB_ECUDA, "stretched-grid factor upload"));
    g.nonuni = 1;
    g.fxm = dfac; g.fxp = g.fxm + cfg->nx;
    g.fym = g.fxp + cfg->nx; g.fyp = g.fym + cfg->ny;
    g.fzm = g.fyp + cfg->ny; g.fzp = g.fzm + cfg->nz;
    g.jpv = djp;
    double *rows = nullptr;
    if ((rc = dalloc(c, &rows, 14 * (size_t)c->ncell))) return bail(rc);
    g.cof[0] = rows;
    g.cof[1] = rows + 7 * c->ncell;
  }
  // solver launch geometry: k along x (k_block_width), j along y, i strided over grid z
  g.lbx = k_block_width(cfg->nz);
  g.lby = kBlock / g.lbx;
  g.lgx = (cfg->nz + g.lbx - 1) / g.lbx;
  g.lgy = (cfg->ny + g.lby - 1) / g.lby;
  g.lgz = std::max(1, std::min(cfg->nx, c->nsm * 8 / std::max(1, g.lgx * g.lgy)));
  int nblk3 = g.lgx * g.lgy * g.lgz;
  // vectorised FP32 kernels: quads of four k cells per thread when nz % 4 == 0
  // (the stretched grid's MIXED sweeps run the scalar kernels, on its stored FP32 rows)
  // the flat pointwise kernels (every SM filled): the FP32 quad kernels and the MIXED
  // refinement's sum and correction on any grid
  g.xgrid = c->nsm * fp32_pointwise_blocks_per_sm();
  nblk3 = std::max(nblk3, g.xgrid);
  if (cfg->nz % 4 == 0 && !std::getenv("CFDGB_SCALAR_FP32") && cfg->grid != CFDGB_GRID_SML) {
    const int nq = cfg->nz / 4;
    g.vbx = 1;
    while (g.vbx < nq && g.vbx < 32) g.vbx *= 2;
    g.vby = kBlock / g.vbx;
    g.vgx = (nq + g.vbx - 1) / g.vbx;
    g.vgy = (cfg->ny + g.vby - 1) / g.vby;
    // the stencil kernels march along x through chunks of planes: a few resident blocks
    // per SM, each with a long chunk (one extra plane read per chunk)
    const char *bps = std::getenv("CFDGB_FP32_BLOCKS_PER_SM");
    const int per_sm = bps ? std::max(1, std::atoi(bps)) : 4;
    g.vgz = std::max(1, std::min(cfg->nx, c->nsm * per_sm / std::max(1, g.vgx * g.vgy)));
    nblk3 = std::max(nblk3, g.vgx * g.vgy * g.vgz);
    int tbps = 0, tbps2 = 0;
    if (!std::getenv("CFDGB_NO_TMA") && fp32_stage_plan(cfg->nz, &g.tj, &g.tsmem, &tbps, &g.tsmem2, &tbps2)) {
      g.tma = 1;
      g.tgx = (cfg->ny + g.tj - 1) / g.tj;
      g.tgy = std::max(1, std::min(cfg->nx, c->nsm * tbps / g.tgx));  // one wave of resident blocks
      g.tgy2 = std::max(1, std::min(cfg->nx, c->nsm * tbps2 / g.tgx));
      nblk3 = std::max(nblk3, g.tgx * std::max(g.tgy, g.tgy2));
    }
  }
  if (g.nonuni) {  // the stored rows, from the same per-axis factors and jpv
    launch_build_rows(c->stream, g, 0, const_cast<double *>(g.cof[0]));
    launch_build_rows(c->stream, g, 1, const_cast<double *>(g.cof[1]));
    if (cfg->precision == CFDGB_MIXED) {
      float *r32 = nullptr;
      if ((rc = dalloc(c, &r32, 14 * (size_t)c->ncell))) return bail(rc);
      launch_rows_f32(c->stream, 14 * c->ncell, g.cof[0], r32);  // cof[1] follows cof[0]
      g.cof32[0] = r32;
      g.cof32[1] = r32 + 7 * c->ncell;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(fail(CFDGB_ECUDA, "stretched-grid rows"));
  }
  // fields and solver vectors
  double **pad[] = {&c->u, &c->v, &c->w, &c->us, &c->vs, &c->ws, &c->ui, &c->vi, &c->wi, &c->p, &c->eta};
  for (auto **q : pad)
    if ((rc = dalloc(c, q, c->npad))) return bail(rc);
  double **cmp[] = {&c->b, &c->x, &c->px1, &c->px2};
  for (auto **q : cmp)
    if ((rc = dalloc(c, q, c->ncell))) return bail(rc);
  c->k64.x = c->x;
  if (cfg->solver != CFDGB_RBSOR) {  // MIXED keeps them for its FP64 finish
    double **kv[] = {&c->k64.r0, &c->k64.r1, &c->k64.p1, &c->k64.s, &c->k64.ap, &c->k64.as};
    for (auto **q : kv)
      if ((rc = dalloc(c, q, c->ncell))) return bail(rc);
  }
  if (cfg->precision == CFDGB_MIXED) {
    if ((rc = dalloc(c, &c->rf, c->ncell))) return bail(rc);
    float **kv[] = {&c->k32.x, &c->k32.r0, &c->k32.r1, &c->k32.s, &c->k32.as, &c->p32[0], &c->p32[1],
                    &c->ap32[0], &c->ap32[1], &c->k32.xb};
    for (auto **q : kv)
      if ((rc = dalloc(c, q, c->ncell))) return bail(rc);
  }
  if (cfg->time_order > 1) {  // Adams-Bashforth history
    for (int q = 0; q < (cfg->time_order == 3 ? 2 : 1); ++q)
      for (int a = 0; a < 3; ++a)
        if ((rc = dalloc(c, &c->hb[q][a], c->npad))) return bail(rc);
    if (cfg->time_order == 2)
      for (int a = 0; a < 3; ++a) c->hb[1][a] = c->hb[0][a];
  }
  if (cfg->precision == CFDGB_MIXED && cfg->scheme == CFDGB_QUICK && !cfg->les && cfg->time_order <= 1) {
    if ((rc = dalloc(c, &c->u32, c->npad)) || (rc = dalloc(c, &c->v32, c->npad)) || (rc = dalloc(c, &c->w32, c->npad)))
      return bail(rc);
  }
  if (cfg->precond == CFDGB_PRECOND_MULTIGRID && cfg->precision == CFDGB_FP64) {  // the FP64 hierarchy
    mg_plan(cfg->nx, cfg->ny, cfg->nz, cfg->lx / cfg->nx, cfg->ly / cfg->ny, cfg->lz / cfg->nz, c->nsm, false,
            &c->mg64, g.pz != 0);
    mg_prepare<double>();
    if ((rc = upload_dense_coarse(c, c->mg64))) return bail(rc);
    if ((rc = dalloc(c, &c->ph64, c->ncell)) || (rc = dalloc(c, &c->sh64, c->ncell))) return bail(rc);
    for (int l = 1; l < c->mg64.nlev; ++l) {
      MgLevelT<double> &L = c->mg64.lev[l];
      const size_t n = (size_t)L.nx * L.ny * L.nz;
      if ((rc = dalloc(c, &L.x, n)) || (rc = dalloc(c, &L.b, n))) return bail(rc);
    }
    c->use_mg64 = true;
  }
  if (cfg->precond == CFDGB_PRECOND_MULTIGRID && cfg->precision == CFDGB_MIXED) {  // levels >= 1, M p, M s
    mg_plan(cfg->nx, cfg->ny, cfg->nz, cfg->lx / cfg->nx, cfg->ly / cfg->ny, cfg->lz / cfg->nz, c->nsm,
            !std::getenv("CFDGB_SCALAR_FP32"), &c->mg, g.pz != 0);
    if (std::getenv("CFDGB_MG_PER_PASS"))  // every level on the per-pass kernels (tests compare)
      for (int l = 0; l < c->mg.nlev; ++l) c->mg.lev[l].march = 0;
    mg_prepare<float>();
    if ((rc = upload_dense_coarse(c, c->mg))) return bail(rc);
    if ((rc = dalloc(c, &c->ph32, c->ncell)) || (rc = dalloc(c, &c->sh32, c->ncell))) return bail(rc);
    for (int l = 1; l < c->mg.nlev; ++l) {
      MgLevel &L = c->mg.lev[l];
      const size_t n = (size_t)L.nx * L.ny * L.nz;
      if ((rc = dalloc(c, &L.x, n)) || (rc = dalloc(c, &L.b, n))) return bail(rc);
    }
    c->use_mg = true;
  }
  if ((rc = dalloc(c, &c->part, 8 * (size_t)std::max(c->nblk, nblk3)))) return bail(rc);
  if ((rc = dalloc(c, &c->sc, 1)) || (rc = dalloc(c, &c->sc32, 1)) || (rc = dalloc(c, &c->ss, 1))) return bail(rc);
  cudaMemset(c->sc, 0, sizeof(SolverScal));
  cudaMemset(c->sc32, 0, sizeof(SolverScal));
  cudaMemset(c->ss, 0, sizeof(StepScal));
  if (cudaMallocHost(&c->h_sc, sizeof(SolverScal)) != cudaSuccess ||
      cudaMallocHost(&c->h_ss, sizeof(StepScal)) != cudaSuccess)
    return bail(fail(CFDGB_ENOMEM, "pinned scalars"));
  // solid fraction (DFIB_CylinderZ, RUN_CPU.cpp:228-234)
  cudaMemsetAsync(c->eta, 0, c->npad * sizeof(double), c->stream);
  if (cfg->dfib) launch_eta(c->stream, c->nblk, c->g, c->Xd, c->Yd, cfg->cx, cfg->cy, cfg->radius, c->eta);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(CFDGB_ECUDA, "set-up kernels: %s", cudaGetErrorString(cudaGetLastError())));
  if (cfg->les && (rc = ensure_les(c))) return bail(rc);
  *out = c;
  return 0;
}

int cfdgb_destroy(cfdgb_ctx *c) {
  if (!c) return 0;
  if (c->stream) cudaStreamSynchronize(c->stream);
  resolve_events(c);
  for (auto e : c->ev_free) cudaEventDestroy(e);
  if (c->chunk64) cudaGraphExecDestroy(c->chunk64);
  if (c->chunk32) cudaGraphExecDestroy(c->chunk32);
  drop_step_graph(c);
  if (c->h_ring) cudaFreeHost(c->h_ring);
  if (c->side) cudaStreamDestroy(c->side);
  for (void *q : c->allocs) cudaFree(q);
  if (c->h_p3d) cudaFreeHost(c->h_p3d);
  if (c->h_sc) cudaFreeHost(c->h_sc);
  if (c->h_ss) cudaFreeHost(c->h_ss);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return 0;
}

int cfdgb_padded_dims(const cfdgb_ctx *c, int *nxp, int *nyp, int *nzp) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (nxp) *nxp = c->g.nx;
  if (nyp) *nyp = c->g.ny;
  if (nzp) *nzp = c->g.nz;
  return 0;
}

int cfdgb_stream(const cfdgb_ctx *c, void **s) {
  if (!c || !s) return fail(CFDGB_EINVAL, "null argument");
  *s = (void *)c->stream;
  return 0;
}

int cfdgb_init_fields(cfdgb_ctx *c, const double *u, const double *v, const double *w, const double *p) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  const size_t n = c->npad;
  std::vector<double> hu, hv, hw;
  if (!u || !v || !w) {
    // iniU(1, 0, 0) (RUN_CPU.cpp:66-76) plus the seeded perturbation of the interior
    hu.assign(n, 1.0);
    hv.assign(n, 0.0);
    hw.assign(n, 0.0);
    if (c->cfg.amp != 0.0) {
      uint64_t s = c->cfg.seed;
      std::vector<double> *f[3] = {&hu, &hv, &hw};
      for (auto *fa : f)
        for (int i = 2; i < c->g.nx - 2; ++i)
          for (int j = 2; j < c->g.ny - 2; ++j)
            for (int k = 2; k < c->g.nz - 2; ++k) {
              const double r = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
              (*fa)[((size_t)i * c->g.ny + j) * c->g.nz + k] += c->cfg.amp * (2.0 * r - 1.0);
            }
    }
    if (u) std::memcpy(hu.data(), u, n * sizeof(double));
    if (v) std::memcpy(hv.data(), v, n * sizeof(double));
    if (w) std::memcpy(hw.data(), w, n * sizeof(double));
    u = hu.data(); v = hv.data(); w = hw.data();
  }
  TRY(h2d(c, c->u, u, n));
  TRY(h2d(c, c->v, v, n));
  TRY(h2d(c, c->w, w, n));
  if (p) TRY(h2d(c, c->p, p, n));
  else CK(cudaMemsetAsync(c->p, 0, n * sizeof(double), c->stream));
  TRY(apply_init_bc(c));
  return sync(c);
}

int cfdgb_set_fields(cfdgb_ctx *c, const double *u, const double *v, const double *w, const double *p) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (!c->have_fields) return fail(CFDGB_ESTATE, "init_fields must come first");
  const size_t n = c->npad;
  if (u) TRY(h2d(c, c->u, u, n));
  if (v) TRY(h2d(c, c->v, v, n));
  if (w) TRY(h2d(c, c->w, w, n));
  // p is the padded pressure (t1.p); the solver's warm start (X_result) is kept as is
  if (p) TRY(h2d(c, c->p, p, n));
  CK(cudaGetLastError());
  return 0;
}

int cfdgb_get_fields(cfdgb_ctx *c, double *u, double *v, double *w, double *p) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  const size_t n = c->npad;
  if (u) TRY(d2h(c, u, c->u, n));
  if (v) TRY(d2h(c, v, c->v, n));
  if (w) TRY(d2h(c, w, c->w, n));
  if (p) TRY(d2h(c, p, c->p, n));
  return sync(c);
}

int cfdgb_get_eta(cfdgb_ctx *c, double *eta) {
  if (!c || !eta) return fail(CFDGB_EINVAL, "null argument");
  TRY(d2h(c, eta, c->eta, c->npad));
  return sync(c);
}

int cfdgb_set_eta(cfdgb_ctx *c, const double *eta) {
  if (!c || !eta) return fail(CFDGB_EINVAL, "null argument");
  TRY(h2d(c, c->eta, eta, c->npad));
  return sync(c);
}

int cfdgb_step(cfdgb_ctx *c, int nsteps, cfdgb_step_stats *stats) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (!c->have_fields) TRY(cfdgb_init_fields(c, nullptr, nullptr, nullptr, nullptr));
  if (nsteps < 0) return fail(CFDGB_EINVAL, "negative step count");
  const double nu = 1.0 / c->cfg.Re;  // 0_1_SimulationVariable.hpp:26-31
  int worst = 0;
  for (int s = 0; s < nsteps; ++s) {
    if (c->loop >= 1 && use_step_graph(c)) {  // the remaining steps, one graph each
      TRY(run_step_graphs(c, nsteps - s, stats ? stats + s : nullptr, &worst));
      break;
    }
    const int loop = ++c->loop;
    // 1. u* (RUN_CPU.cpp:268) and, from the same kernel, the CFL diagnostic on u* (get_Cfl,
    // RUN_CPU.cpp:274) with the next dt of an adaptive rule (timestepper, :275)
    convdiff(c, c->u, c->v, c->w, c->us, c->vs, c->ws, true);
    // 2. pressure, not at the first step (RUN_CPU.cpp:303)
    int iters = 0, outer = 0, status = 0;
    double relres = 0.0;
    if (loop > 1) {
      TRY(solve_pressure(c, &iters, &outer, &relres, &status));
      L(c, K_TRANSFORM, 1, [&] { launch_transform(c->stream, c->nblk, c->g, c->x, c->p); });
    }
    // 3. correction + DFIB + drag into T0, 4. ghost fill and copy into T1
    enqueue_update_bc(c);
    CK(cudaMemcpyAsync(c->h_ss, c->ss, sizeof(StepScal), cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    resolve_events(c);
    if (c->h_ss->nan_flag && status == 0) status = CFDGB_ENAN;
    if (stats) {
      cfdgb_step_stats &st = stats[s];
      st.step = loop;
      st.iters = iters;
      st.outer = outer;
      st.status = status;
      st.relres = relres;
      st.cd = c->h_ss->cd;
      st.cl = c->h_ss->cl;
      st.cfl = c->h_ss->cfl[0];
      st.dt = c->h_ss->dt_step;
      st.time = c->h_ss->time;
    }
    if (status < worst) worst = status;
  }
  if (worst < 0) fail(worst, "step finished with status %d", worst);
  return worst;
}

int cfdgb_pressure_solve(cfdgb_ctx *c, int *iters, double *relres) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (!c->have_fields) return fail(CFDGB_ESTATE, "init_fields must come first");
  int it = 0, outer = 0, status = 0;
  double rr = 0.0;
  TRY(solve_pressure(c, &it, &outer, &rr, &status));
  launch_transform(c->stream, c->nblk, c->g, c->x, c->p);
  TRY(sync(c));
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return status;
}

int cfdgb_set_kernel_timing(cfdgb_ctx *c, int enable) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (c->timing) {
    CK(cudaStreamSynchronize(c->stream));
    resolve_events(c);
  }
  c->timing = enable != 0;
  return 0;
}

int cfdgb_reset_counters(cfdgb_ctx *c) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  CK(cudaStreamSynchronize(c->stream));
  resolve_events(c);
  c->launches = 0;
  for (int q = 0; q < K_COUNT; ++q) { c->kms[q] = 0.0; c->kn[q] = 0; }
  return 0;
}

int cfdgb_launch_count(const cfdgb_ctx *c, long long *launches) {
  if (!c || !launches) return fail(CFDGB_EINVAL, "null argument");
  *launches = c->launches;
  return 0;
}

int cfdgb_kernel_stat(cfdgb_ctx *c, int idx, const char **name, double *total_ms, long long *launches) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (idx < 0 || idx >= K_COUNT) return fail(CFDGB_EINVAL, "kernel index out of range");
  if (name) *name = kKernelNames[idx];
  if (total_ms) *total_ms = c->kms[idx];
  if (launches) *launches = c->kn[idx];
  return 0;
}

// ---- per-function entry points ----

int cfdgb_op_convection_diffusion(cfdgb_ctx *c, const double *u, const double *v, const double *w, double *us,
                                  double *vs, double *ws) {
  if (!c || !u || !v || !w || !us || !vs || !ws) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[0], u, n)); TRY(h2d(c, o[1], v, n)); TRY(h2d(c, o[2], w, n));
  TRY(h2d(c, o[3], us, n)); TRY(h2d(c, o[4], vs, n)); TRY(h2d(c, o[5], ws, n));
  convdiff(c, o[0], o[1], o[2], o[3], o[4], o[5], false);
  TRY(d2h(c, us, o[3], n)); TRY(d2h(c, vs, o[4], n)); TRY(d2h(c, ws, o[5], n));
  return sync(c);
}

int cfdgb_op_smagorinsky(cfdgb_ctx *c, const double *u, const double *v, const double *w, double *nut) {
  if (!c || !u || !v || !w || !nut) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  TRY(ensure_les(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[0], u, n)); TRY(h2d(c, o[1], v, n)); TRY(h2d(c, o[2], w, n));
  launch_smagorinsky(c->stream, c->nblk, c->g, c->les_l2, o[0], o[1], o[2], c->nut);
  TRY(d2h(c, nut, c->nut, (size_t)c->ncell));
  return sync(c);
}

int cfdgb_op_bc_main(cfdgb_ctx *c, double *u, double *v, double *w, double *p) {
  if (!c || !u || !v || !w || !p) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[0], u, n)); TRY(h2d(c, o[1], v, n)); TRY(h2d(c, o[2], w, n)); TRY(h2d(c, o[6], p, n));
  launch_bc(c->stream, c->g, o[0], o[1], o[2], o[6], nullptr, nullptr, nullptr, 1, nullptr, 0, c->part, c->ss,
            c->nblk);
  TRY(d2h(c, u, o[0], n)); TRY(d2h(c, v, o[1], n)); TRY(d2h(c, w, o[2], n)); TRY(d2h(c, p, o[6], n));
  return sync(c);
}

int cfdgb_op_bc_copy(cfdgb_ctx *c, const double *u, const double *v, const double *w, double *us, double *vs,
                     double *ws) {
  if (!c || !u || !v || !w || !us || !vs || !ws) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[0], u, n)); TRY(h2d(c, o[1], v, n)); TRY(h2d(c, o[2], w, n));
  TRY(h2d(c, o[3], us, n)); TRY(h2d(c, o[4], vs, n)); TRY(h2d(c, o[5], ws, n));
  launch_bc(c->stream, c->g, o[0], o[1], o[2], nullptr, o[3], o[4], o[5], 0);
  TRY(d2h(c, us, o[3], n)); TRY(d2h(c, vs, o[4], n)); TRY(d2h(c, ws, o[5], n));
  return sync(c);
}

int cfdgb_op_rhs(cfdgb_ctx *c, int jacobi, const double *us, const double *vs, const double *ws, double *b) {
  if (!c || !us || !vs || !ws || !b) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[3], us, n)); TRY(h2d(c, o[4], vs, n)); TRY(h2d(c, o[5], ws, n));
  launch_rhs_exact(c->stream, c->nblk, c->g, c->cfg.dt, nullptr, o[3], o[4], o[5], jacobi != 0, c->jac64, c->opc[0]);
  TRY(d2h(c, b, c->opc[0], c->ncell));
  return sync(c);
}

int cfdgb_op_spmv(cfdgb_ctx *c, int jacobi, const double *x, double *y) {
  if (!c || !x || !y) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  TRY(h2d(c, c->opc[0], x, c->ncell));
  launch_spmv_exact(c->stream, c->nblk, c->g, jacobi ? c->jac64 : c->spe64, c->opc[0], c->opc[1]);
  TRY(d2h(c, y, c->opc[1], c->ncell));
  return sync(c);
}

int cfdgb_op_bicgstab(cfdgb_ctx *c, int solver, double tol, int maxit, const double *rhs, double *x, int *iters,
                      double *relres) {
  if (!c || !rhs || !x) return fail(CFDGB_EINVAL, "null argument");
  if (solver != CFDGB_BICGSTAB && solver != CFDGB_BICGSTAB_JACOBI) return fail(CFDGB_EINVAL, "solver must be BiCGSTAB");
  if (c->cfg.precision != CFDGB_FP64 || c->cfg.solver == CFDGB_RBSOR)
    return fail(CFDGB_EINVAL, "op_bicgstab needs an FP64 BiCGSTAB context");
  if (!(tol > 0) || maxit < 1) return fail(CFDGB_EINVAL, "bad tol/maxit");
  // solve in the context's own Krylov buffers with the caller's rhs and warm start; the
  // context's step state (x, history) is saved and restored around the call
  std::vector<double> save_x(c->ncell), save_1(c->ncell), save_2(c->ncell);
  TRY(d2h(c, save_x.data(), c->x, c->ncell));
  TRY(d2h(c, save_1.data(), c->px1, c->ncell));
  TRY(d2h(c, save_2.data(), c->px2, c->ncell));
  SolverScal save_sc;
  CK(cudaMemcpyAsync(&save_sc, c->sc, sizeof(SolverScal), cudaMemcpyDeviceToHost, c->stream));
  TRY(sync(c));
  TRY(h2d(c, c->b, rhs, c->ncell));
  TRY(h2d(c, c->x, x, c->ncell));
  CK(cudaMemsetAsync(c->sc, 0, sizeof(SolverScal), c->stream));  // a fresh solver object
  const int keep_maxit = c->cfg.maxit;
  c->cfg.maxit = maxit;
  TRY(set_solver_params(c, c->sc, tol, maxit));
  launch_bicg_setup64(c->stream, c->nblk, c->g, solver == CFDGB_BICGSTAB_JACOBI ? c->jac64 : c->spe64, c->k64, c->b,
                      c->px1, c->px2, c->part, c->sc);
  // the chunk graph bakes in the configured operator; use direct launches here
  const Stencil<double> &st = solver == CFDGB_BICGSTAB_JACOBI ? c->jac64 : c->spe64;
  SolverScal r{};
  int rc = 0;
  for (long long q = 0; q < (long long)maxit / 8 + 3; ++q) {
    for (int m = 0; m < 8; ++m)
      for (int part = 0; part < 5; ++part) launch_bicg64_part(c->stream, part, c->g, st, c->k64, c->part, c->sc);
    CK(cudaMemcpyAsync(c->h_sc, c->sc, sizeof(SolverScal), cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    if (c->h_sc->done) { r = *c->h_sc; break; }
  }
  c->cfg.maxit = keep_maxit;
  if (r.status == CFDGB_ENOCONV) launch_bicg_nan_reset(c->stream, c->nblk, c->g, c->x, c->px1, c->px2, c->part, c->sc);
  TRY(d2h(c, x, c->x, c->ncell));
  TRY(sync(c));
  if (iters) *iters = r.iter;
  if (relres) *relres = r.relres;
  rc = r.status;
  TRY(h2d(c, c->x, save_x.data(), c->ncell));
  TRY(h2d(c, c->px1, save_1.data(), c->ncell));
  TRY(h2d(c, c->px2, save_2.data(), c->ncell));
  CK(cudaMemcpyAsync(c->sc, &save_sc, sizeof(SolverScal), cudaMemcpyHostToDevice, c->stream));
  TRY(sync(c));
  if (rc < 0) fail(rc, "bicgstab hit its iteration cap");
  return rc;
}

int cfdgb_op_update_uf(cfdgb_ctx *c, const double *eta, const double *p, const double *us, const double *vs,
                       const double *ws, double *u3, double *v3, double *w3, double *f, double *cd, double *cl) {
  if (!c || !eta || !p || !us || !vs || !ws || !u3 || !v3 || !w3) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  const size_t n = c->npad;
  double **o = c->op;
  TRY(h2d(c, o[6], eta, n)); TRY(h2d(c, o[0], p, n));
  TRY(h2d(c, o[3], us, n)); TRY(h2d(c, o[4], vs, n)); TRY(h2d(c, o[5], ws, n));
  TRY(h2d(c, o[1], u3, n)); TRY(h2d(c, o[2], v3, n)); TRY(h2d(c, o[8], w3, n));
  if (f) TRY(h2d(c, o[7], f, 3 * n));
  launch_update_uf_exact(c->stream, c->nblk, c->g, c->cfg.dt, nullptr, 0, c->cfg.lz, o[6], o[0], o[3], o[4], o[5],
                         o[1], o[2], o[8], f ? o[7] : nullptr, nullptr, nullptr, nullptr, c->part, c->ss);
  TRY(d2h(c, u3, o[1], n)); TRY(d2h(c, v3, o[2], n)); TRY(d2h(c, w3, o[8], n));
  if (f) TRY(d2h(c, f, o[7], 3 * n));
  CK(cudaMemcpyAsync(c->h_ss, c->ss, sizeof(StepScal), cudaMemcpyDeviceToHost, c->stream));
  TRY(sync(c));
  if (cd) *cd = c->h_ss->cd;
  if (cl) *cl = c->h_ss->cl;
  return 0;
}

int cfdgb_op_solid_fraction(cfdgb_ctx *c, double *eta) {
  if (!c || !eta) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  CK(cudaMemsetAsync(c->op[6], 0, c->npad * sizeof(double), c->stream));
  launch_eta(c->stream, c->nblk, c->g, c->Xd, c->Yd, c->cfg.cx, c->cfg.cy, c->cfg.radius, c->op[6]);
  TRY(d2h(c, eta, c->op[6], c->npad));
  return sync(c);
}

int cfdgb_op_cfl(cfdgb_ctx *c, const double *us, const double *vs, const double *ws, double *out7) {
  if (!c || !us || !vs || !ws || !out7) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  TRY(h2d(c, c->op[0], us, c->npad));
  TRY(h2d(c, c->op[1], vs, c->npad));
  TRY(h2d(c, c->op[2], ws, c->npad));
  launch_cfl(c->stream, c->nblk, c->g, c->cfg.dt, c->op[0], c->op[1], c->op[2], c->part, c->ss);
  CK(cudaMemcpyAsync(c->h_ss, c->ss, sizeof(StepScal), cudaMemcpyDeviceToHost, c->stream));
  TRY(sync(c));
  for (int q = 0; q < 7; ++q) out7[q] = c->h_ss->cfl[q];
  return 0;
}

int cfdgb_set_dt(cfdgb_ctx *c, double dt) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(CFDGB_EINVAL, "dt must be positive");
  c->cfg.dt = dt;
  drop_step_graph(c);  // a graph holds the CFL rule's dt bound, taken from dt
  c->g.div2 = division_twice(c) ? 1 : 0;  // dt is a divisor too
  if (c->cfg.time_order == 3 && c->ss)  // the constant-step history is of the old dt
    CK(cudaMemsetAsync(&c->ss->hist, 0, 2 * sizeof(int), c->stream));
  // the step kernels read dt from the step scalars
  const double h[2] = {dt, dt};
  CK(cudaMemcpyAsync(&c->ss->dt, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  return sync(c);
}

int cfdgb_write_plot3d(cfdgb_ctx *c, const char *xpath, const char *qpath, double time) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  const int hdr[4] = {1, c->cfg.nx, c->cfg.ny, c->cfg.nz};
  if (xpath) {  // xfileWrite.hpp:14-47: cell centres, k-j-i order (structureGrid.hpp:219)
    FILE *f = std::fopen(xpath, "wb");
    if (!f) return fail(CFDGB_EINVAL, "cannot write %s", xpath);
    std::fwrite(hdr, sizeof(int), 4, f);
    const std::vector<double> *N[3] = {&c->X, &c->Y, &c->Z};
    const int n[3] = {c->cfg.nx, c->cfg.ny, c->cfg.nz};
    std::vector<float> line;
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j) {
          line.clear();
          for (int i = 0; i < n[0]; ++i) {
            const int q = a == 0 ? i : (a == 1 ? j : k);
            line.push_back((float)(((*N[a])[q + 2] + (*N[a])[q + 3]) / 2.0));
          }
          std::fwrite(line.data(), sizeof(float), line.size(), f);
        }
    const bool ok = std::fclose(f) == 0;
    if (!ok) return fail(CFDGB_EINVAL, "write of %s failed", xpath);
  }
  if (qpath) {  // qfile.hpp:6-105: the current T0, p and eta, packed on the device
    if (!c->have_fields) return fail(CFDGB_ESTATE, "no fields yet");
    const size_t n = (size_t)c->ncell;
    TRY(ensure_p3d(c));
    launch_plot3d_pack(c->stream, c->nblk, c->g, c->p, c->u, c->v, c->w, c->eta, c->p3d);
    CK(cudaMemcpyAsync(c->h_p3d, c->p3d, 5 * n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    FILE *f = std::fopen(qpath, "wb");
    if (!f) return fail(CFDGB_EINVAL, "cannot write %s", qpath);
    const float head[4] = {0.0f, 0.0f, (float)c->cfg.Re, (float)time};  // mach, alpha, Re, time
    std::fwrite(hdr, sizeof(int), 4, f);
    std::fwrite(head, sizeof(float), 4, f);
    const size_t wrote = std::fwrite(c->h_p3d, sizeof(float), 5 * n, f);
    const bool ok = std::fclose(f) == 0 && wrote == 5 * n;
    if (!ok) return fail(CFDGB_EINVAL, "write of %s failed", qpath);
  }
  return 0;
}

int cfdgb_op_plot3d_read(cfdgb_ctx *c, const float *q, double *p, double *u, double *v, double *w, double *eta) {
  if (!c || !q || !p || !u || !v || !w || !eta) return fail(CFDGB_EINVAL, "null argument");
  TRY(ensure_op_buffers(c));
  TRY(ensure_p3d(c));
  const size_t n = (size_t)c->ncell;
  std::memcpy(c->h_p3d, q, 5 * n * sizeof(float));
  CK(cudaMemcpyAsync(c->p3d, c->h_p3d, 5 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  for (int a = 0; a < 5; ++a) CK(cudaMemsetAsync(c->op[a], 0, c->npad * sizeof(double), c->stream));
  launch_plot3d_unpack(c->stream, c->nblk, c->g, c->p3d, c->op[0], c->op[1], c->op[2], c->op[3], c->op[4]);
  double *out[5] = {p, u, v, w, eta};
  for (int a = 0; a < 5; ++a) TRY(d2h(c, out[a], c->op[a], c->npad));
  return sync(c);
}

int cfdgb_read_plot3d(cfdgb_ctx *c, const char *qpath, double *head) {
  if (!c || !qpath) return fail(CFDGB_EINVAL, "null argument");
  const size_t n = (size_t)c->ncell;
  FILE *f = std::fopen(qpath, "rb");
  if (!f) return fail(CFDGB_EINVAL, "cannot open %s", qpath);
  int ih[4] = {0, 0, 0, 0};
  float fh[4] = {0, 0, 0, 0};
  const bool hok = std::fread(ih, sizeof(int), 4, f) == 4 && std::fread(fh, sizeof(float), 4, f) == 4;
  if (!hok || ih[1] != c->cfg.nx || ih[2] != c->cfg.ny || ih[3] != c->cfg.nz) {
    std::fclose(f);
    return fail(CFDGB_EINVAL, "%s is not a Plot3D solution of a %dx%dx%d grid", qpath, c->cfg.nx, c->cfg.ny,
                c->cfg.nz);
  }
  if (int rc = ensure_p3d(c)) {
    std::fclose(f);
    return rc;
  }
  const size_t got = std::fread(c->h_p3d, sizeof(float), 5 * n, f);
  std::fclose(f);
  if (got != 5 * n) return fail(CFDGB_EINVAL, "%s is truncated", qpath);
  if (head) {
    head[0] = ih[0];
    for (int a = 0; a < 4; ++a) head[1 + a] = fh[a];
  }
  CK(cudaMemcpyAsync(c->p3d, c->h_p3d, 5 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  double *st[4] = {c->p, c->u, c->v, c->w};
  for (auto *a : st) CK(cudaMemsetAsync(a, 0, c->npad * sizeof(double), c->stream));
  launch_plot3d_unpack(c->stream, c->nblk, c->g, c->p3d, c->p, c->u, c->v, c->w, nullptr);
  TRY(apply_init_bc(c));  // the loaded state starts a run, as cfdgb_init_fields does
  return sync(c);
}

// ---- discrete adjoint -------------------------------------------------------------------

int cfdgb_set_inlet(cfdgb_ctx *c, const double *u_in) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  drop_step_graph(c);  // the ghost fill's inlet pointer is part of a step graph
  if (!u_in) {
    c->inlet = nullptr;
    c->g.uconv = inlet_mean(c, nullptr);
    return 0;
  }
  const size_t n = (size_t)c->cfg.ny * c->cfg.nz;
  if (!c->inlet_buf) TRY(dalloc(c, &c->inlet_buf, n));
  c->inlet = c->inlet_buf;
  c->g.uconv = inlet_mean(c, u_in);  // the convective outflow's velocity
  TRY(h2d(c, c->inlet, u_in, n));
  return sync(c);
}

namespace {

int dd_copy(cfdgb_ctx *c, double *dst, const double *src, size_t n) {
  CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return 0;
}

// Adjoint Poisson solve A y = rhs with the unscaled operator (symmetric on the uniform
// grid), zero start.  FP64 contexts: its own scalars (no restarts: a fresh solver object
// each time), with the context's FP64 V-cycle where it has the multigrid preconditioner.
int adjoint_solve(cfdgb_ctx *c, const double *rhs, double tol, int *iters) {
  if (c->cfg.precision == CFDGB_MIXED) {
    // a MIXED context solves as its forward does (FP32 sweeps in FP64 refinement, its
    // solver and preconditioner), on the forward's b and x: free here, as every step rebuilds
    // b and each recompute window restores x from its checkpoint.  The Jacobi rows take
    // jp * rhs (the same solution).  The answer goes to ka.x, zero start.
    const bool jac = c->cfg.solver == CFDGB_BICGSTAB_JACOBI;
    launch_scale_rows(c->stream, c->g, c->jac64, jac ? 1 : 0, rhs, c->b);
    CK(cudaMemsetAsync(c->x, 0, c->ncell * sizeof(double), c->stream));
    int outer = 0, status = 0;
    double rr = 0.0;
    TRY(solve_mixed(c, tol, iters, &outer, &rr, &status));
    CK(cudaMemcpyAsync(c->ka.x, c->x, c->ncell * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return status;
  }
  CK(cudaMemsetAsync(c->sca, 0, sizeof(SolverScal), c->stream));
  CK(cudaMemsetAsync(c->ka.x, 0, c->ncell * sizeof(double), c->stream));
  TRY(set_solver_params(c, c->sca, tol, c->cfg.maxit));
  // with the multigrid preconditioner the transposed system (the same symmetric operator)
  // gets the FP64 V-cycle; M p, M s in the two history vectors, free during the solve
  const bool mg = c->adj_mg;
  launch_bicg_setup64(c->stream, c->nblk, c->g, c->spe64, c->ka, rhs, c->kapx[0], c->kapx[1], c->part, c->sca,
                      mg ? 1 : 0);
  const PrecVecsT<double> pv{c->ka.x, c->ka.r0, c->ka.r1, c->ka.p1, c->ka.ap, c->ka.s, c->ka.as, c->kapx[0],
                             c->kapx[1], nullptr};
  for (long long q = 0; q < (long long)c->cfg.maxit / 8 + 3; ++q) {
    for (int m = 0; m < 8; ++m) {
      if (mg) {
        for (int part = 0; part < kPrecParts; ++part) {
          L(c, kPrecKid64[part], part == 1 || part == 4 ? mg_vcycle_launches(c->mg64) : 1, [&] {
            if (part == 1) launch_mg_vcycle(c->stream, c->mg64, 0, (const double *)pv.p, pv.ph, c->sca);
            else if (part == 4) launch_mg_vcycle(c->stream, c->mg64, 0, (const double *)pv.s, pv.sh, c->sca);
            else launch_bicgp64_part(c->stream, part == 0 ? 0 : part == 2 ? 1 : part == 3 ? 2 : part == 5 ? 3 : 4,
                                     c->g, c->spe64, pv, c->part, c->sca);
          });
        }
        continue;
      }
      for (int part = 0; part < 5; ++part)
        L(c, K_AP64 + part, 1, [&] { launch_bicg64_part(c->stream, part, c->g, c->spe64, c->ka, c->part, c->sca); });
    }
    CK(cudaMemcpyAsync(c->h_sc, c->sca, sizeof(SolverScal), cudaMemcpyDeviceToHost, c->stream));
    TRY(sync(c));
    if (c->h_sc->done) {
      *iters = c->h_sc->iter;
      return c->h_sc->status;
    }
  }
  return fail(CFDGB_ECUDA, "adjoint solver did not report completion");
}

}  // namespace

int cfdgb_forward(cfdgb_ctx *c, const cfdgb_objective *obj, double *J) {
  if (!c || !obj) return fail(CFDGB_EINVAL, "null argument");
  if (c->cfg.solver == CFDGB_RBSOR)  // the replay and the transposed solve are the Krylov solvers'
    return fail(CFDGB_EINVAL, "the adjoint needs a Krylov-solver context (FP64 or MIXED)");
  if (c->g.nonuni)  // its transposed solve relies on the symmetric uniform-grid operator
    return fail(CFDGB_EINVAL, "the adjoint is implemented on the uniform grid");
  if (c->cfg.scheme != CFDGB_QUICK || c->cfg.les)  // its transposed stencil is QUICK's
    return fail(CFDGB_EINVAL, "the adjoint is implemented for QUICK without the Smagorinsky model");
  if (c->cfg.dt_mode != CFDGB_DT_FIXED)  // its reverse sweep replays the steps at one dt
    return fail(CFDGB_EINVAL, "the adjoint needs a fixed dt (CFDGB_DT_FIXED)");
  if (c->cfg.time_order > 1)  // its transposed step is the Euler step's
    return fail(CFDGB_EINVAL, "the adjoint is implemented for the Euler step (time_order 1)");
  if (c->g.pz || c->g.outflow)  // its transposed ghost fill is the reference's table
    return fail(CFDGB_EINVAL, "the adjoint is implemented for the reference's boundary rows (no periodic z or "
                              "convective outflow)");
  if (obj->nsteps < 1 || obj->first < 1 || obj->last < obj->first || obj->last > obj->nsteps || obj->ckpt_every < 1)
    return fail(CFDGB_EINVAL, "bad objective window");
  if (!c->have_fields || c->loop != 0) return fail(CFDGB_ESTATE, "cfdgb_init_fields must come right before");
  c->obj = *obj;
  c->fwd_done = false;
  const int K = obj->ckpt_every, nck = (obj->nsteps + K - 1) / K;
  // checkpoint q: u, v, w (padded), p (padded; only q = 0: later ones rebuild it from x, which
  // holds p's interior after the step before, the ghosts being the boundary fill's), x
  while ((int)c->ck_f.size() < 5 * nck) {
    const int slot = (int)(c->ck_f.size() % 5), q = (int)(c->ck_f.size() / 5);
    double *d = nullptr;
    if (slot != 3 || q == 0) TRY(dalloc(c, &d, slot == 4 ? c->ncell : c->npad));
    c->ck_f.push_back(d);
  }
  c->ck_sc.assign(nck, SolverScal{});
  c->ck_loop.assign(nck, 0);
  double sum = 0.0;
  for (int n = 1; n <= obj->nsteps; ++n) {
    if ((n - 1) % K == 0) {
      const int q = (n - 1) / K;
      double **f = &c->ck_f[5 * q];
      TRY(dd_copy(c, f[0], c->u, c->npad));
      TRY(dd_copy(c, f[1], c->v, c->npad));
      TRY(dd_copy(c, f[2], c->w, c->npad));
      if (f[3]) TRY(dd_copy(c, f[3], c->p, c->npad));
      TRY(dd_copy(c, f[4], c->x, c->ncell));
      CK(cudaMemcpyAsync(&c->ck_sc[q], c->sc, sizeof(SolverScal), cudaMemcpyDeviceToHost, c->stream));
      c->ck_loop[q] = c->loop;
    }
    cfdgb_step_stats st{};
    const int rc = cfdgb_step(c, 1, &st);
    if (rc < 0 && rc != CFDGB_ENOCONV) return rc;
    if (n >= obj->first && n <= obj->last) sum += st.cd;
  }
  TRY(sync(c));
  c->J = sum / (obj->last - obj->first + 1);
  c->fwd_done = true;
  if (J) *J = c->J;
  return 0;
}

int cfdgb_backward(cfdgb_ctx *c, double *dJ_dinlet, double *dJ_deta) {
  if (!c) return fail(CFDGB_EINVAL, "null context");
  if (!c->fwd_done) return fail(CFDGB_ESTATE, "cfdgb_forward must come first");
  const cfdgb_objective &obj = c->obj;
  const int K = obj.ckpt_every, nck = (obj.nsteps + K - 1) / K;
  const size_t np = c->npad;
  // buffers (allocated once per context, zeroed per call)
  if (!c->leta) {
    for (int a = 0; a < 3; ++a) {
      TRY(dalloc(c, &c->lA[a], np)); TRY(dalloc(c, &c->lB[a], np));
      TRY(dalloc(c, &c->lus[a], np)); TRY(dalloc(c, &c->le[a], np));
    }
    TRY(dalloc(c, &c->leta, np));
    TRY(dalloc(c, &c->lx, c->ncell));
    TRY(dalloc(c, &c->linlet, (size_t)c->cfg.ny * c->cfg.nz));
    TRY(dalloc(c, &c->ka.x, c->ncell));
    if (c->cfg.precision == CFDGB_FP64) {  // the FP64 transposed solve's vectors (MIXED solves as its forward)
      double **kv[] = {&c->ka.r0, &c->ka.r1, &c->ka.p1, &c->ka.s, &c->ka.ap, &c->ka.as, &c->kapx[0], &c->kapx[1]};
      for (auto **q : kv) TRY(dalloc(c, q, c->ncell));
    }
    TRY(dalloc(c, &c->sca, 1));
  }
  while ((int)c->win.size() < 3 * K) {
    double *d = nullptr;
    TRY(dalloc(c, &d, np));
    c->win.push_back(d);
  }
  while ((int)c->winp.size() < K) {
    float *d = nullptr;
    TRY(dalloc(c, &d, np));
    c->winp.push_back(d);
  }
  c->adj_mg = c->use_mg64;  // FP64 multigrid contexts: the transposed solve takes their V-cycle
  for (int a = 0; a < 3; ++a) {
    CK(cudaMemsetAsync(c->lA[a], 0, np * sizeof(double), c->stream));
    CK(cudaMemsetAsync(c->lus[a], 0, np * sizeof(double), c->stream));
    CK(cudaMemsetAsync(c->le[a], 0, np * sizeof(double), c->stream));
  }
  CK(cudaMemsetAsync(c->leta, 0, np * sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->linlet, 0, (size_t)c->cfg.ny * c->cfg.nz * sizeof(double), c->stream));
  const double nu = 1.0 / c->cfg.Re, dt = c->cfg.dt;
  const double cw_in = 2.0 / (c->cfg.lz * dt) / (double)(obj.last - obj.first + 1);
  int worst = 0;
  for (int q = nck - 1; q >= 0; --q) {
    const int n0 = q * K + 1, n1 = std::min(n0 + K - 1, obj.nsteps);
    // restore the checkpoint and recompute the window forward, keeping U^n and p^n
    double **f = &c->ck_f[5 * q];
    TRY(dd_copy(c, c->u, f[0], np));
    TRY(dd_copy(c, c->v, f[1], np));
    TRY(dd_copy(c, c->w, f[2], np));
    TRY(dd_copy(c, c->x, f[4], c->ncell));
    CK(cudaMemcpyAsync(c->sc, &c->ck_sc[q], sizeof(SolverScal), cudaMemcpyHostToDevice, c->stream));
    if (f[3]) {
      TRY(dd_copy(c, c->p, f[3], np));
      launch_bc(c->stream, c->g, c->u, c->v, c->w, nullptr, c->us, c->vs, c->ws, 0);  // T1's copies of T0
    } else {
      // p = its interior from x, then the ghost fill (which rewrites u, v, w's ghosts with the
      // values they hold) and T1's copies
      launch_transform(c->stream, c->nblk, c->g, c->x, c->p);
      launch_bc(c->stream, c->g, c->u, c->v, c->w, c->p, c->us, c->vs, c->ws, 1, c->inlet);
    }
    c->loop = c->ck_loop[q];
    for (int n = n0; n <= n1; ++n) {
      double **wv = &c->win[3 * (n - n0)];
      TRY(dd_copy(c, wv[0], c->u, np));
      TRY(dd_copy(c, wv[1], c->v, np));
      TRY(dd_copy(c, wv[2], c->w, np));
      cfdgb_step_stats st{};
      const int rc = cfdgb_step(c, 1, &st);
      if (rc < 0 && rc != CFDGB_ENOCONV) return rc;
      launch_f64_to_f32(c->stream, (long long)np, c->p, c->winp[n - n0]);
    }
    // reverse sweep over the window (p^n back to FP64 in the context's p, free here)
    for (int n = n1; n >= n0; --n) {
      double **wv = &c->win[3 * (n - n0)];
      launch_f32_to_f64(c->stream, (long long)np, c->winp[n - n0], c->p);
      launch_adj_bc(c->stream, c->g, c->lA[0], c->lA[1], c->lA[2], c->linlet);
      // u* of step n (interior faces), from U^n, by the kernel the forward step ran (MIXED:
      // the FP32 stencil on FP32 copies, which reproduces the forward's u* bit for bit)
      if (fast_convdiff(c)) {
        launch_mirror32(c->stream, c->g, wv[0], wv[1], wv[2], c->u32, c->v32, c->w32);
        launch_convdiff_f32(c->stream, c->nblk, c->g, c->tab32, c->tab32_uni.empty() ? nullptr : c->tab32_uni.data(),
                            dt, nu, wv[0], wv[1], wv[2], c->u32, c->v32, c->w32, c->us, c->vs, c->ws, StepCtl{});
      } else {
        launch_convdiff_exact(c->stream, c->nblk, c->g, CFDGB_QUICK, dt, nu, nullptr, wv[0], wv[1], wv[2], c->us,
                              c->vs, c->ws, StepCtl{});
      }
      const double cw = (n >= obj.first && n <= obj.last) ? cw_in : 0.0;
      launch_adj_corr(c->stream, c->nblk, c->g, dt, cw, c->eta, c->p, c->us, c->vs, c->ws, c->lA[0], c->lA[1],
                      c->lA[2], c->lus[0], c->lus[1], c->lus[2], c->le[0], c->le[1], c->le[2], c->lx, c->leta,
                      c->part, c->ss);
      for (int a = 0; a < 3; ++a) CK(cudaMemsetAsync(c->lB[a], 0, np * sizeof(double), c->stream));
      if (n > 1) {
        // lambda_b = A^+ lambda_x (both sides mean-free)
        launch_remove_mean(c->stream, c->nblk, c->g, c->lx, c->part, c->ss, true);
        int it = 0;
        const int rc = adjoint_solve(c, c->lx, c->cfg.tol, &it);
        if (rc < worst) worst = rc;
        launch_remove_mean(c->stream, c->nblk, c->g, c->ka.x, c->part, c->ss, false);
        launch_adj_rhs(c->stream, c->nblk, c->g, dt, c->ka.x, c->lus[0], c->lus[1], c->lus[2], c->lB[0], c->lB[1],
                       c->lB[2]);
      }
      if (fast_convdiff(c))  // the transpose of the FP32 stencil the forward ran (u32.. hold U^n)
        launch_adj_convdiff_f32(c->stream, c->nblk, c->g, c->tab32,
                                c->tab32_uni.empty() ? nullptr : c->tab32_uni.data(), dt, nu, c->u32, c->v32, c->w32,
                                c->lus[0], c->lus[1], c->lus[2], c->lB[0], c->lB[1], c->lB[2]);
      else
        launch_adj_convdiff(c->stream, c->nblk, c->g, dt, nu, wv[0], wv[1], wv[2], c->lus[0], c->lus[1],
                            c->lus[2], c->lB[0], c->lB[1], c->lB[2]);
      for (int a = 0; a < 3; ++a) std::swap(c->lA[a], c->lB[a]);
    }
  }
  // the ghost fill of the initial state (cfdgb_init_fields) also reads the inlet
  launch_adj_bc(c->stream, c->g, c->lA[0], c->lA[1], c->lA[2], c->linlet);
  CK(cudaGetLastError());
  if (dJ_dinlet) TRY(d2h(c, dJ_dinlet, c->linlet, (size_t)c->cfg.ny * c->cfg.nz));
  if (dJ_deta) TRY(d2h(c, dJ_deta, c->leta, np));
  TRY(sync(c));
  // the fields now hold the first recompute window's end state: stepping on needs a new
  // cfdgb_init_fields (cfdgb_backward may be called again: it restarts from checkpoints)
  c->have_fields = false;
  if (worst < 0) fail(worst, "an adjoint Poisson solve ended with status %d", worst);
  return worst;
}

}  // extern "C"
