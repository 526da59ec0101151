// Kernel launchers shared between the translation units (all enqueue on stream s).
#pragma once

#include <vector>

#include "cfdgb_internal.cuh"

namespace cfdgb {

// step_exact.cu (bit-exact FP64, reference operation order)
// scheme: a cfdgb_scheme value; nut (compact, may be null): eddy viscosity added to nu.
// Fused CFL reduction into sc.ss (none when sc.ss is null); dt from sc.dtp when set.
void launch_convdiff_exact(cudaStream_t s, int nblk, const Geo &g, int scheme, double dt, double nu,
                           const double *nut, const double *u, const double *v, const double *w, double *us,
                           double *vs, double *ws, const StepCtl &sc);
// SmagorinskyModel on u, v, w into compact nut; l2 = (CS delta)^2 per compact row
void launch_smagorinsky(cudaStream_t s, int nblk, const Geo &g, const double *l2, const double *u, const double *v,
                        const double *w, double *nut);
// dtp: dt on the device (null: dt)
void launch_rhs_exact(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, const double *us,
                      const double *vs, const double *ws, int jacobi, const Stencil<double> &st, double *b);
void launch_spmv_exact(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *x,
                       double *y);
void launch_transform(cudaStream_t s, int nblk, const Geo &g, const double *x, double *p);
// get_Cfl on u* into ss->cfl (cfl, U_max[3], U_min[3])
void launch_cfl(cudaStream_t s, int nblk, const Geo &g, double dt, const double *us, const double *vs,
                const double *ws, double *part, StepScal *ss);
// Plot3D solution arrays p, u, v, w, eta (float32, k-j-i order) into out[5 * ncell]
void launch_plot3d_pack(cudaStream_t s, int nblk, const Geo &g, const double *p, const double *u, const double *v,
                        const double *w, const double *eta, float *out);
// QfileRead: in[5 * ncell] (p, u, v, w, eta cell-centred, i fastest, as in a .q file) to
// the interior of padded p, u, v, w (faces) and eta (may be null)
void launch_plot3d_unpack(cudaStream_t s, int nblk, const Geo &g, const float *in, double *p, double *u, double *v,
                          double *w, double *eta);
// dtp: dt on the device (null: dt); step_mode: 0 a single call, 1 a time step (time += dt),
// 2 a time step with an adaptive dt (then dt = dt_next)
void launch_update_uf_exact(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, int step_mode,
                            double lz, const double *eta, const double *p, const double *us, const double *vs,
                            const double *ws, double *u3, double *v3, double *w3, double *f, const double *ui,
                            const double *vi, const double *wi, double *part, StepScal *ss);
// MIXED: the same correction with reciprocal multiplications (not the reference's rounding)
// and the DFIB arithmetic only where eta is non-zero on either side of a face
void launch_update_uf_fast(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, int step_mode,
                           double lz, const double *eta, const double *p, const double *us, const double *vs,
                           const double *ws, double *u3, double *v3, double *w3, const double *ui, const double *vi,
                           const double *wi, double *part, StepScal *ss);
// inlet: nyc*nzc inlet u values (NULL: the reference's constant Dir[0][0] = 1).
// Convective outflow (g.outflow): conv = 1 in a time step (the outlet advances from the
// last step's values in us, vs, ws, with the step's dt in ss->dt_step), 0 at init; the
// flux reduction uses part (nblk blocks at most) and ss.
void launch_bc(cudaStream_t s, const Geo &g, double *u, double *v, double *w, double *p, double *us,
               double *vs, double *ws, int do_main, const double *inlet = nullptr, int conv = 0,
               double *part = nullptr, StepScal *ss = nullptr, int nblk = 1);
void launch_eta(cudaStream_t s, int nblk, const Geo &g, const double *X, const double *Y, double cx, double cy,
                double R, double *eta);

// step_fast.cu (MIXED: FP32 arithmetic on the FP64 state)
// u32, v32, w32: FP32 copies of the padded u, v, w (launch_mirror32), which the stencil
// reads; u, v, w (FP64) give u* = u + increment.  Fused CFL reduction into sc.ss.  tab: the
// per-axis FP32 tables (device); uni: on a uniform grid, the one value of each of their
// rows (host, 3 x 11), which the kernel then takes as parameters; NULL otherwise.
void launch_convdiff_f32(cudaStream_t s, int nblk, const Geo &g, const float *tab, const float *uni, double dt,
                         double nu, const double *u, const double *v, const double *w, const float *u32,
                         const float *v32, const float *w32, double *us, double *vs, double *ws, const StepCtl &sc);
// the adjoint of launch_convdiff_f32 (MIXED contexts): lambda of u*, v*, w* (lus, lvs,
// lws) into lambda of U^n (lu, lv, lw, accumulated), with u32, v32, w32 the FP32 copies of
// U^n the forward's stencil read
void launch_adj_convdiff_f32(cudaStream_t s, int nblk, const Geo &g, const float *tab, const float *uni, double dt,
                             double nu, const float *u32, const float *v32, const float *w32, const double *lus,
                             const double *lvs, const double *lws, double *lu, double *lv, double *lw);
// MIXED: createBMatrix with the reciprocal metrics (multiplications)
void launch_rhs_fast(cudaStream_t s, int nblk, const Geo &g, double dt, const double *dtp, const double *us,
                     const double *vs, const double *ws, int jacobi, const Stencil<double> &st, double *b);
// padded FP32 copies of u, v, w (rounded to nearest)
void launch_mirror32(cudaStream_t s, const Geo &g, const double *u, const double *v, const double *w, float *u32,
                     float *v32, float *w32);

// solver.cu
template <typename T>
struct KrylovVecs {
  T *x, *r0, *r1, *p1, *s, *ap, *as;
  T *xb;  // FP32 BiCGSTAB sweep: the best iterate kept so far (unused elsewhere)
};

// stretched grid: store the SPE (jac 0) or Jacobi-scaled CSR (jac 1) rows into out[7][ncell]
void launch_build_rows(cudaStream_t s, const Geo &g, int jac, double *out);
// out[q] = (float)in[q], q < n (the stored rows for the MIXED sweeps)
void launch_rows_f32(cudaStream_t s, long long n, const double *in, float *out);
// FP64 BiCGSTAB (bicgstabRe2) set-up: r0 = b - A x, r1 = p1 = r0, history px2 <- px1 <- x
void launch_bicg_setup64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st,
                         KrylovVecs<double> v, const double *b, double *px1, double *px2, double *part,
                         SolverScal *sc, int restart = 0);
// FP64 iteration, kernel `part` 0..4 (ap, s, as, xr, p); each a no-op once sc->done is set
void launch_bicg64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                        double *part_buf, SolverScal *sc);
// FP32 iteration, kernel `part` 0..2 (p update + A p, s + A s, x and r1); p and ap are
// double-buffered: p2[sc->par] holds the previous p, p2[sc->par ^ 1] receives the new one
void launch_bicg32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st, KrylovVecs<float> v,
                        float *const p2[2], float *const ap2[2], double *part_buf, SolverScal *sc);
// resident blocks per SM of the pointwise FP32 kernel (sizes Geo::xgrid)
int fp32_pointwise_blocks_per_sm();
// bulk-copy pipeline of the FP32 stencil kernels: rows per block, dynamic shared memory and
// resident blocks per SM of the pap kernel and (smem2, blocks2) of the two-vector kernels;
// returns 0 when the grid does not fit it
int fp32_stage_plan(int nzc, int *tj, int *smem_bytes, int *blocks_per_sm, int *smem2_bytes, int *blocks2_per_sm);
// CG on the SPE operator (inc/solver/cg.hpp): set-up r = b - A x, p = r; FP64 iteration
// kernels 0..2 (q = A p, x and r, p update); FP32 sweep kernels 0..1 (p update + A p,
// x and r), p double-buffered like the BiCGSTAB sweeps, q in ap2[0]
void launch_cg_setup64(cudaStream_t s, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v, const double *b,
                       double *px1, double *px2, double *part, SolverScal *sc);
void launch_cg64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, KrylovVecs<double> v,
                      double *part_buf, SolverScal *sc);
void launch_cg32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st, KrylovVecs<float> v,
                      float *const p2[2], float *const ap2[2], double *part_buf, SolverScal *sc);
// after the loop: NaN/Inf recovery of bicgstabRe2.hpp:133-153 when the cap was hit
void launch_bicg_nan_reset(cudaStream_t s, int nblk, const Geo &g, double *x, const double *px1,
                           const double *px2, double *part, SolverScal *sc);

// MIXED refinement pieces: FP64 residual, stored rounded to FP32 in rf (flags: 1 = also
// ||b||, 2 = also the sweep scale) and the start of an FP32 sweep on it (first: also the
// solve's set-up)
void launch_residual64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, int jacobi, const double *b,
                       const double *x, float *rf, double *part, StepScal *ss, SolverScal *inner, int flags);
void launch_refine_start32(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, KrylovVecs<float> v,
                           float *const p2[2], float *const ap2[2], const float *rf, const StepScal *ss,
                           double delta, double peak, int first, double *part, SolverScal *sc);
void launch_sum32(cudaStream_t s, const Geo &g, const float *e, double *part, StepScal *ss);
// x += factor (e - mean e), the mean taken from the preceding launch_sum32; factor = +-2^k
// (sweep_scale)
void launch_correct64(cudaStream_t s, int nblk, const Geo &g, double *x, const float *e, double factor,
                      const StepScal *ss);

// adjoint.cu (discrete adjoint of the FP64 step)
void launch_adj_bc(cudaStream_t s, const Geo &g, double *lu, double *lv, double *lw, double *linlet);
void launch_adj_corr(cudaStream_t s, int nblk, const Geo &g, double dt, double cw, const double *eta, const double *p,
                     const double *us, const double *vs, const double *ws, const double *lu, const double *lv,
                     const double *lw, double *lus, double *lvs, double *lws, double *lex, double *ley, double *lez,
                     double *lx, double *leta, double *part, StepScal *ss);
// y -= mean(y); sum_known: the previous kernel left sum(y) in ss->fsum[0]
void launch_remove_mean(cudaStream_t s, int nblk, const Geo &g, double *y, double *part, StepScal *ss, bool sum_known);
// padded field conversions of the adjoint's window storage
void launch_f64_to_f32(cudaStream_t s, long long n, const double *a, float *b);
void launch_f32_to_f64(cudaStream_t s, long long n, const float *a, double *b);
void launch_adj_rhs(cudaStream_t s, int nblk, const Geo &g, double dt, const double *lb, double *lus, double *lvs,
                    double *lws, double *lu, double *lv, double *lw);
void launch_adj_convdiff(cudaStream_t s, int nblk, const Geo &g, double dt, double nu, const double *u, const double *v,
                         const double *w, const double *lus, const double *lvs, const double *lws, double *lu,
                         double *lv, double *lw);

// out = jp * in for the Jacobi-scaled rows, in otherwise (a right-hand side in the rows of
// the context's solver)
void launch_scale_rows(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, const double *in,
                       double *out);
// b -= its null-space part (mean of the unscaled rhs; jp-weighted for the Jacobi rows)
void launch_project_rhs(cudaStream_t s, const Geo &g, const Stencil<double> &st, int jacobi, double *b, double *part,
                        StepScal *ss);

// ---- multigrid.cu: geometric multigrid V-cycle, the preconditioner of the FP32 sweep ----
// Level 0 is the Poisson grid; each coarser level halves every even extent (cell-centred
// agglomeration of two cells per halved axis) until at most kMgCoarseCells cells remain
// or no extent is even.  Operator on every level: the unscaled 7-point Neumann Laplacian
// of that level's spacing (1/h^2 per axis), the uniform-grid SPE rows rediscretised;
// periodic in z on every level when the grid is (the z ends coupled, nz even on each).
constexpr int kMgMaxLevels = 16;
constexpr int kMgCoarseCells = 64;      // coarsening stops at or below this many cells
constexpr int kMgSharedCells = 4096;    // largest coarsest level solved in one block
constexpr int kMgDenseCells = 256;      // largest coarsest level solved by its dense pseudo-inverse
template <typename T>
struct MgLevelT {
  int nx, ny, nz;          // cells
  T wx, wy, wz;            // 1/h^2 per axis
  int fx, fy, fz;          // cells of this level per cell of the next one, per axis (1, 2)
  T *x, *b;                // correction and right-hand side (levels >= 1)
  int bx, by, gx, gy, gz;  // launch geometry: bx along k, by along j, gz planes strided over i
  int qgrid;               // 1: the quad smoother (FP32, nz % 4 == 0), 0: the scalar one
  int qbx, qby, qgx, qgy, qgz;  // its launch: quads along x, rows along y, planes strided over z
  int pz;                  // periodic z (every level; nz even or 1 on each)
  // 1: the level's V-cycle work runs as two marching kernels (k_mg_down4, k_mg_up4; FP32
  // quads, every axis halves, nz / 4 a power of two up to 16): a block of nz / 4 x (mty + 4)
  // threads owns a band of mty rows and marches over a segment of msx planes; mgx x mgy blocks
  int march, mty, msx, mgx, mgy;
  // division of a cell index by nz, ny and nz / 2 (the one-block kernels' cell loops): the
  // multiplier and shift of a division by an invariant integer (div_magic in multigrid.cu)
  unsigned dz_m, dy_m, dh_m;
  int dz_l, dy_l, dh_l;
  // 1/diag of a row by its neighbour counts along x, y, z (each 0..2): idg[9 cx + 3 cy + cz]
  // (0 where a row has no neighbour); the smoother multiplies instead of dividing
  T idg[27];
};
template <typename T>
struct MgPlanT {
  int nlev;
  int coarse_sweeps;  // red-black sweeps of the coarsest solve
  int tail;           // levels tail..nlev-1 run in one block's shared memory (tail >= 1); nlev: none
  const T *cinv;      // the coarsest level's dense pseudo-inverse (device), or null: red-black sweeps
  MgLevelT<T> lev[kMgMaxLevels];
};
using MgLevel = MgLevelT<float>;
using MgPlan = MgPlanT<float>;
// levels of an nx x ny x nz grid with spacing hx, hy, hz (arrays left null); false when
// the grid has a single level too large for the one-block coarsest solve, or (pz: periodic
// z on every level) a level with an odd nz above 1.  T: the element type of the hierarchy
// (float: the MIXED sweeps' preconditioner; double: FP64's)
template <typename T>
bool mg_plan(int nx, int ny, int nz, double hx, double hy, double hz, int nsm, bool quads, MgPlanT<T> *mg,
             bool pz = false);
// kernels one V-cycle launches
template <typename T>
int mg_vcycle_launches(const MgPlanT<T> &mg);
// the pseudo-inverse of the coarsest level's operator, row-major, when that level has at
// most kMgDenseCells cells (the caller uploads it and sets mg.cinv)
template <typename T>
bool mg_dense_inverse(const MgPlanT<T> &mg, std::vector<T> &M);
// kernel attributes the hierarchy needs (shared memory of the one-block kernels); once,
// before the first V-cycle
template <typename T>
void mg_prepare();
// x0 = M b0, one V(1,1) cycle: red-black Gauss-Seidel smoothing from a zero start,
// averaging restriction, cell-centred trilinear prolongation, a one-block red-black solve
// on the coarsest level.  jacobi: b0 holds Jacobi-scaled rows (jp = 1/diag), so M applies
// to diag * b0.  Every kernel returns at once when sc->done is set.
template <typename T>
void launch_mg_vcycle(cudaStream_t s, const MgPlanT<T> &mg, int jacobi, const T *b0, T *x0, const SolverScal *sc);

// FP32 BiCGSTAB with a right preconditioner M (the V-cycle), kernel `part` 0..4:
// 0 p = r1 + beta (p - omega v) (or r1 on restart, r0 = r1); 1 v = A ph, alpha;
// 2 s = r1 - alpha v; 3 t = A sh, omega; 4 x += alpha ph + omega sh, r1 = s - omega t,
// stop test and beta.  ph = M p and sh = M s come from the V-cycles between them.
template <typename T>
struct PrecVecsT {
  T *x, *r0, *r1, *p, *v, *s, *t, *ph, *sh, *xb;
};
using PrecVecs = PrecVecsT<float>;
void launch_bicgp32_part(cudaStream_t s, int part, const Geo &g, const Stencil<float> &st, PrecVecs v,
                         double *part_buf, SolverScal *sc);
// The FP64 iteration with the FP64 V-cycle as right preconditioner (the same five kernels
// and order; xb unused): the like-for-like FP64 counterpart of the MIXED multigrid sweep.
// It stops on the tolerance or the cap and restarts only on a Lanczos breakdown.
void launch_bicgp64_part(cudaStream_t s, int part, const Geo &g, const Stencil<double> &st, PrecVecsT<double> v,
                         double *part_buf, SolverScal *sc);

// red-black SOR on the same operator (FP64)
void launch_rbsor_sweep(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *b,
                        double *x, double omega);
void launch_residual_norm64(cudaStream_t s, int nblk, const Geo &g, const Stencil<double> &st, const double *b,
                            const double *x, double *part, StepScal *ss);
void launch_vec_norm64(cudaStream_t s, int nblk, const Geo &g, const double *b, double *part, StepScal *ss);

}  // namespace cfdgb
