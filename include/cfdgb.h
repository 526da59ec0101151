/* cfdgb -- GB300-native (sm_103a) projection time step for incompressible flow past a
 * circular cylinder on a staggered MAC grid: convection-diffusion (QUICK by default),
 * direct-forcing immersed boundary (DFIB), pressure Poisson solve and velocity correction.
 *
 * Drop-in for the projection step of jimmy3769tw/CFD_NSsolver_forHPC_flowPassingCylinder.
 * Each entry point names the reference interface it replaces (paths relative to that
 * project's root).  Field arrays use the reference's padded layout: doubles of
 * (nx+4)*(ny+4)*(nz+4), index i*(ny+4)*(nz+4) + j*(nz+4) + k, two ghost layers per side,
 * u stored at face i+1/2, v at j+1/2, w at k+1/2 (inc/grid/structureGrid.hpp:154).
 * Poisson vectors are compact interior arrays, index (i-2)*ny*nz + (j-2)*nz + (k-2)
 * (structureGrid.hpp:178).
 *
 * Every function returns an int status (cfdgb_status).  Calls on one context are not
 * thread-safe; each context owns one CUDA stream on the current device.  Host pointers
 * are caller-owned and only read or written during the call. */
#ifndef CFDGB_H
#define CFDGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CFDGB_ABI_VERSION 9

typedef enum cfdgb_status {
  CFDGB_OK = 0,
  CFDGB_EINVAL = -1,     /* bad argument or configuration */
  CFDGB_ECUDA = -2,      /* CUDA runtime error (message via cfdgb_last_error) */
  CFDGB_ENOCONV = -3,    /* Poisson solver hit its iteration cap (solution still written,
                            as the reference does: bicgstabRe2.hpp:133-153) */
  CFDGB_ENAN = -4,       /* NaN/Inf detected in the solution or the drag */
  CFDGB_ENOMEM = -5,     /* device allocation failed */
  CFDGB_ESTATE = -6      /* call out of order (e.g. step before fields exist) */
} cfdgb_status;

typedef enum cfdgb_solver {
  CFDGB_BICGSTAB = 0,        /* SPE operator, unscaled (P_SOLVER_BICG_SPE, the default) */
  CFDGB_BICGSTAB_JACOBI = 1, /* rows and rhs scaled by 1/diag (P_SOLVER_BICG_CSR) */
  CFDGB_RBSOR = 2,           /* red-black SOR on the same Neumann operator */
  CFDGB_CG = 3               /* conjugate gradients on the SPE operator (inc/solver/cg.hpp,
                                P_SOLVER_CG_ELL; the operator is symmetric on a uniform grid) */
} cfdgb_solver;

typedef enum cfdgb_precision {
  CFDGB_FP64 = 0,  /* every kernel in FP64 */
  CFDGB_MIXED = 1  /* FP32 stencil sweep and FP32 BiCGSTAB sweeps inside FP64 iterative
                      refinement (defect correction): each sweep starts from the FP64
                      residual and runs until its own residual has dropped by inner_tol;
                      its correction is added to the FP64 solution and the residual is
                      recomputed in FP64.  FP64 outer residual, global dots and
                      divergence check */
} cfdgb_precision;

typedef enum cfdgb_grid {
  CFDGB_GRID_UNIFORM = 0,  /* init_uniform (inc/grid/structureGrid.hpp:336) */
  CFDGB_GRID_SML = 1       /* the reference's default stretched grid, "non_uniform-SML"
                              (structureGrid.hpp:250-329): 100 fine cells over 30 % of x
                              (shifted 4 cells upstream) and of y, coarse cells outside, z
                              uniform; the BiCGSTAB solvers, FP64 or MIXED (the FP32 sweeps
                              on its stored rows rounded to FP32); nx even > 108, ny even > 100 */
} cfdgb_grid;

/* The y-wall rows of the reference's boundary table (inc/BoundaryCondition/FLOWpassing.hpp). */
typedef enum cfdgb_walls {
  CFDGB_WALLS_ZERO_GRADIENT = 0,  /* the active rows (:23-29): u, v, w zero-gradient (default) */
  CFDGB_WALLS_FREE_SLIP = 1       /* the rows left commented out there (:14-21): v = 0 on the
                                     walls, u and w zero-gradient */
} cfdgb_walls;

/* The z faces.  The reference has only its zero-gradient rows (FLOWpassing.hpp:30-39); its
   periodic Poisson terms (inc/matrix/PressureMatrix.hpp:83-101) are unused. */
typedef enum cfdgb_bc_z {
  CFDGB_Z_ZERO_GRADIENT = 0,  /* the reference's rows (default) */
  CFDGB_Z_PERIODIC = 1        /* periodic in z (not in the reference): the ghost layers wrap over
                                 the whole padded (i, j) plane, w has nz unknown faces (face 0 is
                                 the image of the top face), every Poisson row keeps both z terms
                                 and rows k = 0 and nz-1 couple.  No multigrid preconditioner;
                                 RBSOR needs nz even; no adjoint */
} cfdgb_bc_z;

/* The x+ (outlet) face. */
typedef enum cfdgb_outflow {
  CFDGB_OUTFLOW_ZERO_GRADIENT = 0,  /* the reference's row (FLOWpassing.hpp:23-29), default */
  CFDGB_OUTFLOW_CONVECTIVE = 1      /* convective outflow (not in the reference): d(phi)/dt +
                                       Uc d(phi)/dx = 0 for the outlet u face and the v, w ghost
                                       cells beyond it, implicit upwind in time, Uc the area-
                                       weighted mean inlet u; then a uniform correction of the
                                       outlet u that makes the net flux through the domain's
                                       boundary zero, so the Neumann Poisson problem is
                                       consistent.  At init the outlet starts from the
                                       zero-gradient values (corrected).  No adjoint */
} cfdgb_outflow;

/* The reference's compile-time convection switch (inc/0_General.hpp:114-118). */
typedef enum cfdgb_scheme {
  CFDGB_QUICK = 0,  /* QuickUnitA/B (Convection_Difussion.hpp:20-90), the default */
  CFDGB_LUD = 1,    /* linear upwind, LudUnitA/B (:96-147) */
  CFDGB_UD = 2      /* first-order upwind, UdUnit (:150-168) */
} cfdgb_scheme;

/* Preconditioner of the BiCGSTAB solvers (the reference has none: its bicgstabRe2 is
   unpreconditioned, and so is CFDGB_PRECOND_NONE here). */
typedef enum cfdgb_precond {
  CFDGB_PRECOND_NONE = 0,      /* the plain sweep (default) */
  CFDGB_PRECOND_MULTIGRID = 1  /* one geometric multigrid V-cycle per application (right
                                  preconditioning): red-black Gauss-Seidel smoothing, cell-
                                  centred transfers, the uniform-grid Laplacian rediscretised
                                  per level.  MIXED: an FP32 V-cycle in the FP32 sweeps; FP64:
                                  the same V-cycle in FP64 in an FP64 BiCGSTAB that stops on the
                                  tolerance or the cap and restarts only on breakdown (not the
                                  reference's iteration).  BICGSTAB or BICGSTAB_JACOBI, uniform
                                  grid; the grid must coarsen (by halving its even extents) to
                                  at most 4096 cells */
} cfdgb_precond;

/* How dt changes from step to step.  The reference keeps dt fixed: its adaptive
   timestepper (inc/0_1_SimulationVariable.hpp:172-185) is commented out at
   src/RUN_CPU.cpp:275.  Both adaptive rules run on the device, in the reduction that the
   convection-diffusion kernel makes over u* for the CFL number; the new dt takes effect
   at the next step (finishloop, 0_1_SimulationVariable.hpp:139-155). */
typedef enum cfdgb_dt_mode {
  CFDGB_DT_FIXED = 0,      /* dt as set by cfdgb_config.dt and cfdgb_set_dt (default) */
  CFDGB_DT_REFERENCE = 1,  /* timestepper as written: dt_next = the least of 0.05 / (Re U_max^2)
                              and 0.15 * 0.5 * Re U_min^2 over the three components, at least
                              1e-12, with U_max, U_min the extremes of u*, v*, w* since init
                              (get_Cfl keeps them from step to step, cfl.hpp:12-13).  A component
                              whose minimum is zero, such as w in a flow without z motion, drives
                              dt to that 1e-12 floor */
  CFDGB_DT_CFL = 2         /* dt_next = cfl_target / max over cells of (u/Dxs + v/Dys + w/Dzs),
                              the get_Cfl number divided by dt, and at most dt_max */
} cfdgb_dt_mode;

typedef struct cfdgb_config {
  int nx, ny, nz;            /* interior cells (nxCal, nyCal, nzCal) */
  double lx, ly, lz;         /* domain [0,lx]x[0,ly]x[0,lz]; spacing per cfdgb_config.grid */
  double cx, cy, radius;     /* cylinder axis along z (DFIB_CylinderZ, setEta.hpp:136) */
  double Re, dt;             /* nu = 1/Re (0_1_SimulationVariable.hpp:26) */
  int solver;                /* cfdgb_solver */
  int precision;             /* cfdgb_precision */
  double tol;                /* relative residual ||b-Ax||/||b|| (p_criteria) */
  int maxit;                 /* iteration cap per solve (5000: bicgstabRe2.hpp:47); MIXED caps
                                its FP32 iterations over all sweeps at maxit, and an FP64
                                finish, when one runs, at maxit again */
  double omega;              /* SOR relaxation; 0: the optimal one for the grid, 2 / (1 + sqrt(1 -
                                mu^2)) with mu the Jacobi iteration's spectral radius on the
                                non-constant modes of the uniform-grid operator */
  double inner_tol;          /* MIXED: residual reduction of each FP32 sweep; 0 (default):
                                0.3 for the BiCGSTAB solvers, 3e-4 for CG */
  int max_outer;             /* MIXED: cap on FP64 refinements per solve */
  int check_every;           /* SOR: residual checked every this many sweeps */
  int dfib;                  /* 1: cylinder solid fraction on; 0: no immersed body */
  uint64_t seed;             /* perturbation seed (splitmix64), used when amp != 0 */
  double amp;                /* uniform(-amp, amp) added to interior u, v, w at init */
  int project_rhs;           /* 1: remove the Poisson right-hand side's null-space part (its
                                mean; jp-weighted for the Jacobi rows) before each solve, which
                                makes the Neumann problem consistent for any inflow; 0: the
                                reference, which solves b as it is (default) */
  int grid;                  /* a cfdgb_grid value; default uniform */
  int scheme;                /* a cfdgb_scheme value; default QUICK.  MIXED precision runs its
                                FP32 stencil sweep for QUICK only; the other schemes use the
                                FP64 kernel there */
  int les;                   /* 1: Smagorinsky eddy viscosity (TERBULENCE_SMAGORINSKY,
                                inc/source/SmagorinskyModel.hpp:30, CS = 0.18) added to nu,
                                from T0 before each convection-diffusion; 0: off (default) */
  int walls;                 /* a cfdgb_walls value; default zero-gradient */
  int precond;               /* a cfdgb_precond value: the preconditioner of the MIXED
                                BiCGSTAB sweeps; default none (the reference's iteration) */
  int dt_mode;               /* a cfdgb_dt_mode value; default fixed */
  double cfl_target;         /* CFDGB_DT_CFL: the CFL number each step aims at (default 0.5) */
  double dt_max;             /* CFDGB_DT_CFL: upper bound of dt (default: cfdgb_config.dt) */
  int time_order;            /* time stepping of u*: 1 the reference's explicit Euler step
                                (default); 2 Adams-Bashforth, variable step; 3 Adams-Bashforth,
                                constant step (CFDGB_DT_FIXED).  Not a drop-in: the reference's
                                2nd/3rd-order branch (inc/source/sourceTerm.hpp:9-108) does not
                                compile, and as written it would overwrite the stored increment
                                before reading it.  The order builds up from 1 over the first
                                steps after init (cfdgb_set_dt restarts order 3); MIXED then
                                uses the FP64 convection-diffusion kernel; no adjoint */
  int bc_z;                  /* a cfdgb_bc_z value; default zero-gradient */
  int outflow;               /* a cfdgb_outflow value; default zero-gradient */
} cfdgb_config;

typedef struct cfdgb_step_stats {
  int step;          /* 1-based step number (simu.loop) */
  int iters;         /* Poisson iterations (inner iterations summed for MIXED) */
  int outer;         /* MIXED: FP64 refinements (true-residual updates); 0 otherwise */
  int status;        /* cfdgb_status of this step's solve */
  double relres;     /* final relative residual of the solve (FP64) */
  double cd, cl;     /* drag and lift coefficients (CD_CL, virtualForceIntergrator.hpp:92) */
  double cfl;        /* CFL number of u* (get_Cfl, inc/analyses/cfl.hpp:3, src/RUN_CPU.cpp:274) */
  double dt;         /* dt of this step */
  double time;       /* simulated time at the end of this step (simu.time after finishloop) */
} cfdgb_step_stats;

/* Library identity and last error text (thread-local). */
int cfdgb_abi_version(void);
const char *cfdgb_last_error(void);

/* Defaults: the reference's config-1 case (96x48x4, [0,24]x[0,12]x[0,1], cylinder at
 * (6,6), Re 100, dt 0.005, SPE BiCGSTAB, tol 1e-8, 5000 iterations). */
int cfdgb_config_default(cfdgb_config *cfg);

/* Context: grid, metrics, operator, solid fraction and all device buffers.  Replaces the
 * set-up half of runSeqOmp (src/RUN_CPU.cpp:9-255): resize_variable, generateGride
 * (uniform), SPE_matrix::setupPressure / createPressureMatrixCSR, DFIB_CylinderZ. */
typedef struct cfdgb_ctx cfdgb_ctx;
int cfdgb_create(const cfdgb_config *cfg, cfdgb_ctx **out);
int cfdgb_destroy(cfdgb_ctx *ctx);
int cfdgb_padded_dims(const cfdgb_ctx *ctx, int *nxp, int *nyp, int *nzp);
/* cudaStream_t of the context, as void* (for events / interop). */
int cfdgb_stream(const cfdgb_ctx *ctx, void **stream);

/* Initial condition (src/RUN_CPU.cpp:66-109): u,v,w,p become T0 (and the T1/T3 copies),
 * then BC_staggered_main and BC_staggered_copy run and the step counter restarts at 1
 * (so the next step, like loop 1, has no pressure solve).  NULL fields select the
 * reference's iniU(1,0,0) / p=0, plus the configured perturbation. */
int cfdgb_init_fields(cfdgb_ctx *ctx, const double *u, const double *v, const double *w,
                      const double *p);
/* Overwrite the current state (T0 and p after a step) without restarting the run. */
int cfdgb_set_fields(cfdgb_ctx *ctx, const double *u, const double *v, const double *w,
                     const double *p);
/* Copy the current state out; NULL skips a field. */
int cfdgb_get_fields(cfdgb_ctx *ctx, double *u, double *v, double *w, double *p);
int cfdgb_get_eta(cfdgb_ctx *ctx, double *eta);
int cfdgb_set_eta(cfdgb_ctx *ctx, const double *eta);

/* nsteps projection steps (the loop body src/RUN_CPU.cpp:257-436).  stats: NULL or
 * nsteps entries.  Returns the worst status over the steps. */
int cfdgb_step(cfdgb_ctx *ctx, int nsteps, cfdgb_step_stats *stats);

/* ---- discrete adjoint (no reference counterpart: the reference has no gradients) ----
 * Objective J: drag coefficient averaged over steps first..last of an nsteps run that
 * starts from the state cfdgb_init_fields set.  cfdgb_forward runs it (a Krylov solver,
 * FP64 or MIXED, fixed dt, the Euler step, QUICK without the Smagorinsky model, uniform
 * grid), keeping a checkpoint every ckpt_every steps, and returns J.  cfdgb_backward sweeps
 * the steps in reverse, recomputing each checkpoint window forward first (in the context's
 * precision), and returns dJ/d(inlet u profile) (ny*nz values, the inlet ghost value of
 * BC_staggered_main's face 0 per (j,k)) and dJ/d(solid fraction eta) (padded field).  The
 * transposed Poisson solve (the operator is symmetric on the uniform grid) is the
 * context's own: FP64 BiCGSTAB (preconditioned by the FP64 V-cycle when the context has
 * the multigrid preconditioner), or for a MIXED context the same FP32 sweeps in FP64
 * refinement as its forward solves, to the same FP64 tolerance.  Memory beyond the
 * forward's: per checkpoint u, v, w (padded FP64) and the solver's warm start (compact; p
 * is rebuilt from it), plus p for the first; per window step u, v, w (padded FP64) and p
 * (padded FP32); about 14 padded FP64 fields of adjoint state, and 1 compact one (MIXED)
 * or 9 (FP64). */
typedef struct cfdgb_objective {
  int nsteps;      /* forward steps */
  int first, last; /* drag averaged over these steps (1-based, inclusive) */
  int ckpt_every;  /* checkpoint interval K */
} cfdgb_objective;
/* Inlet u per (j,k) of the inlet face (ny*nz, k fastest), replacing the reference's
 * constant Dir[0][0] = 1 (FLOWpassing.hpp:6); NULL restores the constant. */
int cfdgb_set_inlet(cfdgb_ctx *ctx, const double *u_in);
int cfdgb_forward(cfdgb_ctx *ctx, const cfdgb_objective *obj, double *J);
int cfdgb_backward(cfdgb_ctx *ctx, double *dJ_dinlet, double *dJ_deta);

/* ---- allocation-free Poisson solve (no counterpart in the reference) ----
 * The BiCGSTAB solve of cfdgb_op_bicgstab (SPE operator, or the Jacobi-scaled rows for
 * CFDGB_BICGSTAB_JACOBI) for callers that cannot allocate device memory: hosts whose
 * framework owns all device memory through its own pool, and services that must not
 * allocate after start-up.  Grid: nx*ny*nz interior cells with uniform spacing dx, dy, dz.
 * d_rhs and d_x (warm start in, solution out) are the caller's DEVICE arrays of nx*ny*nz
 * doubles; the work is enqueued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and the call returns after it finished.  No cudaMalloc/cudaFree or allocating
 * library call is made: all work vectors live in a static device array reserved on every
 * GPU that loads the library (17,039,616 bytes, about 17.0 MB: 8 vectors of 2 MiB, block
 * partials and scalars) and shared by all calls, so at most 2^18 = 262,144 unknowns (larger
 * grids: CFDGB_EINVAL), and calls whose work overlaps on the GPU race.  The call polls the
 * solver's convergence from the host, waiting on `stream` every 8 iterations, so a stream
 * that is capturing into a CUDA graph is rejected (CFDGB_EINVAL).  The first call on a
 * device looks up the array's device address. */
int cfdgb_poisson_solve_static(int nx, int ny, int nz, double dx, double dy, double dz, int solver, double tol,
                               int maxit, const double *d_rhs, double *d_x, void *stream, int *iters,
                               double *relres);

/* ---- instrumentation (no reference counterpart: the reference times phases with
 * std::chrono stopwatches, inc/profiling/STL_clock.hpp:8) ---- */
/* Kernel timing: while enabled, every kernel the step driver launches is bracketed by a
 * CUDA-event pair on the context's stream (the solver's iteration graphs are replaced by
 * direct launches of the same kernels). */
int cfdgb_set_kernel_timing(cfdgb_ctx *ctx, int enable);
int cfdgb_reset_counters(cfdgb_ctx *ctx);
/* Kernels launched by the step driver since the last reset (graph nodes counted). */
int cfdgb_launch_count(const cfdgb_ctx *ctx, long long *launches);
/* idx in [0, n): kernel name, summed device milliseconds (timing on), launches; returns
 * CFDGB_EINVAL past the last kernel. */
int cfdgb_kernel_stat(cfdgb_ctx *ctx, int idx, const char **name, double *total_ms, long long *launches);

/* ---- per-function entry points on host buffers (one kernel each; for drop-in use of a
 * single reference function and for parity tests) ---- */

/* ConvectionDifussion (inc/source/Convection_Difussion.hpp:174) with the context's scheme
 * (and, les = 1, the eddy viscosity of u,v,w as the step computes it): reads u,v,w, writes
 * the interior faces of us,vs,ws (other entries of us,vs,ws are left as passed in). */
int cfdgb_op_convection_diffusion(cfdgb_ctx *ctx, const double *u, const double *v,
                                  const double *w, double *us, double *vs, double *ws);
/* SmagorinskyModel (inc/source/SmagorinskyModel.hpp:30): the eddy viscosity (Viseff) of
 * padded u,v,w, into the compact array nut (nx*ny*nz). */
int cfdgb_op_smagorinsky(cfdgb_ctx *ctx, const double *u, const double *v, const double *w,
                         double *nut);
/* BC_staggered_main (inc/BoundaryCondition/Boundary_Condition.hpp:37), in place. */
int cfdgb_op_bc_main(cfdgb_ctx *ctx, double *u, double *v, double *w, double *p);
/* BC_staggered_copy (inc/BoundaryCondition/updateBC.hpp:6): ghosts of u,v,w into us,vs,ws. */
int cfdgb_op_bc_copy(cfdgb_ctx *ctx, const double *u, const double *v, const double *w,
                     double *us, double *vs, double *ws);
/* createBMatrix_omp (inc/matrix/b_matrix.hpp:35): b (compact) from u*; jacobi != 0
 * scales by jp = 1/diag as the CSR path does. */
int cfdgb_op_rhs(cfdgb_ctx *ctx, int jacobi, const double *us, const double *vs,
                 const double *ws, double *b);
/* SPE_matrix::multiply_omp (inc/matrix/SPE_sparseMatrix.hpp:92) or, jacobi != 0, the
 * scaled CSR_matrix::multiply_omp (inc/matrix/CSR_sparseMatrix.hpp:232); compact x, y. */
int cfdgb_op_spmv(cfdgb_ctx *ctx, int jacobi, const double *x, double *y);
/* bicgstabRe2::solve (inc/solver/bicgstabRe2.hpp:84) on compact rhs, x (x in: warm
 * start, out: solution).  solver: CFDGB_BICGSTAB or CFDGB_BICGSTAB_JACOBI (rhs must then
 * already be scaled, as createBMatrix_omp does). */
int cfdgb_op_bicgstab(cfdgb_ctx *ctx, int solver, double tol, int maxit, const double *rhs,
                      double *x, int *iters, double *relres);
/* update_UandF_omp (inc/dfib/updateUandF.hpp:90): u3,v3,w3 interior faces from u*, p,
 * eta; f (3*padded, may be NULL) gets the DFIB force; cd/cl (may be NULL) its CD_CL. */
int cfdgb_op_update_uf(cfdgb_ctx *ctx, const double *eta, const double *p, const double *us,
                       const double *vs, const double *ws, double *u3, double *v3,
                       double *w3, double *f, double *cd, double *cl);
/* DFIB_CylinderZ (inc/dfib/setEta.hpp:136): solid fraction of the context's cylinder. */
int cfdgb_op_solid_fraction(cfdgb_ctx *ctx, double *eta);
/* get_Cfl (inc/analyses/cfl.hpp:3) on padded u*, v*, w*: out7 = {cfl (max over cells of
 * u/Dxs + v/Dys + w/Dzs, times dt), U_max[3], U_min[3]}. */
int cfdgb_op_cfl(cfdgb_ctx *ctx, const double *us, const double *vs, const double *ws, double *out7);

/* ---- time step and output ---- */
/* New dt for the following steps (simu.dt).  With an adaptive cfdgb_dt_mode the next
 * step's own rule takes over again after that step. */
int cfdgb_set_dt(cfdgb_ctx *ctx, double dt);
/* Plot3D files of the current state, byte-compatible with the reference's writers:
 * xpath (may be NULL) the grid file of OutputPlot3D_Xfile (inc/io/Plot3D/xfileWrite.hpp:6),
 * qpath (may be NULL) the solution file of OutputPLOT3D_Qfile (inc/io/Plot3D/qfile.hpp:6):
 * header (1 block, nx, ny, nz; mach 0, alpha 0, Re, time) and float32 p, cell-centred
 * u, v, w and eta in k-j-i order.  The arrays are packed on the GPU and copied out once. */
int cfdgb_write_plot3d(cfdgb_ctx *ctx, const char *xpath, const char *qpath, double time);
/* QfileRead (inc/io/Plot3D/qfileRead.hpp:6) and the restart it feeds (src/RUN_CPU.cpp:88-99,
 * commented out in the reference): the solution file at qpath, which must be of this
 * context's grid, becomes the state as cfdgb_init_fields would set it from p, u, v, w.  Faces
 * get the float sum of the two cell-centred values beside them, halved; the last face of
 * each axis its cell's value.  The context's eta is kept.  head (5 doubles, may be NULL):
 * blocks, mach, alpha, Re, time of the file's header. */
int cfdgb_read_plot3d(cfdgb_ctx *ctx, const char *qpath, double *head);
/* QfileRead's arrays alone: q holds the 5 * nx*ny*nz float32 values of a .q file after its
 * header; p, u, v, w, eta get the padded fields it returns (zero outside the interior). */
int cfdgb_op_plot3d_read(cfdgb_ctx *ctx, const float *q, double *p, double *u, double *v,
                         double *w, double *eta);
/* Pressure solve on the current u* of the context (createBMatrix + solve +
 * Pressure_transform_X_result, src/RUN_CPU.cpp:310-320) with the configured solver. */
int cfdgb_pressure_solve(cfdgb_ctx *ctx, int *iters, double *relres);

/* ---- self-check ---- */
/* The step kernels divide by a metric or dt through its reciprocal (Markstein's FMA
 * correction, correctly rounded like IEEE division): once for a divisor b whose reciprocal
 * y = RN(1/b) satisfies |b y - 1| < 2^-54 (then Markstein's theorem covers every dividend),
 * twice in a context where some divisor does not.  On the current GPU: n seeded dividends
 * (random sign, significand and exponent in [2^-40, 2^40], a tenth of them exact multiples
 * of b, and zeros) divided by b both ways, with the form a context whose only divisor is b
 * would use; *mismatches counts results whose bits differ. */
int cfdgb_check_division(long long n, uint64_t seed, double b, unsigned long long *mismatches);

#ifdef __cplusplus
}
#endif
#endif
