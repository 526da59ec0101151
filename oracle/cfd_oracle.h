/* CPU restatement of the reference projection step (jimmy3769tw/CFD_NSsolver_forHPC_
 * flowPassingCylinder) in plain C.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and bench.py's CPU-baseline leg call it as the checker; the shipped
 * library never links it.
 *
 * Parity is pinned: with -ffp-contract=off it reproduces, bit for bit, the reference's
 * own functions compiled from its sources by oracle/build_ref.py (one OpenMP thread),
 * on the golden vectors under tests/golden/.
 *
 * Layout is the reference's: padded arrays of (nxc+4)(nyc+4)(nzc+4) doubles,
 * icel = i*ny*nz + j*nz + k (inc/grid/structureGrid.hpp:154), interior i in [2, nx-2);
 * compact Poisson vectors use icelCal = (i-2)*nyc*nzc + (j-2)*nzc + (k-2) (:178). */
#ifndef CFD_ORACLE_H
#define CFD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct og_grid {
  int nxc, nyc, nzc; /* interior cells */
  int nx, ny, nz;    /* padded sizes, nxc + 4 */
  double lx, ly, lz, cx, cy, radius;
  double *X, *Y, *Z;           /* node coordinates, nx+1 / ny+1 / nz+1 */
  double *Dx, *Dy, *Dz;        /* cell widths, nx / ny / nz */
  double *Dxs, *Dys, *Dzs;     /* centre spacings */
  int scheme;                  /* convection scheme: OG_SCHEME_* (0 after init: QUICK) */
  int les;                     /* != 0: Smagorinsky eddy viscosity in og_run_ex */
  int walls;                   /* y walls: OG_WALLS_* (0 after init: zero-gradient) */
  int time_order;              /* og_run_ex's time stepping: 0 or 1 explicit Euler (the
                                  reference), 2 or 3 Adams-Bashforth (not in the reference) */
  int periodic_z;              /* != 0: periodic in z (not in the reference, whose periodic
                                  Poisson terms, inc/matrix/PressureMatrix.hpp:83-101, are
                                  unused): ghosts wrap, w has nzc unknown faces (face nzc is
                                  the image of face 0), Poisson rows k = 0 and nzc-1 couple */
  int outflow;                 /* OG_OUTFLOW_*: the x+ face (0 after init: zero-gradient) */
} og_grid;

/* the x+ (outlet) face: the reference's zero-gradient row (FLOWpassing.hpp:23-29), or a
 * convective outflow (not in the reference): d(phi)/dt + Uc d(phi)/dx = 0 for the outlet
 * u face and the v, w ghost cells beyond it, implicit upwind in time, Uc the mean inlet
 * velocity, followed by a uniform correction of the outlet u that makes the net flux
 * through the domain boundary zero (the Neumann Poisson problem then is consistent) */
enum { OG_OUTFLOW_ZERO_GRADIENT = 0, OG_OUTFLOW_CONVECTIVE = 1 };

/* Adams-Bashforth history of og_convection_diffusion_ab (no counterpart in the reference,
 * whose 2nd/3rd-order branch does not compile): order 1 is the reference's Euler step;
 * order 2 takes u* = u + (inc + (0.5 r) (inc - r h1)) with r = dt_n / dt_(n-1); order 3
 * (constant dt) u* = u + ((23 inc - 16 h1) + 5 h2) / 12; inc = convection + diffusion of
 * this step, h1 and h2 those of the two steps before.  hnew (may alias h1 for order 2, h2
 * for order 3) receives inc. */
typedef struct og_ab {
  int order;
  double r;
  double *h1[3], *h2[3], *hnew[3];
} og_ab;

/* the y-wall rows of the Dir/Num table (inc/BoundaryCondition/FLOWpassing.hpp): the active
 * zero-gradient rows (:23-29) or the free-slip rows left commented out there (:14-21) */
enum { OG_WALLS_ZERO_GRADIENT = 0, OG_WALLS_FREE_SLIP = 1 };

/* the reference's compile-time convection switch, inc/0_General.hpp:114-118 */
enum { OG_SCHEME_QUICK = 0, OG_SCHEME_LUD = 1, OG_SCHEME_UD = 2 };

int og_grid_init_uniform(og_grid *g, int nxc, int nyc, int nzc, double lx, double ly,
                         double lz, double cx, double cy, double radius);
/* The reference's default stretched "non_uniform-SML" grid (structureGrid.hpp:250-329,
 * 433-487); needs nxc even and > 108, nyc even and > 100.  Returns -1 otherwise. */
int og_grid_init_sml(og_grid *g, int nxc, int nyc, int nzc, double lx, double ly, double lz, double cx,
                     double cy, double radius);
void og_grid_free(og_grid *g);
long og_padded(const og_grid *g);
long og_cells(const og_grid *g);

void og_perturb(const og_grid *g, double *u, double *v, double *w, uint64_t seed, double amp);
void og_convection_diffusion(const og_grid *g, double dt, double nu, const double *u,
                             const double *v, const double *w, double *us, double *vs,
                             double *ws);
/* with g->scheme and, nut != NULL (compact, og_smagorinsky), nu + nut per cell */
void og_convection_diffusion_ex(const og_grid *g, double dt, double nu, const double *nut, const double *u,
                                const double *v, const double *w, double *us, double *vs, double *ws);
void og_convection_diffusion_ab(const og_grid *g, double dt, double nu, const double *nut, const og_ab *ab,
                                const double *u, const double *v, const double *w, double *us, double *vs,
                                double *ws);
/* SmagorinskyModel (inc/source/SmagorinskyModel.hpp:30): compact eddy viscosity of T0 */
void og_smagorinsky(const og_grid *g, const double *u, const double *v, const double *w, double *nut);
void og_bc_main(const og_grid *g, double *u, double *v, double *w, double *p);
/* the ghost fill of a time step with the grid's outflow and z options: us, vs, ws (may be
 * NULL: the fill at init, where the outlet starts from the zero-gradient values) hold the
 * last step's outlet values (the copies og_bc_copy made), dt the step, inlet the inlet u
 * per (j, k) or NULL (1.0) */
void og_bc_main_ex(const og_grid *g, double *u, double *v, double *w, double *p, const double *inlet,
                   const double *us, const double *vs, const double *ws, double dt);
/* the convective velocity of the outflow: the area-weighted mean of the inlet u */
double og_inlet_mean(const og_grid *g, const double *inlet);
void og_bc_copy(const og_grid *g, const double *u, const double *v, const double *w,
                double *us, double *vs, double *ws);
void og_rhs(const og_grid *g, double dt, const double *us, const double *vs,
            const double *ws, const double *jp, double *b);
void og_jacobi_scale(const og_grid *g, double *jp);
void og_spe_setup(const og_grid *g, double *val7);
void og_spe_multiply(const og_grid *g, const double *val7, const double *x, double *y);
void og_csr_multiply(const og_grid *g, const double *jp, const double *x, double *y);

typedef struct og_bicg {
  long n;
  int timestep, iters_max;
  double tol, restart_factor;
  double *r0, *r1, *p1, *s1, *ap, *as, *px1, *px2;
  /* operator: 0 = SPE (unscaled), 1 = CSR rows scaled by jp */
  int kind;
  const og_grid *g;
  double *val7, *jp;
} og_bicg;
int og_bicg_init(og_bicg *s, const og_grid *g, int kind, double tol);
void og_bicg_free(og_bicg *s);
int og_bicg_solve(og_bicg *s, const double *rhs, double *x, double *relres);

/* Conjugate gradients on the SPE operator, the method of inc/solver/cg.hpp (which does
 * not compile as published): r = b - A x, p = r; alpha = <r,r>/<p,Ap>; x += alpha p;
 * r -= alpha Ap; stop on ||r||/||b|| < tol (bicgstabRe2's test) or maxit; beta = <r,r>
 * new/old; p = r + beta p.  Warm start from x.  Returns the iterations. */
int og_cg_solve(const og_grid *g, const double *val7, const double *rhs, double *x, double tol, int maxit,
                double *relres);

int og_sor(const og_grid *g, double dt, double omega, double tol, int itmax,
           const double *us, const double *vs, const double *ws, double *p, double *err);
void og_transform(const og_grid *g, const double *x, double *p);
void og_update_uf(const og_grid *g, double dt, const double *eta, const double *p,
                  const double *us, const double *vs, const double *ws, double *u3,
                  double *v3, double *w3, double *f);
void og_dfib_cylinder_z(const og_grid *g, double *eta);
double og_force_sum(const og_grid *g, const double *f, int dir);

/* get_Cfl (inc/analyses/cfl.hpp:3) on u*: per cell c = u/Dxs + v/Dys + w/Dzs (each face
 * term left out on the last face of its axis), out = {max(c)*dt, U_max[3], U_min[3]}. */
void og_cfl(const og_grid *g, double dt, const double *us, const double *vs, const double *ws,
            double *out7);
/* Plot3D files of the reference (inc/io/Plot3D/xfileWrite.hpp, qfile.hpp): int header,
 * then float32 arrays in k-j-i order (i fastest).  x: cell-centre X, Y, Z.  q: mach 0,
 * alpha 0, Re, time, then p, the cell-centred u, v, w (mean of the two faces) and eta.
 * Return 0, or -1 if the file cannot be written. */
int og_plot3d_x(const og_grid *g, const char *path);
int og_plot3d_q(const og_grid *g, const double *p, const double *u, const double *v, const double *w,
                const double *eta, double Re, double time, const char *path);
/* QfileRead (inc/io/Plot3D/qfileRead.hpp:6): head = {blocks, mach, alpha, Re, time}; the
 * padded p, u, v, w, eta it rebuilds from the cell-centred file (zero outside the interior).
 * Return 0, or -1 if the file cannot be read or its sizes are not this grid's. */
int og_plot3d_read(const og_grid *g, const char *path, double head[5], double *p, double *u, double *v, double *w,
                   double *eta);

/* Whole run in the order of src/RUN_CPU.cpp:257-436.  solver: 0 SPE-BiCGSTAB,
 * 1 CSR(Jacobi)-BiCGSTAB, 2 lexicographic SOR, 3 SPE-CG (og_cg_solve).  Fields in/out are padded; stats gets
 * 4 doubles per step (iters, err, cd, cl).  u,v,w,p on entry: the initial state before
 * the first ghost fill (uniform u=1 plus any perturbation); on exit: T0 and p after the
 * last step. */
int og_run(const og_grid *g, int steps, double Re, double dt, double tol, int solver,
           double omega, double *u, double *v, double *w, double *p, double *eta,
           double *stats);
/* og_run with the two parameters of the adjoint exposed: eta_in (padded solid fraction,
 * NULL: DFIB_CylinderZ) and inlet (ny*nz inlet u per (j,k), NULL: the constant 1 of
 * FLOWpassing.hpp:6); project != 0 removes the right-hand side's null-space part before
 * each BiCGSTAB solve (og_project_rhs; not in the reference). */
int og_run_ex(const og_grid *g, int steps, double Re, double dt, double tol, int solver,
              double omega, double *u, double *v, double *w, double *p, double *eta,
              double *stats, const double *eta_in, const double *inlet, int project);
/* b -= mean of the unscaled rhs (jp != NULL: b holds jp-scaled rows, b -= mean(b/jp) jp).
 * Not in the reference: with a non-uniform inflow its Neumann problem has no solution and
 * its BiCGSTAB diverges; this makes the system consistent. */
void og_project_rhs(const og_grid *g, const double *jp, double *b);

#ifdef __cplusplus
}
#endif
#endif
