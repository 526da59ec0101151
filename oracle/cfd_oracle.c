/* CPU restatement of the reference projection step -- TEST INFRASTRUCTURE ONLY.
 *
 * Each function follows one reference function (file:line cited) operation by operation,
 * in the same left-to-right floating-point order, so that with -ffp-contract=off it
 * agrees bit for bit with the reference compiled at one OpenMP thread (pinned by the
 * golden vectors under tests/golden/, made by tests/golden/make_golden.py from the
 * reference's own code).  Loops are serial: the checker favours exactness over speed.
 * Paths are relative to the reference project's root. */
#include "cfd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#define IC(g, i, j, k) (((long)(i) * (g)->ny + (j)) * (g)->nz + (k))
#define GC 2

static double *dalloc(long n) { return (double *)calloc((size_t)n, sizeof(double)); }

long og_padded(const og_grid *g) { return (long)g->nx * g->ny * g->nz; }
long og_cells(const og_grid *g) { return (long)g->nxc * g->nyc * g->nzc; }

/* inc/grid/structureGrid.hpp:336-367 (init_uniform); X[0] = -2dx, then running sums */
int og_grid_init_uniform(og_grid *g, int nxc, int nyc, int nzc, double lx, double ly,
                         double lz, double cx, double cy, double radius) {
  memset(g, 0, sizeof(*g));
  if (nxc < 3 || nyc < 3 || nzc < 3) return -1;
  g->nxc = nxc; g->nyc = nyc; g->nzc = nzc;
  g->nx = nxc + 2 * GC; g->ny = nyc + 2 * GC; g->nz = nzc + 2 * GC;
  g->lx = lx; g->ly = ly; g->lz = lz; g->cx = cx; g->cy = cy; g->radius = radius;
  g->X = dalloc(g->nx + 1); g->Y = dalloc(g->ny + 1); g->Z = dalloc(g->nz + 1);
  g->Dx = dalloc(g->nx); g->Dy = dalloc(g->ny); g->Dz = dalloc(g->nz);
  g->Dxs = dalloc(g->nx); g->Dys = dalloc(g->ny); g->Dzs = dalloc(g->nz);
  const double dx = lx / (g->nx - 2.0 * GC);
  const double dy = ly / (g->ny - 2.0 * GC);
  const double dz = lz / (g->nz - 2.0 * GC);
  g->X[0] = 0.0 - 2.0 * dx;
  for (int i = 1; i < g->nx + 1; ++i) g->X[i] = g->X[i - 1] + dx;
  g->Y[0] = 0.0 - 2.0 * dy;
  for (int j = 1; j < g->ny + 1; ++j) g->Y[j] = g->Y[j - 1] + dy;
  g->Z[0] = 0.0 - 2.0 * dz;
  for (int k = 1; k < g->nz + 1; ++k) g->Z[k] = g->Z[k - 1] + dz;
  for (int i = 0; i < g->nx; ++i) { g->Dx[i] = dx; g->Dxs[i] = dx; }
  for (int j = 0; j < g->ny; ++j) { g->Dy[j] = dy; g->Dys[j] = dy; }
  for (int k = 0; k < g->nz; ++k) { g->Dz[k] = dz; g->Dzs[k] = dz; }
  return 0;
}

/* inc/grid/structureGrid.hpp:250-310 (unit_SML): nodes a[gC..] of one axis of n padded
 * cells, three uniform parts (coarse d, fine dS = lSml/nS, coarse d), the fine part
 * shifted by off cells; nS = 0 is the plain uniform axis. */
static int unit_sml(double *a, double lsml, int ns, int off, double l, int n) {
  const int ncal = n - 2 * GC;
  const double dS = lsml / ns, d = (l - lsml) / (ncal - ns);
  a[GC] = 0.0;
  if (ns != 0) {
    if ((n - ns) % 2 != 0) return -1;
    int nl0 = (ncal - ns) / 2;
    int ns0 = nl0 + ns;
    const int nl1 = ns0 + nl0;
    nl0 += off;
    ns0 += off;
    if (nl0 <= 0) return -1;
    for (int i = 0; i < nl0; i++) a[i + GC + 1] = a[i + GC] + d;
    for (int i = nl0; i < ns0; ++i) a[i + GC + 1] = a[i + GC] + dS;
    for (int i = ns0; i < nl1; i++) a[i + GC + 1] = a[i + GC] + d;
  } else {
    for (int i = GC; i < n - GC; i++) a[i + 1] = a[i] + l / ncal;
  }
  return 0;
}

/* structureGrid.hpp:433-487 (init_gC_dx): ghost nodes by linear extrapolation, widths
 * and centre spacings, ghost widths copied from the nearest interior ones */
static void init_gc_dx(double *X, double *Dx, double *Dxs, int nx) {
  X[1] = 2 * X[2] - X[3];
  X[0] = 2 * X[1] - X[2];
  X[nx - 1] = 2 * X[nx - 2] - X[nx - 3];
  X[nx] = 2 * X[nx - 1] - X[nx - 2];
  for (int i = GC; i < nx - GC - 1; ++i) Dxs[i] = (X[i + 2] - X[i]) / 2.0;
  for (int i = GC; i < nx - GC - 1; ++i) Dx[i] = (X[i + 1] - X[i]);
  Dx[0] = Dx[1] = Dx[2];
  Dxs[0] = Dxs[1] = Dxs[2];
  Dx[nx - 1] = Dx[nx - 2] = Dx[nx - 3] = X[nx - 2] - X[nx - 3];
  Dxs[nx - 1] = Dxs[nx - 2] = Dxs[nx - 3] = Dxs[nx - 4];
}

/* structureGrid.hpp:312-329 (init_nonuniform_SML, the reference's default gridder):
 * 30 % of x and y resolved by 100 fine cells (x shifted 4 cells upstream), z uniform */
int og_grid_init_sml(og_grid *g, int nxc, int nyc, int nzc, double lx, double ly, double lz, double cx,
                     double cy, double radius) {
  if (og_grid_init_uniform(g, nxc, nyc, nzc, lx, ly, lz, cx, cy, radius)) return -1;
  if (unit_sml(g->X, 0.3 * lx, 100, -4, lx, g->nx) || unit_sml(g->Y, 0.3 * ly, 100, 0, ly, g->ny) ||
      unit_sml(g->Z, 0.5 * lz, 0, 0, lz, g->nz)) {
    og_grid_free(g);
    return -1;
  }
  init_gc_dx(g->X, g->Dx, g->Dxs, g->nx);
  init_gc_dx(g->Y, g->Dy, g->Dys, g->ny);
  init_gc_dx(g->Z, g->Dz, g->Dzs, g->nz);
  return 0;
}

void og_grid_free(og_grid *g) {
  free(g->X); free(g->Y); free(g->Z);
  free(g->Dx); free(g->Dy); free(g->Dz);
  free(g->Dxs); free(g->Dys); free(g->Dzs);
  memset(g, 0, sizeof(*g));
}

/* seeded perturbation added to the interior of u, then v, then w (icel order) */
static uint64_t splitmix64(uint64_t *s) {
  *s += 0x9E3779B97F4A7C15ULL;
  uint64_t z = *s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
void og_perturb(const og_grid *g, double *u, double *v, double *w, uint64_t seed, double amp) {
  uint64_t s = seed;
  double *f[3] = {u, v, w};
  for (int c = 0; c < 3; ++c)
    for (int i = GC; i < g->nx - GC; ++i)
      for (int j = GC; j < g->ny - GC; ++j)
        for (int k = GC; k < g->nz - GC; ++k) {
          const double r = (double)(splitmix64(&s) >> 11) * (1.0 / 9007199254740992.0);
          f[c][IC(g, i, j, k)] += amp * (2.0 * r - 1.0);
        }
}

/* inc/source/Convection_Difussion.hpp:20-51 (QuickUnitA) */
static void quick_a(double Up, double Un, long pp, long p, long ic, long n, long nn,
                    const double *Di, const double *Ds, int I, const double *phi,
                    double *P, double *N) {
  if (Up > 0.0)
    *P = 0.5 * (phi[ic] + phi[p]) - 0.125 * Di[I + 1] * Di[I + 1] / Ds[I] *
             ((phi[p] - phi[ic]) / Di[I + 1] - (phi[ic] - phi[n]) / Di[I]);
  else
    *P = 0.5 * (phi[ic] + phi[p]) - 0.125 * Di[I + 1] * Di[I + 1] / Ds[I + 1] *
             ((phi[pp] - phi[p]) / Di[I + 2] - (phi[p] - phi[ic]) / Di[I + 1]);
  if (Un > 0.0)
    *N = 0.5 * (phi[n] + phi[ic]) - 0.125 * Di[I] * Di[I] / Ds[I - 1] *
             ((phi[ic] - phi[n]) / Di[I] - (phi[n] - phi[nn]) / Di[I - 1]);
  else
    *N = 0.5 * (phi[n] + phi[ic]) - 0.125 * Di[I] * Di[I] / Ds[I] *
             ((phi[p] - phi[ic]) / Di[I + 1] - (phi[ic] - phi[n]) / Di[I]);
}

/* inc/source/Convection_Difussion.hpp:55-90 (QuickUnitB) */
static void quick_b(double Up, double Un, long pp, long p, long ic, long n, long nn,
                    const double *Di, const double *Ds, int I, const double *phi,
                    double *P, double *N) {
  if (Up > 0.0)
    *P = 0.5 * (phi[ic] + phi[p]) - 0.125 * Ds[I] * Ds[I] / Di[I] *
             ((phi[p] - phi[ic]) / Ds[I] - (phi[ic] - phi[n]) / Ds[I - 1]);
  else
    *P = 0.5 * (phi[ic] + phi[p]) - 0.125 * Ds[I] * Ds[I] / Di[I + 1] *
             ((phi[pp] - phi[p]) / Ds[I + 1] - (phi[p] - phi[ic]) / Ds[I]);
  if (Un > 0.0)
    *N = 0.5 * (phi[n] + phi[ic]) - 0.125 * Ds[I - 1] * Ds[I - 1] / Di[I - 1] *
             ((phi[ic] - phi[n]) / Ds[I - 1] - (phi[n] - phi[nn]) / Ds[I - 2]);
  else
    *N = 0.5 * (phi[n] + phi[ic]) - 0.125 * Ds[I - 1] * Ds[I - 1] / Di[I] *
             ((phi[p] - phi[ic]) / Ds[I] - (phi[ic] - phi[n]) / Ds[I - 1]);
}

/* inc/source/Convection_Difussion.hpp:96-147 (LudUnitA; LudUnitB has the same body):
 * linear upwind, the upwind cell extrapolated half a spacing */
static void lud(double Up, double Un, long pp, long p, long ic, long n, long nn, const double *Di,
                const double *Ds, int I, const double *phi, double *P, double *N) {
  if (Up > 0.0)
    *P = (phi[ic] + 0.5 * Ds[I] * (phi[ic] - phi[n]) / Di[I]);
  else
    *P = (phi[p] + 0.5 * Ds[I + 1] * (phi[p] - phi[pp]) / Di[I + 1]);
  if (Un > 0.0)
    *N = (phi[n] + 0.5 * Ds[I - 1] * (phi[n] - phi[nn]) / Di[I - 1]);
  else
    *N = (phi[ic] + 0.5 * Ds[I] * (phi[ic] - phi[p]) / Di[I + 1]);
}

/* inc/source/Convection_Difussion.hpp:150-168 (UdUnit): first-order upwind */
static void ud(double Up, double Un, long p, long ic, long n, const double *phi, double *P, double *N) {
  *P = Up > 0.0 ? phi[ic] : phi[p];
  *N = Un > 0.0 ? phi[n] : phi[ic];
}

/* the face values of one axis under the compile-time scheme switch of
 * inc/0_General.hpp:114-118; own: the axis is the component's own (the "A" units) */
static void face(int scheme, int own, double Up, double Un, long pp, long p, long ic, long n, long nn,
                 const double *Di, const double *Ds, int I, const double *phi, double *P, double *N) {
  if (scheme == OG_SCHEME_LUD)
    lud(Up, Un, pp, p, ic, n, nn, Di, Ds, I, phi, P, N);
  else if (scheme == OG_SCHEME_UD)
    ud(Up, Un, p, ic, n, phi, P, N);
  else if (own)
    quick_a(Up, Un, pp, p, ic, n, nn, Di, Ds, I, phi, P, N);
  else
    quick_b(Up, Un, pp, p, ic, n, nn, Di, Ds, I, phi, P, N);
}

/* inc/source/SmagorinskyModel.hpp:30-79 (SmagorinskyModel, CS = 0.18) with GradientGauss
 * (:6-26): nut[icelCal] = (CS delta)^2 sqrt|S| of T0, central differences of u (metrics
 * Dxs, Dy, Dz), v (Dx, Dys, Dz) and w (Dx, Dy, Dzs) at the cell, delta = the cube root of
 * the cell volume.  The reference's sum is kept as written: the factor 2 multiplies
 * du/dx^2 alone, and its gradients carry the opposite sign (they are only squared). */
void og_smagorinsky(const og_grid *g, const double *u, const double *v, const double *w, double *nut) {
  const double CS = 0.18;
  const long sx = (long)g->ny * g->nz, sy = g->nz;
  const double *M[3][3] = {{g->Dxs, g->Dy, g->Dz}, {g->Dx, g->Dys, g->Dz}, {g->Dx, g->Dy, g->Dzs}};
  const double *F[3] = {u, v, w};
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k) {
        const long c = IC(g, i, j, k);
        double d[3][3]; /* d[field][axis] */
        for (int f = 0; f < 3; ++f) {
          d[f][0] = 0.5 / M[f][0][i] * (F[f][c - sx] - F[f][c + sx]);
          d[f][1] = 0.5 / M[f][1][j] * (F[f][c - sy] - F[f][c + sy]);
          d[f][2] = 0.5 / M[f][2][k] * (F[f][c - 1] - F[f][c + 1]);
        }
        const double a = d[0][1] + d[1][0], b = d[0][2] + d[2][0], e = d[1][2] + d[2][1];
        const double temp = fabs(2.0 * (d[0][0] * d[0][0]) + d[1][1] * d[1][1] + d[2][2] * d[2][2] + a * a +
                                 b * b + e * e);
        const double delta = pow(g->Dx[i] * g->Dy[j] * g->Dz[k], 1.0 / 3.0);
        const double l = CS * delta;
        nut[((long)(i - GC) * g->nyc + (j - GC)) * g->nzc + (k - GC)] = (l * l) * sqrt(temp);
      }
}

/* inc/source/Convection_Difussion.hpp:174-450 (ConvectionDifussion, 1st order in time) */
void og_convection_diffusion(const og_grid *g, double dt, double nu, const double *u,
                             const double *v, const double *w, double *us, double *vs,
                             double *ws) {
  og_convection_diffusion_ex(g, dt, nu, NULL, u, v, w, us, vs, ws);
}

/* the same with the scheme of g->scheme and, nut != NULL, the eddy viscosity of the
 * Smagorinsky model added to nu per cell (Convection_Difussion.hpp:251-256) */
void og_convection_diffusion_ex(const og_grid *g, double dt, double nu0, const double *nut, const double *u,
                                const double *v, const double *w, double *us, double *vs, double *ws) {
  og_convection_diffusion_ab(g, dt, nu0, nut, NULL, u, v, w, us, vs, ws);
}

/* the new value of a component: the reference's u + convection + diffusion (ab NULL or
 * order 1), else the Adams-Bashforth combination of og_ab */
static double ab_value(const og_ab *ab, int c, long ic, double uc, double convection, double difussion) {
  if (!ab || ab->order <= 1) {
    if (ab && ab->hnew[c]) ab->hnew[c][ic] = convection + difussion;
    return uc + convection + difussion;
  }
  const double inc = convection + difussion;
  const double h1 = ab->h1[c][ic];
  double r;
  if (ab->order == 2) {
    r = uc + (inc + (0.5 * ab->r) * (inc - ab->r * h1));
  } else {
    r = uc + ((23.0 * inc - 16.0 * h1) + 5.0 * ab->h2[c][ic]) / 12.0;
  }
  ab->hnew[c][ic] = inc;
  return r;
}

void og_convection_diffusion_ab(const og_grid *g, double dt, double nu0, const double *nut, const og_ab *ab,
                                const double *u, const double *v, const double *w, double *us, double *vs,
                                double *ws) {
  const long sx = (long)g->ny * g->nz, sy = g->nz, sz = 1;
  const int sc = g->scheme;
#define NU_AT(i, j, k) (nut ? nu0 + nut[((long)((i) - GC) * g->nyc + ((j) - GC)) * g->nzc + ((k) - GC)] : nu0)
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  /* u: last x face (i = nx-3) is a boundary face (:198-204) */
  for (int i = GC; i < nx - GC - 1; ++i)
    for (int j = GC; j < ny - GC; ++j)
      for (int k = GC; k < nz - GC; ++k) {
        const long ic = IC(g, i, j, k);
        const long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                   zp = ic + sz;
        const double IT = (g->Dxs[i] * 0.5) / g->Dx[i];
        const double Up = 0.5 * (u[xp] + u[ic]);
        const double Un = 0.5 * (u[xm] + u[ic]);
        const double Vp = v[ic] + (v[xp] - v[ic]) * IT;
        const double Vn = v[ym] + (v[ym + xp - ic] - v[ym]) * IT;
        const double Wp = w[ic] + (w[xp] - w[ic]) * IT;
        const double Wn = w[zm] + (w[zm + xp - ic] - w[zm]) * IT;
        double uPx, uNx, uPy, uNy, uPz, uNz;
        face(sc, 1, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, g->Dx, g->Dxs, i, u, &uPx, &uNx);
        face(sc, 0, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, g->Dy, g->Dys, j, u, &uPy, &uNy);
        face(sc, 0, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, g->Dz, g->Dzs, k, u, &uPz, &uNz);
        const double convection = -dt * ((uPx * uPx - uNx * uNx) / g->Dxs[i] +
                                         (uPy * Vp - uNy * Vn) / g->Dy[j] +
                                         (uPz * Wp - uNz * Wn) / g->Dz[k]);
        const double nu = NU_AT(i, j, k);
        const double difussion =
            nu * dt *
            (((u[xp] - u[ic]) / g->Dx[i + 1] - (u[ic] - u[xm]) / g->Dx[i]) / g->Dxs[i] +
             ((u[yp] - u[ic]) / g->Dys[j] - (u[ic] - u[ym]) / g->Dys[j - 1]) / g->Dy[j] +
             ((u[zp] - u[ic]) / g->Dzs[k] - (u[ic] - u[zm]) / g->Dzs[k - 1]) / g->Dz[k]);
        us[ic] = ab_value(ab, 0, ic, u[ic], convection, difussion);
      }
  /* v: :276-355 */
  for (int i = GC; i < nx - GC; ++i)
    for (int j = GC; j < ny - GC - 1; ++j)
      for (int k = GC; k < nz - GC; ++k) {
        const long ic = IC(g, i, j, k);
        const long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                   zp = ic + sz;
        const double IT = (g->Dys[j] * 0.5) / g->Dy[j];
        const double Vp = 0.5 * (v[yp] + v[ic]);
        const double Vn = 0.5 * (v[ym] + v[ic]);
        const double Up = u[ic] + (u[yp] - u[ic]) * IT;
        const double Un = u[xm] + (u[xm + yp - ic] - u[xm]) * IT;
        const double Wp = w[ic] + (w[yp] - w[ic]) * IT;
        const double Wn = w[zm] + (w[zm + yp - ic] - w[zm]) * IT;
        double vPx, vNx, vPy, vNy, vPz, vNz;
        face(sc, 0, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, g->Dx, g->Dxs, i, v, &vPx, &vNx);
        face(sc, 1, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, g->Dy, g->Dys, j, v, &vPy, &vNy);
        face(sc, 0, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, g->Dz, g->Dzs, k, v, &vPz, &vNz);
        const double convection = -dt * ((Up * vPx - Un * vNx) / g->Dx[i] +
                                         (vPy * vPy - vNy * vNy) / g->Dys[j] +
                                         (Wp * vPz - Wn * vNz) / g->Dz[k]);
        const double nu = NU_AT(i, j, k);
        const double difussion =
            nu * dt *
            (((v[xp] - v[ic]) / g->Dxs[i] - (v[ic] - v[xm]) / g->Dxs[i - 1]) / g->Dx[i] +
             ((v[yp] - v[ic]) / g->Dy[j + 1] - (v[ic] - v[ym]) / g->Dy[j]) / g->Dys[j] +
             ((v[zp] - v[ic]) / g->Dzs[k] - (v[ic] - v[zm]) / g->Dzs[k - 1]) / g->Dz[k]);
        vs[ic] = ab_value(ab, 1, ic, v[ic], convection, difussion);
      }
  /* w: :359-438; periodic z adds the top face nz-3 (the image of face 1) as an unknown */
  const int kw_end = nz - GC - 1 + (g->periodic_z != 0);
  for (int i = GC; i < nx - GC; ++i)
    for (int j = GC; j < ny - GC; ++j)
      for (int k = GC; k < kw_end; ++k) {
        const long ic = IC(g, i, j, k);
        const long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                   zp = ic + sz;
        const double IT = (g->Dzs[k] * 0.5) / g->Dz[k];
        const double Wp = 0.5 * (w[zp] + w[ic]);
        const double Wn = 0.5 * (w[zm] + w[ic]);
        const double Up = u[ic] + (u[zp] - u[ic]) * IT;
        const double Un = u[xm] + (u[xm + zp - ic] - u[xm]) * IT;
        const double Vp = v[ic] + (v[zp] - v[ic]) * IT;
        const double Vn = v[ym] + (v[ym + zp - ic] - v[ym]) * IT;
        double wPx, wNx, wPy, wNy, wPz, wNz;
        face(sc, 0, Up, Un, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, g->Dx, g->Dxs, i, w, &wPx, &wNx);
        face(sc, 0, Vp, Vn, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, g->Dy, g->Dys, j, w, &wPy, &wNy);
        face(sc, 1, Wp, Wn, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, g->Dz, g->Dzs, k, w, &wPz, &wNz);
        const double convection = -dt * ((Up * wPx - Un * wNx) / g->Dx[i] +
                                         (Vp * wPy - Vn * wNy) / g->Dy[j] +
                                         (wPz * wPz - wNz * wNz) / g->Dzs[k]);
        const double nu = NU_AT(i, j, k);
        const double difussion =
            nu * dt *
            (((w[xp] - w[ic]) / g->Dxs[i] - (w[ic] - w[xm]) / g->Dxs[i - 1]) / g->Dx[i] +
             ((w[yp] - w[ic]) / g->Dys[j] - (w[ic] - w[ym]) / g->Dys[j - 1]) / g->Dy[j] +
             ((w[zp] - w[ic]) / g->Dz[k + 1] - (w[ic] - w[zm]) / g->Dz[k]) / g->Dzs[k]);
        ws[ic] = ab_value(ab, 2, ic, w[ic], convection, difussion);
      }
#undef NU_AT
}

/* Dir/Num table of inc/BoundaryCondition/FLOWpassing.hpp:6-40: face 0 inlet u=1 with
 * reflected (no-slip) v,w; every other face zero-gradient on u, v and w. */
static const double kDir[6][3] = {{1, 0, 0}, {0, 0, 0}, {0, 0, 0},
                                  {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
static const double kNum[6][3] = {{0, 0, 0}, {1, 1, 1}, {1, 1, 1},
                                  {1, 1, 1}, {1, 1, 1}, {1, 1, 1}};

/* the Num rows with the grid's choice of y walls (free slip: v Dirichlet 0 on faces 2, 3) */
static void num_table(const og_grid *g, double N[6][3]) {
  memcpy(N, kNum, sizeof(kNum));
  if (g->walls == OG_WALLS_FREE_SLIP) N[2][1] = N[3][1] = 0.0;
}

double og_inlet_mean(const og_grid *g, const double *inlet) {
  double q = 0.0, a = 0.0;
  for (int j = GC; j < g->ny - GC; ++j)
    for (int k = GC; k < g->nz - GC; ++k) {
      const double da = g->Dy[j] * g->Dz[k];
      q += (inlet ? inlet[(j - GC) * g->nzc + (k - GC)] : kDir[0][0]) * da;
      a += da;
    }
  return q / a;
}

/* convective outflow: the outlet u face before the flux correction -- at init (us NULL) the
 * zero-gradient value, in a step (u_b + cu u_(nx-4)) / (1 + cu) with u_b the last step's
 * outlet value (kept in us by og_bc_copy) and cu = Uc dt / Dx of the last cell */
static double outlet_u(const og_grid *g, const double *u, const double *us, double cu, int j, int k) {
  const int nx = g->nx;
  if (!us) return u[IC(g, nx - 4, j, k)];
  return (us[IC(g, nx - 3, j, k)] + cu * u[IC(g, nx - 4, j, k)]) / (1.0 + cu);
}
/* the v or w ghost cell beyond the outlet, the same way from the last cell (cv = Uc dt / Dxs) */
static double outlet_ghost(const og_grid *g, const double *f, const double *fs, double cv, int j, int k) {
  const int nx = g->nx;
  if (!fs) return f[IC(g, nx - 3, j, k)];
  return (fs[IC(g, nx - 2, j, k)] + cv * f[IC(g, nx - 3, j, k)]) / (1.0 + cv);
}

/* the uniform correction of the outlet u that makes the net boundary flux zero: inlet u
 * face, outlet faces (outlet_u), and, with the values the ghost fill gives them, the y-wall
 * v faces and (not periodic) the z-wall w faces, each times its face area; divided by the
 * outlet's area */
static double outflow_correction(const og_grid *g, const double kN[6][3], const double *u, const double *v,
                                 const double *w, const double *inlet, const double *us, double cu) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  double F = 0.0, A = 0.0;
  for (int j = GC; j < ny - GC; ++j)
    for (int k = GC; k < nz - GC; ++k) {
      const double a = g->Dy[j] * g->Dz[k];
      const double uin = (inlet ? inlet[(j - GC) * g->nzc + (k - GC)] : kDir[0][0]) + kN[0][0] * u[IC(g, 2, j, k)];
      F += (uin - outlet_u(g, u, us, cu, j, k)) * a;
      A += a;
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int k = GC; k < nz - GC; ++k) {
      const double vb = kDir[2][1] + kN[2][1] * v[IC(g, i, 2, k)];
      const double vt = kDir[3][1] + kN[3][1] * v[IC(g, i, ny - 4, k)];
      F += (vb - vt) * (g->Dx[i] * g->Dz[k]);
    }
  if (!g->periodic_z)
    for (int i = GC; i < nx - GC; ++i)
      for (int j = GC; j < ny - GC; ++j) {
        const double wb = kDir[4][2] + kN[4][2] * w[IC(g, i, j, 2)];
        const double wt = kDir[5][2] + kN[5][2] * w[IC(g, i, j, nz - 4)];
        F += (wb - wt) * (g->Dx[i] * g->Dy[j]);
      }
  return F / A;
}

/* periodic z: the two ghost layers on each side take the images of the cells nzc away
 * (for w, face 1 is the image of the top face nz-3), over every (i, j) of the padded plane
 * so that edges and corners next to the z ghosts are periodic too */
static void periodic_z_fill(const og_grid *g, double *f) {
  const int nz = g->nz;
  for (int i = 0; i < g->nx; ++i)
    for (int j = 0; j < g->ny; ++j) {
      const long b = IC(g, i, j, 0);
      f[b + 0] = f[b + nz - 4];
      f[b + 1] = f[b + nz - 3];
      f[b + nz - 2] = f[b + 2];
      f[b + nz - 1] = f[b + 3];
    }
}

/* inc/BoundaryCondition/Boundary_Condition.hpp:37-176 (BC_staggered_main), in the
 * order one thread executes it: faces 0..5 for u,v,w, then pressure.  With the grid's
 * options (not in the reference): the convective outflow in place of face 1's rows, and
 * periodic z in place of faces 4 and 5 and of the pressure's z rows. */
static void bc_main_in(const og_grid *g, double *u, double *v, double *w, double *p, const double *inlet,
                       const double *us, const double *vs, const double *ws, double dt) {
  double kN[6][3];
  num_table(g, kN);
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  double *vel[3] = {u, v, w};
  const int conv = g->outflow == OG_OUTFLOW_CONVECTIVE;
  double cu = 0.0, cv = 0.0, corr = 0.0;
  if (conv) {
    if (us) {
      const double uc = og_inlet_mean(g, inlet);
      cu = uc * dt / g->Dx[nx - 3];
      cv = uc * dt / g->Dxs[nx - 3];
    }
    corr = outflow_correction(g, (const double(*)[3])kN, u, v, w, inlet, us, cu);
  }
  for (int j = GC; j < ny - GC; ++j)
    for (int k = GC; k < nz - GC; ++k) { /* BC_0 */
      const double din = inlet ? inlet[(j - GC) * g->nzc + (k - GC)] : kDir[0][0];
      u[IC(g, 1, j, k)] = u[IC(g, 0, j, k)] = din + kN[0][0] * u[IC(g, 2, j, k)];
      v[IC(g, 1, j, k)] = v[IC(g, 0, j, k)] =
          kDir[0][1] * 2. + (2.0 * kN[0][1] - 1.0) * v[IC(g, 2, j, k)];
      w[IC(g, 1, j, k)] = w[IC(g, 0, j, k)] =
          kDir[0][2] * 2. + (2.0 * kN[0][2] - 1.0) * w[IC(g, 2, j, k)];
    }
  for (int j = GC; j < ny - GC && conv; ++j)
    for (int k = GC; k < nz - GC; ++k) { /* convective outflow */
      u[IC(g, nx - 1, j, k)] = u[IC(g, nx - 2, j, k)] = u[IC(g, nx - 3, j, k)] =
          outlet_u(g, u, us, cu, j, k) + corr;
      v[IC(g, nx - 1, j, k)] = v[IC(g, nx - 2, j, k)] = outlet_ghost(g, v, vs, cv, j, k);
      w[IC(g, nx - 1, j, k)] = w[IC(g, nx - 2, j, k)] = outlet_ghost(g, w, ws, cv, j, k);
    }
  for (int j = GC; j < ny - GC && !conv; ++j)
    for (int k = GC; k < nz - GC; ++k) { /* BC_1 */
      u[IC(g, nx - 1, j, k)] = u[IC(g, nx - 2, j, k)] = u[IC(g, nx - 3, j, k)] =
          kDir[1][0] + kN[1][0] * u[IC(g, nx - 4, j, k)];
      v[IC(g, nx - 1, j, k)] = v[IC(g, nx - 2, j, k)] =
          kDir[1][1] * 2. + (2.0 * kN[1][1] - 1.0) * v[IC(g, nx - 3, j, k)];
      w[IC(g, nx - 1, j, k)] = w[IC(g, nx - 2, j, k)] =
          kDir[1][2] * 2. + (2.0 * kN[1][2] - 1.0) * w[IC(g, nx - 3, j, k)];
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int k = GC; k < nz - GC; ++k) { /* BC_2 */
      u[IC(g, i, 1, k)] = u[IC(g, i, 0, k)] =
          kDir[2][0] * 2. + (2.0 * kN[2][0] - 1.0) * u[IC(g, i, 2, k)];
      v[IC(g, i, 1, k)] = v[IC(g, i, 0, k)] = kDir[2][1] + kN[2][1] * v[IC(g, i, 2, k)];
      w[IC(g, i, 1, k)] = w[IC(g, i, 0, k)] =
          kDir[2][2] * 2. + (2.0 * kN[2][2] - 1.0) * w[IC(g, i, 2, k)];
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int k = GC; k < nz - GC; ++k) { /* BC_3 */
      v[IC(g, i, ny - 1, k)] = v[IC(g, i, ny - 2, k)] = v[IC(g, i, ny - 3, k)] =
          kDir[3][1] + kN[3][1] * v[IC(g, i, ny - 4, k)];
      u[IC(g, i, ny - 1, k)] = u[IC(g, i, ny - 2, k)] =
          kDir[3][0] * 2. + (2.0 * kN[3][0] - 1.0) * u[IC(g, i, ny - 3, k)];
      w[IC(g, i, ny - 1, k)] = w[IC(g, i, ny - 2, k)] =
          kDir[3][2] * 2. + (2.0 * kN[3][2] - 1.0) * w[IC(g, i, ny - 3, k)];
    }
  if (g->periodic_z)
    for (int c = 0; c < 3; ++c) periodic_z_fill(g, vel[c]);
  for (int i = GC; i < nx - GC && !g->periodic_z; ++i)
    for (int j = GC; j < ny - GC; ++j) { /* BC_4 */
      u[IC(g, i, j, 1)] = u[IC(g, i, j, 0)] =
          kDir[4][0] * 2. + (2.0 * kN[4][0] - 1.0) * u[IC(g, i, j, 2)];
      v[IC(g, i, j, 1)] = v[IC(g, i, j, 0)] =
          kDir[4][1] * 2. + (2.0 * kN[4][1] - 1.0) * v[IC(g, i, j, 2)];
      w[IC(g, i, j, 1)] = w[IC(g, i, j, 0)] = kDir[4][2] + kN[4][2] * w[IC(g, i, j, 2)];
    }
  for (int i = GC; i < nx - GC && !g->periodic_z; ++i)
    for (int j = GC; j < ny - GC; ++j) { /* BC_5 */
      w[IC(g, i, j, nz - 1)] = w[IC(g, i, j, nz - 2)] = w[IC(g, i, j, nz - 3)] =
          kDir[5][2] + kN[5][2] * w[IC(g, i, j, nz - 4)];
      u[IC(g, i, j, nz - 1)] = u[IC(g, i, j, nz - 2)] =
          kDir[5][0] * 2. + (2.0 * kN[5][0] - 1.0) * u[IC(g, i, j, nz - 3)];
      v[IC(g, i, j, nz - 1)] = v[IC(g, i, j, nz - 2)] =
          kDir[5][1] * 2. + (2.0 * kN[5][1] - 1.0) * v[IC(g, i, j, nz - 3)];
    }
  /* pressure: homogeneous Neumann, :148-172 */
  for (int j = GC; j < ny - GC; ++j)
    for (int k = GC; k < nz - GC; ++k) {
      p[IC(g, 1, j, k)] = p[IC(g, 0, j, k)] = p[IC(g, 2, j, k)];
      p[IC(g, nx - 2, j, k)] = p[IC(g, nx - 1, j, k)] = p[IC(g, nx - 3, j, k)];
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int k = GC; k < nz - GC; ++k) {
      p[IC(g, i, 1, k)] = p[IC(g, i, 0, k)] = p[IC(g, i, 2, k)];
      p[IC(g, i, ny - 2, k)] = p[IC(g, i, ny - 1, k)] = p[IC(g, i, ny - 3, k)];
    }
  if (g->periodic_z) {
    periodic_z_fill(g, p);
    return;
  }
  for (int i = GC; i < nx - GC; ++i)
    for (int j = GC; j < ny - GC; ++j) {
      p[IC(g, i, j, 1)] = p[IC(g, i, j, 0)] = p[IC(g, i, j, 2)];
      p[IC(g, i, j, nz - 2)] = p[IC(g, i, j, nz - 1)] = p[IC(g, i, j, nz - 3)];
    }
}

void og_bc_main(const og_grid *g, double *u, double *v, double *w, double *p) {
  bc_main_in(g, u, v, w, p, NULL, NULL, NULL, NULL, 0.0);
}

void og_bc_main_ex(const og_grid *g, double *u, double *v, double *w, double *p, const double *inlet,
                   const double *us, const double *vs, const double *ws, double dt) {
  bc_main_in(g, u, v, w, p, inlet, us, vs, ws, dt);
}

/* inc/BoundaryCondition/updateBC.hpp:6-108 (BC_staggered_copy) */
void og_bc_copy(const og_grid *g, const double *u, const double *v, const double *w,
                double *us, double *vs, double *ws) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
#define CP(a, b, idx) (b)[idx] = (a)[idx]
  for (int j = GC; j < ny - GC; ++j)
    for (int k = GC; k < nz - GC; ++k) {
      const int iu[5] = {0, 1, nx - 1, nx - 3, nx - 2};
      for (int q = 0; q < 5; ++q) CP(u, us, IC(g, iu[q], j, k));
      const int iv[4] = {0, 1, nx - 2, nx - 1};
      for (int q = 0; q < 4; ++q) { CP(v, vs, IC(g, iv[q], j, k)); CP(w, ws, IC(g, iv[q], j, k)); }
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int k = GC; k < nz - GC; ++k) {
      const int ju[4] = {0, 1, ny - 2, ny - 1};
      for (int q = 0; q < 4; ++q) { CP(u, us, IC(g, i, ju[q], k)); CP(w, ws, IC(g, i, ju[q], k)); }
      const int jv[5] = {0, 1, ny - 3, ny - 2, ny - 1};
      for (int q = 0; q < 5; ++q) CP(v, vs, IC(g, i, jv[q], k));
    }
  for (int i = GC; i < nx - GC; ++i)
    for (int j = GC; j < ny - GC; ++j) {
      const int ku[4] = {0, 1, nz - 2, nz - 1};
      for (int q = 0; q < 4; ++q) { CP(u, us, IC(g, i, j, ku[q])); CP(v, vs, IC(g, i, j, ku[q])); }
      const int kw[5] = {0, 1, nz - 3, nz - 2, nz - 1};
      for (int q = 0; q < 5; ++q) CP(w, ws, IC(g, i, j, kw[q]));
    }
#undef CP
}

/* inc/matrix/b_matrix.hpp:35-98 (createBMatrix_omp); jp == NULL is the unscaled branch */
void og_rhs(const og_grid *g, double dt, const double *us, const double *vs,
            const double *ws, const double *jp, double *b) {
  const double ddt = 1.0 / dt;
  const long sx = (long)g->ny * g->nz, sy = g->nz;
  long row = 0;
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k, ++row) {
        const long ic = IC(g, i, j, k);
        /* periodic z: the bottom face of the first cell is the top face nz-3 */
        const long zb = (g->periodic_z && k == GC) ? IC(g, i, j, g->nz - 3) : ic - 1;
        const double div = (us[ic] - us[ic - sx]) / g->Dx[i] + (vs[ic] - vs[ic - sy]) / g->Dy[j] +
                           (ws[ic] - ws[zb]) / g->Dz[k];
        if (jp)
          b[row] = -jp[row] * ddt * div;
        else
          b[row] = -ddt * div;
      }
}

/* coefficient helpers of inc/grid/structureGrid.hpp:560-566 and SPE_sparseMatrix.hpp:93-99 */
static double cxp(const og_grid *g, int i) { return 1.0 / g->Dx[i + GC] / g->Dxs[i + GC]; }
static double cyp(const og_grid *g, int j) { return 1.0 / g->Dy[j + GC] / g->Dys[j + GC]; }
static double czp(const og_grid *g, int k) { return 1.0 / g->Dz[k + GC] / g->Dzs[k + GC]; }
static double cxm(const og_grid *g, int i) { return 1.0 / g->Dx[i + GC] / g->Dxs[i + GC - 1]; }
static double cym(const og_grid *g, int j) { return 1.0 / g->Dy[j + GC] / g->Dys[j + GC - 1]; }
static double czm(const og_grid *g, int k) { return 1.0 / g->Dz[k + GC] / g->Dzs[k + GC - 1]; }

/* inc/grid/structureGrid.hpp:583-603: jp = 1/diag of the Neumann operator */
void og_jacobi_scale(const og_grid *g, double *jp) {
  long row = 0;
  for (int i = 0; i < g->nxc; ++i)
    for (int j = 0; j < g->nyc; ++j)
      for (int k = 0; k < g->nzc; ++k, ++row) {
        double aa = 0.0, bb = 0.0, cc = 0.0;
        if (i == 0) aa = -cxm(g, i);
        if (i == g->nxc - 1) aa = -cxp(g, i);
        if (j == 0) bb = -cym(g, j);
        if (j == g->nyc - 1) bb = -cyp(g, j);
        if (k == 0 && !g->periodic_z) cc = -czm(g, k);
        if (k == g->nzc - 1 && !g->periodic_z) cc = -czp(g, k);
        const double ijk = cxm(g, i) + cym(g, j) + czm(g, k) + cxp(g, i) + cyp(g, j) +
                           czp(g, k) + aa + bb + cc;
        jp[row] = 1.0 / ijk;
      }
}

/* inc/matrix/SPE_sparseMatrix.hpp:42-88 (setupPressure), including the swapped
 * y-coefficients of :79/:83 (identical on a uniform grid).  Periodic z: every row keeps
 * both z terms, the k = 0 and nzc-1 rows' outer ones coupling them (og_spe_multiply). */
void og_spe_setup(const og_grid *g, double *val) {
  const int nx = g->nxc, ny = g->nyc, nz = g->nzc, pz = g->periodic_z != 0;
  memset(val, 0, sizeof(double) * 7 * (size_t)og_cells(g));
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        const long ic7 = ((long)k + (long)j * nz + (long)i * ny * nz) * 7;
        double ijk = cxm(g, i) + cym(g, j) + czm(g, k) + cxp(g, i) + cyp(g, j) + czp(g, k);
        if (i == 0) ijk -= cxm(g, i);
        if (i == nx - 1) ijk -= cxp(g, i);
        if (j == 0) ijk -= cym(g, j);
        if (j == ny - 1) ijk -= cyp(g, j);
        if (k == 0 && !pz) ijk -= czm(g, k);
        if (k == nz - 1 && !pz) ijk -= czp(g, k);
        if (i != 0) val[ic7 + 0] = -cxm(g, i);
        if (j != 0) val[ic7 + 1] = -cyp(g, j);
        if (k != 0 || pz) val[ic7 + 2] = -czm(g, k);
        val[ic7 + 3] = ijk;
        if (k != nz - 1 || pz) val[ic7 + 4] = -czp(g, k);
        if (j != ny - 1) val[ic7 + 5] = -cym(g, j);
        if (i != nx - 1) val[ic7 + 6] = -cxp(g, i);
      }
}

/* inc/matrix/SPE_sparseMatrix.hpp:92-108 (multiply_omp; bounds tested on the row index) */
void og_spe_multiply(const og_grid *g, const double *val, const double *x, double *r) {
  const long n = og_cells(g), nz = g->nzc, nynz = (long)g->nyc * g->nzc;
  if (g->periodic_z) { /* z neighbours by the cell's k, wrapping at the ends */
    for (long i = 0; i < n; ++i) {
      const long k = i % nz, i7 = i * 7;
      double sum = 0.0;
      if (i - nynz >= 0) sum += val[i7 + 0] * x[i - nynz];
      if (i - nz >= 0) sum += val[i7 + 1] * x[i - nz];
      sum += val[i7 + 2] * x[k == 0 ? i + nz - 1 : i - 1];
      sum += val[i7 + 3] * x[i];
      sum += val[i7 + 4] * x[k == nz - 1 ? i - (nz - 1) : i + 1];
      if (i + nz < n) sum += val[i7 + 5] * x[i + nz];
      if (i + nynz < n) sum += val[i7 + 6] * x[i + nynz];
      r[i] = sum;
    }
    return;
  }
  for (long i = 0; i < n; ++i) {
    double sum = 0.0;
    const long i7 = i * 7;
    if (i - nynz >= 0) sum += val[i7 + 0] * x[i - nynz];
    if (i - nz >= 0) sum += val[i7 + 1] * x[i - nz];
    if (i - 1 >= 0) sum += val[i7 + 2] * x[i - 1];
    sum += val[i7 + 3] * x[i];
    if (i + 1 < n) sum += val[i7 + 4] * x[i + 1];
    if (i + nz < n) sum += val[i7 + 5] * x[i + nz];
    if (i + nynz < n) sum += val[i7 + 6] * x[i + nynz];
    r[i] = sum;
  }
}

/* Jacobi-scaled CSR rows of inc/grid/structureGrid.hpp:557-654 multiplied as in
 * inc/matrix/CSR_sparseMatrix.hpp:232-243; entries in the builder's order. */
void og_csr_multiply(const og_grid *g, const double *jp, const double *x, double *r) {
  const int nx = g->nxc, ny = g->nyc, nz = g->nzc, pz = g->periodic_z != 0;
  const long nyz = (long)ny * nz;
  long row = 0;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k, ++row) {
        double aa = 0.0, bb = 0.0, cc = 0.0;
        if (i == 0) aa = -cxm(g, i);
        if (i == nx - 1) aa = -cxp(g, i);
        if (j == 0) bb = -cym(g, j);
        if (j == ny - 1) bb = -cyp(g, j);
        if (k == 0 && !pz) cc = -czm(g, k);
        if (k == nz - 1 && !pz) cc = -czp(g, k);
        const double ijk = cxm(g, i) + cym(g, j) + czm(g, k) + cxp(g, i) + cyp(g, j) +
                           czp(g, k) + aa + bb + cc;
        const double s = jp[row];
        double acc = 0.0;
        if (i != 0) acc += (-cxm(g, i) * s) * x[row - nyz];
        if (j != 0) acc += (-cym(g, j) * s) * x[row - nz];
        if (k != 0) acc += (-czm(g, k) * s) * x[row - 1];
        else if (pz) acc += (-czm(g, k) * s) * x[row + nz - 1];
        acc += (ijk * s) * x[row];
        if (k != nz - 1) acc += (-czp(g, k) * s) * x[row + 1];
        else if (pz) acc += (-czp(g, k) * s) * x[row - (nz - 1)];
        if (j != ny - 1) acc += (-cyp(g, j) * s) * x[row + nz];
        if (i != nx - 1) acc += (-cxp(g, i) * s) * x[row + nyz];
        r[row] = acc;
      }
}

/* inc/solver/math.hpp:13-36 at one thread: serial sums */
static double dot(long n, const double *a, const double *b) {
  double r = 0.0;
  for (long i = 0; i < n; ++i) r += a[i] * b[i];
  return r;
}
static double l2norm(long n, const double *a) {
  double r = 0.0;
  for (long i = 0; i < n; ++i) r += a[i] * a[i];
  return sqrt(r);
}

int og_bicg_init(og_bicg *s, const og_grid *g, int kind, double tol) {
  memset(s, 0, sizeof(*s));
  s->n = og_cells(g);
  s->iters_max = 5000;           /* bicgstabRe2.hpp:47 */
  s->tol = tol;
  s->restart_factor = 1e-7;      /* :53 */
  s->kind = kind;
  s->g = g;
  double **v[8] = {&s->r0, &s->r1, &s->p1, &s->s1, &s->ap, &s->as, &s->px1, &s->px2};
  for (int q = 0; q < 8; ++q) *v[q] = dalloc(s->n);
  if (kind == 0) {
    s->val7 = dalloc(7 * s->n);
    og_spe_setup(g, s->val7);
  } else {
    s->jp = dalloc(s->n);
    og_jacobi_scale(g, s->jp);
  }
  return 0;
}

void og_bicg_free(og_bicg *s) {
  free(s->r0); free(s->r1); free(s->p1); free(s->s1); free(s->ap); free(s->as);
  free(s->px1); free(s->px2); free(s->val7); free(s->jp);
  memset(s, 0, sizeof(*s));
}

static void apply(og_bicg *s, const double *x, double *y) {
  if (s->kind == 0) og_spe_multiply(s->g, s->val7, x, y);
  else og_csr_multiply(s->g, s->jp, x, y);
}

/* inc/solver/bicgstabRe2.hpp:84-180 (solve) */
int og_bicg_solve(og_bicg *s, const double *rhs, double *x, double *relres) {
  const long n = s->n;
  s->timestep++;
  double r1r0 = 0, r1r0l = 0, a = 0, w = 0, b = 0;
  const double norm0 = l2norm(n, rhs);
  apply(s, x, s->r0);
  memcpy(s->px2, s->px1, sizeof(double) * n);
  memcpy(s->px1, x, sizeof(double) * n);
  for (long i = 0; i < n; ++i) s->r0[i] = rhs[i] - s->r0[i];
  memcpy(s->r1, s->r0, sizeof(double) * n);
  memcpy(s->p1, s->r0, sizeof(double) * n);
  r1r0 = dot(n, s->r1, s->r0);
  int it = 0;
  for (;;) {
    apply(s, s->p1, s->ap);
    a = r1r0 / dot(n, s->ap, s->r0);
    for (long i = 0; i < n; ++i) s->s1[i] = s->r1[i] - a * s->ap[i];
    apply(s, s->s1, s->as);
    w = dot(n, s->as, s->s1) / dot(n, s->as, s->as);
    for (long i = 0; i < n; ++i) {
      x[i] += a * s->p1[i] + w * s->s1[i];
      s->r1[i] = s->s1[i] - w * s->as[i];
    }
    if ((l2norm(n, s->r1) / norm0) < s->tol) break;
    if (it >= s->iters_max) {
      long bad = 0;
      for (long i = 0; i < n; ++i)
        if (isnan(x[i]) || isinf(x[i])) { x[i] = s->px1[i]; ++bad; }
      if (bad > n * 0.1)
        for (long i = 0; i < n; ++i) x[i] = s->px2[i];
      break;
    }
    r1r0l = r1r0;
    r1r0 = dot(n, s->r1, s->r0);
    b = (a / w) * (r1r0 / r1r0l);
    if (s->timestep < 10 || fabs(r1r0l) > s->tol * s->restart_factor) {
      for (long i = 0; i < n; ++i) s->p1[i] = s->r1[i] + b * (s->p1[i] - w * s->ap[i]);
    } else {
      for (long i = 0; i < n; ++i) { s->r0[i] = s->r1[i]; s->p1[i] = s->r1[i]; }
    }
    ++it;
  }
  *relres = l2norm(n, s->r1) / norm0;
  return it;
}

/* inc/pressure/solver/SorPipeLine.omp.hpp:4-129 in one thread's (lexicographic) order;
 * the coefficient cache cf[8] of :33-49 and the stop rule of :110 */
int og_sor(const og_grid *g, double dt, double omega, double tol, int itmax,
           const double *us, const double *vs, const double *ws, double *p, double *err) {
  const long n = og_cells(g);
  double *cf = dalloc(8 * n);
  const double rdt = 1.0 / dt;
  const long sx = (long)g->ny * g->nz, sy = g->nz;
  long row = 0;
  double norm_rhs = 0.0;
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k, ++row) {
        double *c = cf + 8 * row;
        const double *Dx = g->Dx, *Dy = g->Dy, *Dz = g->Dz;
        c[0] = Dy[j] * Dz[k] / g->Dxs[i];
        c[1] = Dy[j] * Dz[k] / g->Dxs[i - 1];
        c[2] = Dx[i] * Dz[k] / g->Dys[j];
        c[3] = Dx[i] * Dz[k] / g->Dys[j - 1];
        c[4] = Dx[i] * Dy[j] / g->Dzs[k];
        c[5] = Dx[i] * Dy[j] / g->Dzs[k - 1];
        const double coef = Dy[j] * Dz[k] / g->Dxs[i] + Dy[j] * Dz[k] / g->Dxs[i - 1] +
                            Dx[i] * Dz[k] / g->Dys[j] + Dx[i] * Dz[k] / g->Dys[j - 1] +
                            Dx[i] * Dy[j] / g->Dzs[k] + Dx[i] * Dy[j] / g->Dzs[k - 1];
        c[7] = -1.0 / coef;
        const long ic = IC(g, i, j, k);
        const long zb = (g->periodic_z && k == GC) ? IC(g, i, j, g->nz - 3) : ic - 1;
        const double mChange = (us[ic] - us[ic - sx]) * Dy[j] * Dz[k] +
                               (vs[ic] - vs[ic - sy]) * Dx[i] * Dz[k] +
                               (ws[ic] - ws[zb]) * Dx[i] * Dy[j];
        c[6] = mChange * rdt;
        norm_rhs += (mChange * rdt) * (mChange * rdt);
      }
  norm_rhs = sqrt(norm_rhs);
  int it;
  double residual = 0.0;
  for (it = 0; it < itmax; ++it) {
    residual = 0;
    row = 0;
    for (int i = GC; i < g->nx - GC; ++i)
      for (int j = GC; j < g->ny - GC; ++j)
        for (int k = GC; k < g->nz - GC; ++k, ++row) {
          const long ic = IC(g, i, j, k);
          const double *c = cf + 8 * row;
          /* periodic z: the neighbours across the ends are the wrapped cells */
          const long zm = (g->periodic_z && k == GC) ? ic + g->nzc - 1 : ic - 1;
          const long zp = (g->periodic_z && k == g->nz - 3) ? ic - (g->nzc - 1) : ic + 1;
          const double pNEW = (-p[ic + sx] * c[0] - p[ic - sx] * c[1] - p[ic + sy] * c[2] -
                               p[ic - sy] * c[3] - p[zp] * c[4] - p[zm] * c[5] + c[6]) *
                              c[7];
          const double pChange = fabs(pNEW - p[ic]);
          p[ic] += omega * (pNEW - p[ic]);
          residual += pChange / norm_rhs;
        }
    if (sqrt(residual) < tol) break;
  }
  *err = sqrt(residual);
  free(cf);
  return it;
}

/* inc/pressure/Transform.hpp:8-20 */
void og_transform(const og_grid *g, const double *x, double *p) {
  long row = 0;
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k, ++row) p[IC(g, i, j, k)] = x[row];
}

/* inc/dfib/updateUandF.hpp:90-180 (update_UandF_omp); solid velocity 0 */
void og_update_uf(const og_grid *g, double dt, const double *eta, const double *p,
                  const double *us, const double *vs, const double *ws, double *u3,
                  double *v3, double *w3, double *f) {
  const long tot = og_padded(g);
  const long sx = (long)g->ny * g->nz, sy = g->nz;
  const double uS = 0.0, vS = 0.0, wS = 0.0;
  for (int i = GC; i < g->nx - GC - 1; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k) {
        const long ic = IC(g, i, j, k), icP = ic + sx;
        const double T2u = us[ic] - dt * (p[icP] - p[ic]) / g->Dxs[i];
        const double e = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dxs[i] * 0.5) / g->Dx[i]);
        u3[ic] = eta[ic] * uS + (1.0 - e) * T2u;
        f[ic] = (u3[ic] - T2u) / dt;
      }
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC - 1; ++j)
      for (int k = GC; k < g->nz - GC; ++k) {
        const long ic = IC(g, i, j, k), icP = ic + sy;
        const double T2v = vs[ic] - dt * (p[icP] - p[ic]) / g->Dys[j];
        const double e = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dys[j] * 0.5) / g->Dy[j]);
        v3[ic] = eta[ic] * vS + (1.0 - e) * T2v;
        f[ic + tot] = (v3[ic] - T2v) / dt;
      }
  /* periodic z: the top face nz-3 too, its upper cell the first one (k = 2) */
  const int pz = g->periodic_z != 0;
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC - 1 + pz; ++k) {
        const long ic = IC(g, i, j, k), icP = (pz && k == g->nz - 3) ? ic - (g->nzc - 1) : ic + 1;
        const double T2w = ws[ic] - dt * (p[icP] - p[ic]) / g->Dzs[k];
        const double e = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dzs[k] * 0.5) / g->Dz[k]);
        w3[ic] = eta[ic] * wS + (1.0 - e) * T2w;
        f[ic + 2 * tot] = (w3[ic] - T2w) / dt;
      }
}

/* inc/dfib/setEta.hpp:136-204 (DFIB_CylinderZ): 100x100 sub-sampling of the cells within
 * half a cell diagonal of the circle, then extrusion along z. */
void og_dfib_cylinder_z(const og_grid *g, double *eta) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, nsub = 100;
  const double cx = g->cx, cy = g->cy, R = g->radius;
  double sdx[101], sdy[101];
  for (int i = GC; i < nx - GC; ++i)
    for (int j = GC; j < ny - GC; ++j) {
      const long icel = IC(g, i, j, 0);
      const double Diagonal = sqrt(g->Dx[i] * g->Dx[i] + g->Dy[j] * g->Dy[j]) * 0.5;
      const double ddx = ((g->X[i] + g->X[i + 1]) * 0.5) - cx;
      const double ddy = ((g->Y[j] + g->Y[j + 1]) * 0.5) - cy;
      const double Distance = sqrt(ddx * ddx + ddy * ddy);
      if (fabs(Distance - R) < Diagonal) {
        long xi = 0;
        const double dyg = g->Dy[j] / (double)nsub;
        const double dxg = g->Dx[i] / (double)nsub;
        for (int q = 0; q < nsub + 1; ++q) {
          sdy[q] = g->Y[j] + (double)q * dyg;
          sdx[q] = g->X[i] + (double)q * dxg;
        }
        for (int ii = 0; ii < nsub; ++ii)
          for (int jj = 0; jj < nsub; ++jj) {
            const double a = (sdx[ii] + sdx[ii + 1]) * 0.5 - cx;
            const double b = (sdy[jj] + sdy[jj + 1]) * 0.5 - cy;
            if (sqrt(a * a + b * b) <= R) ++xi;
          }
        eta[icel] = (double)xi * (1.0 / ((double)nsub * (double)nsub));
      } else if (Distance > R) {
        eta[icel] = 0.;
      } else {
        eta[icel] = 1.;
      }
    }
  for (int i = 0; i < nx - 1; ++i)
    for (int j = 0; j < ny - 1; ++j)
      for (int k = 1; k < nz - 1; ++k) eta[IC(g, i, j, k)] = eta[IC(g, i, j, 0)];
}

/* inc/dfib/virtualForceIntergrator.hpp:67-90 (virtualF_Int) */
double og_force_sum(const og_grid *g, const double *f, int dir) {
  const long tot = og_padded(g);
  double s = 0.0;
  for (int i = GC; i < g->nx - GC; ++i)
    for (int j = GC; j < g->ny - GC; ++j)
      for (int k = GC; k < g->nz - GC; ++k)
        s += f[IC(g, i, j, k) + tot * dir] * (g->Dx[i] * g->Dy[j] * g->Dz[k]);
  return s;
}

int og_run(const og_grid *g, int steps, double Re, double dt, double tol, int solver,
           double omega, double *u, double *v, double *w, double *p, double *eta,
           double *stats) {
  return og_run_ex(g, steps, Re, dt, tol, solver, omega, u, v, w, p, eta, stats, NULL, NULL, 0);
}

void og_cfl(const og_grid *g, double dt, const double *us, const double *vs, const double *ws,
            double *out7) {
  const long n = og_cells(g);
  double *c = dalloc(n);
  double umax[3] = {-1e10, -1e10, -1e10}, umin[3] = {1e10, 1e10, 1e10};
  const double *f[3] = {us, vs, ws};
  const double *Ds[3] = {g->Dxs, g->Dys, g->Dzs};
  /* cfl.hpp:20-63: one loop per component over the interior, the last face of its axis
   * excluded, in the reference's i-j-k order */
  for (int a = 0; a < 3; ++a)
    for (int i = GC; i < g->nx - GC - (a == 0); ++i)
      for (int j = GC; j < g->ny - GC - (a == 1); ++j)
        for (int k = GC; k < g->nz - GC - (a == 2 && !g->periodic_z); ++k) {
          const long ic = IC(g, i, j, k);
          const long r = ((long)(i - GC) * g->nyc + (j - GC)) * g->nzc + (k - GC);
          const int d = a == 0 ? i : (a == 1 ? j : k);
          c[r] += f[a][ic] / Ds[a][d];
          if (f[a][ic] > umax[a]) umax[a] = f[a][ic];
          if (f[a][ic] < umin[a]) umin[a] = f[a][ic];
        }
  double m = c[0];
  for (long r = 1; r < n; ++r)
    if (c[r] > m) m = c[r];
  out7[0] = m * dt; /* cfl.hpp:67-68 */
  for (int a = 0; a < 3; ++a) {
    out7[1 + a] = umax[a];
    out7[4 + a] = umin[a];
  }
  free(c);
}

static void put_header(FILE *f, const og_grid *g) {
  const int h[4] = {1, g->nxc, g->nyc, g->nzc};
  fwrite(h, sizeof(int), 4, f);
}

int og_plot3d_x(const og_grid *g, const char *path) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  put_header(f, g);
  /* xfileWrite.hpp:14-47: cell centres Xc[i] = (X[i+gC] + X[i+gC+1]) / 2 (structureGrid.hpp:219) */
  const double *N[3] = {g->X, g->Y, g->Z};
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < g->nzc; ++k)
      for (int j = 0; j < g->nyc; ++j)
        for (int i = 0; i < g->nxc; ++i) {
          const int q = a == 0 ? i : (a == 1 ? j : k);
          const float v = (float)((N[a][q + GC] + N[a][q + GC + 1]) / 2.0);
          fwrite(&v, sizeof(float), 1, f);
        }
  fclose(f);
  return 0;
}

int og_plot3d_q(const og_grid *g, const double *p, const double *u, const double *v, const double *w,
                const double *eta, double Re, double time, const char *path) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  put_header(f, g);
  const float hdr[4] = {0.0f, 0.0f, (float)Re, (float)time};  /* qfile.hpp:22-25 */
  fwrite(hdr, sizeof(float), 4, f);
  const long sx = (long)g->ny * g->nz, sy = g->nz;
  for (int a = 0; a < 5; ++a)
    for (int k = GC; k < g->nzc + GC; ++k)
      for (int j = GC; j < g->nyc + GC; ++j)
        for (int i = GC; i < g->nxc + GC; ++i) {
          const long ic = IC(g, i, j, k);
          float o;
          switch (a) {
            case 0: o = (float)p[ic]; break;
            case 1: o = (float)(0.5 * (u[ic - sx] + u[ic])); break;
            case 2: o = (float)(0.5 * (v[ic - sy] + v[ic])); break;
            case 3: o = (float)(0.5 * (w[ic - 1] + w[ic])); break;
            default: o = (float)eta[ic]; break;
          }
          fwrite(&o, sizeof(float), 1, f);
        }
  fclose(f);
  return 0;
}

int og_plot3d_read(const og_grid *g, const char *path, double head[5], double *p, double *u, double *v, double *w,
                   double *eta) {
  /* QfileRead (inc/io/Plot3D/qfileRead.hpp:6-106): the header, five float32 arrays in
   * k-j-i order; p and eta go to the interior cells as they are, u, v, w back to faces as
   * the float sum of the two cells beside the face, halved in double (:87-97), the last
   * face of each axis taking its cell's value.  Everything else stays 0. */
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  int ih[4];
  float fh[4];
  const long n = og_cells(g);
  float *q = (float *)malloc(sizeof(float) * 5 * (size_t)n);
  int ok = q && fread(ih, sizeof(int), 4, f) == 4 && fread(fh, sizeof(float), 4, f) == 4 &&
           ih[1] == g->nxc && ih[2] == g->nyc && ih[3] == g->nzc;
  if (ok) ok = fread(q, sizeof(float), 5 * (size_t)n, f) == 5 * (size_t)n;
  fclose(f);
  if (!ok) {
    free(q);
    return -1;
  }
  head[0] = ih[0];
  for (int a = 0; a < 4; ++a) head[1 + a] = fh[a];
  const long np = og_padded(g);
  double *o[5] = {p, u, v, w, eta};
  for (int a = 0; a < 5; ++a) memset(o[a], 0, sizeof(double) * (size_t)np);
  /* file index of compact (i, j, k) and its neighbours along each axis */
#define QF(a, i, j, k) q[(long)(a) * n + (i) + (long)g->nxc * ((j) + (long)g->nyc * (k))]
  for (int k = 0; k < g->nzc; ++k)
    for (int j = 0; j < g->nyc; ++j)
      for (int i = 0; i < g->nxc; ++i) {
        const long c = IC(g, i + GC, j + GC, k + GC);
        p[c] = QF(0, i, j, k);
        eta[c] = QF(4, i, j, k);
        u[c] = i == g->nxc - 1 ? (double)QF(1, i, j, k) : (float)(QF(1, i, j, k) + QF(1, i + 1, j, k)) / 2.0;
        v[c] = j == g->nyc - 1 ? (double)QF(2, i, j, k) : (float)(QF(2, i, j, k) + QF(2, i, j + 1, k)) / 2.0;
        w[c] = k == g->nzc - 1 ? (double)QF(3, i, j, k) : (float)(QF(3, i, j, k) + QF(3, i, j, k + 1)) / 2.0;
      }
#undef QF
  free(q);
  return 0;
}

int og_cg_solve(const og_grid *g, const double *val7, const double *rhs, double *x, double tol, int maxit,
                double *relres) {
  const long n = og_cells(g);
  double *r = dalloc(n), *p = dalloc(n), *q = dalloc(n);
  og_spe_multiply(g, val7, x, q);
  double bb = 0.0, rr = 0.0;
  for (long i = 0; i < n; ++i) {
    r[i] = rhs[i] - q[i];
    p[i] = r[i];
    bb += rhs[i] * rhs[i];
    rr += r[i] * r[i];
  }
  const double norm0 = sqrt(bb);
  double rel = sqrt(rr) / norm0;
  int it = 0;
  while (rel >= tol && it < maxit) {
    og_spe_multiply(g, val7, p, q);
    double pq = 0.0;
    for (long i = 0; i < n; ++i) pq += p[i] * q[i];
    const double a = rr / pq;
    double rn = 0.0;
    for (long i = 0; i < n; ++i) {
      x[i] += a * p[i];
      r[i] -= a * q[i];
      rn += r[i] * r[i];
    }
    ++it;
    rel = sqrt(rn) / norm0;
    if (rel < tol) break;
    const double be = rn / rr;
    rr = rn;
    for (long i = 0; i < n; ++i) p[i] = r[i] + be * p[i];
  }
  free(r); free(p); free(q);
  if (relres) *relres = rel;
  return it;
}

void og_project_rhs(const og_grid *g, const double *jp, double *b) {
  const long n = og_cells(g);
  double sum = 0.0;
  for (long r = 0; r < n; ++r) sum += jp ? b[r] / jp[r] : b[r];
  const double m = sum / (double)n;
  for (long r = 0; r < n; ++r) b[r] -= jp ? m * jp[r] : m;
}

int og_run_ex(const og_grid *g, int steps, double Re, double dt, double tol, int solver,
              double omega, double *u, double *v, double *w, double *p, double *eta,
              double *stats, const double *eta_in, const double *inlet, int project) {
  const long tot = og_padded(g), n = og_cells(g);
  const double nu = 1.0 / Re; /* 0_1_SimulationVariable.hpp:26-31 */
  double *us = dalloc(tot), *vs = dalloc(tot), *ws = dalloc(tot);
  double *u3 = dalloc(tot), *v3 = dalloc(tot), *w3 = dalloc(tot);
  double *f = dalloc(3 * tot), *b = dalloc(n), *x = dalloc(n);
  og_bicg bs;
  int rc = 0;
  /* src/RUN_CPU.cpp:104-109 */
  memcpy(us, u, sizeof(double) * tot); memcpy(u3, u, sizeof(double) * tot);
  memcpy(vs, v, sizeof(double) * tot); memcpy(v3, v, sizeof(double) * tot);
  memcpy(ws, w, sizeof(double) * tot); memcpy(w3, w, sizeof(double) * tot);
  bc_main_in(g, u, v, w, p, inlet, NULL, NULL, NULL, dt);
  og_bc_copy(g, u, v, w, us, vs, ws);
  if (solver == 0 || solver == 1) og_bicg_init(&bs, g, solver, tol);
  double *val7 = solver == 3 ? dalloc(7 * n) : NULL;
  if (val7) og_spe_setup(g, val7);
  if (eta_in) {
    memcpy(eta, eta_in, sizeof(double) * tot);
  } else {
    memset(eta, 0, sizeof(double) * tot);
    og_dfib_cylinder_z(g, eta);
  }
  double *nut = g->les ? dalloc(n) : NULL;
  /* Adams-Bashforth history (time_order 2, 3): increments of the last two steps, slots
   * hs[0], hs[1] swapping roles each step */
  const int order = g->time_order > 1 ? g->time_order : 1;
  double *hs[2][3] = {{NULL, NULL, NULL}, {NULL, NULL, NULL}};
  if (order > 1)
    for (int q = 0; q < 2; ++q)
      for (int c = 0; c < 3; ++c) hs[q][c] = dalloc(tot);
  int nhist = 0, slot = 0;
  for (int s = 1; s <= steps; ++s) {
    if (nut) og_smagorinsky(g, u, v, w, nut); /* RUN_CPU.cpp:261-263, on T0 */
    if (order > 1) {
      og_ab ab;
      ab.order = nhist + 1 < order ? nhist + 1 : order;
      ab.r = 1.0; /* constant dt here */
      for (int c = 0; c < 3; ++c) {
        ab.h1[c] = hs[slot][c];
        ab.h2[c] = hs[1 - slot][c];
        ab.hnew[c] = order == 2 ? hs[slot][c] : hs[1 - slot][c];
      }
      og_convection_diffusion_ab(g, dt, nu, nut, &ab, u, v, w, us, vs, ws);
      if (nhist < 2) ++nhist;
      if (order == 3) slot = 1 - slot;
    } else {
      og_convection_diffusion_ex(g, dt, nu, nut, u, v, w, us, vs, ws);
    }
    int iters = 0;
    double err = 0.0;
    if (s > 1) { /* RUN_CPU.cpp:287/:303: no pressure solve at the first step */
      if (solver == 2) {
        iters = og_sor(g, dt, omega, tol, 5000, us, vs, ws, p, &err);
      } else if (solver == 3) {
        og_rhs(g, dt, us, vs, ws, NULL, b);
        if (project) og_project_rhs(g, NULL, b);
        iters = og_cg_solve(g, val7, b, x, tol, 5000, &err);
        og_transform(g, x, p);
      } else {
        og_rhs(g, dt, us, vs, ws, solver == 1 ? bs.jp : NULL, b);
        if (project) og_project_rhs(g, solver == 1 ? bs.jp : NULL, b);
        iters = og_bicg_solve(&bs, b, x, &err);
        og_transform(g, x, p);
      }
    }
    og_update_uf(g, dt, eta, p, us, vs, ws, u3, v3, w3, f);
    memcpy(u, u3, sizeof(double) * tot); /* copyVel */
    memcpy(v, v3, sizeof(double) * tot);
    memcpy(w, w3, sizeof(double) * tot);
    bc_main_in(g, u, v, w, p, inlet, us, vs, ws, dt);
    og_bc_copy(g, u, v, w, us, vs, ws);
    if (stats) {
      stats[4 * (s - 1) + 0] = iters;
      stats[4 * (s - 1) + 1] = err;
      stats[4 * (s - 1) + 2] = -2.0 * og_force_sum(g, f, 0) / g->lz;
      stats[4 * (s - 1) + 3] = -2.0 * og_force_sum(g, f, 1) / g->lz;
    }
  }
  if (solver == 0 || solver == 1) og_bicg_free(&bs);
  free(val7);
  free(nut);
  for (int q = 0; q < 2; ++q)
    for (int c = 0; c < 3; ++c) free(hs[q][c]);
  free(us); free(vs); free(ws); free(u3); free(v3); free(w3); free(f); free(b); free(x);
  return rc;
}
