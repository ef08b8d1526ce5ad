/* ms_nk.c -- the minimal-surface solve of c/ch7/minimal.c by the method of
 * the GPU library, restated on the CPU in FP64 with OpenMP (TEST
 * INFRASTRUCTURE: bench.py's CPU baseline of the minimal-surface leg; the
 * GPU library never calls it).
 *
 *   - Newton with PETSc's cubic backtracking line search on ||F||^2/2
 *     (SNESLINESEARCHBT defaults, Dennis & Schnabel A6.3.1) and the
 *     SNESConvergedDefault tests (rtol, atol 1e-50, stol 1e-8, 50 steps), as
 *     tests/_ms_oracle.py restates them;
 *   - each step J Y = F solved by BiCGStab from Y = 0 to a relative residual
 *     of ksp_rtol (minimal.c's -ksp_rtol, default 1e-5), right-preconditioned
 *     with one V-cycle of the Poisson multigrid of the fish oracle (the
 *     preconditioning matrix of minimal.c:142-145, Chebyshev/Jacobi
 *     smoothing, levels down to 3 x 3), boundary rows passed through;
 *   - J applied from its nine row weights, formed once per Newton step;
 *   - grid sequencing: the solution interpolated (Q1) onto the next grid.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fish_oracle.h"
#include "minimal_oracle.h"

typedef struct {
  int ngrids;
  int m[16];
  int its[16];
  int reason[16];
  long long ksp_its;
  double errinf;      /* catenoid, q = -1/2: max |u - g| on the last grid; else -1 */
  double fnorm_last;  /* ||F|| of the last grid's solution */
} ms_nk_report;

static double dot(long n, const double *a, const double *b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long q = 0; q < n; q++) s += a[q] * b[q];
  return s;
}

static void jv9(const ms_grid *g, const double *w, const double *v, double *out) {
  const int mx = g->mx, my = g->my;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const long n = (long)j * mx + i;
      const double *wn = w + 9 * n;
      if (i == 0 || j == 0 || i == mx - 1 || j == my - 1) {
        out[n] = v[n];
        continue;
      }
      double s = 0.0;
      for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++) s += wn[(dj + 1) * 3 + di + 1] * v[n + (long)dj * mx + di];
      out[n] = s;
    }
}

/* z = B r: the Poisson V-cycle on the interior, boundary rows passed through */
static void precond(const ms_grid *g, void *mg, const double *r, double *z) {
  or_mg_apply(mg, r, z);
  const int mx = g->mx, my = g->my;
  for (int i = 0; i < mx; i++) {
    z[i] = r[i];
    z[(long)(my - 1) * mx + i] = r[(long)(my - 1) * mx + i];
  }
  for (int j = 0; j < my; j++) {
    z[(long)j * mx] = r[(long)j * mx];
    z[(long)j * mx + mx - 1] = r[(long)j * mx + mx - 1];
  }
}

/* BiCGStab, right preconditioning, x = 0 start; returns the iterations */
static int bicgstab(const ms_grid *g, const double *w, void *mg, const double *b, double *x, double rtol, int maxit,
                    double *work) {
  const long N = (long)g->mx * g->my;
  double *r = work, *rh = r + N, *p = rh + N, *v = p + N, *s = v + N, *t = s + N, *ph = t + N, *sh = ph + N;
  memset(x, 0, sizeof(double) * N);
  memcpy(r, b, sizeof(double) * N);
  memcpy(rh, b, sizeof(double) * N);
  memset(p, 0, sizeof(double) * N);
  memset(v, 0, sizeof(double) * N);
  const double bn = sqrt(dot(N, b, b));
  if (bn == 0.0) return 0;
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= maxit; it++) {
    const double rhon = dot(N, rh, r);
    const double beta = (rhon / rho) * (alpha / omega);
    rho = rhon;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) p[q] = r[q] + beta * (p[q] - omega * v[q]);
    precond(g, mg, p, ph);
    jv9(g, w, ph, v);
    alpha = rho / dot(N, rh, v);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) s[q] = r[q] - alpha * v[q];
    if (sqrt(dot(N, s, s)) <= rtol * bn) {
#pragma omp parallel for schedule(static)
      for (long q = 0; q < N; q++) x[q] += alpha * ph[q];
      return it;
    }
    precond(g, mg, s, sh);
    jv9(g, w, sh, t);
    omega = dot(N, t, s) / dot(N, t, t);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) {
      x[q] += alpha * ph[q] + omega * sh[q];
      r[q] = s[q] - omega * t[q];
    }
    if (sqrt(dot(N, r, r)) <= rtol * bn) return it;
  }
  return maxit;
}

/* cubic backtracking along X - lambda Y; 1 on success (X, F, fnorm updated) */
static int line_search(const ms_grid *g, double *X, double *F, double *fnorm, double *Y, const double *w, double *W,
                       double *G, double *JY, double *ynorm_out) {
  const long N = (long)g->mx * g->my;
  const double alpha = 1e-4, maxstep = 1e8, minlambda = 1e-12;
  double ynorm = sqrt(dot(N, Y, Y));
  if (ynorm > maxstep) {
    for (long q = 0; q < N; q++) Y[q] *= maxstep / ynorm;
    ynorm = maxstep;
  }
  jv9(g, w, Y, JY);
  double initslope = dot(N, F, JY);
  if (initslope > 0.0) initslope = -initslope;
  if (initslope == 0.0) initslope = -1.0;
  const double f0 = *fnorm;
  double lam = 1.0, lamprev = 1.0, gprev = 0.0;
  for (int it = 0; it <= 40; it++) {
    if (it > 0 && lam < minlambda) return 0;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) W[q] = X[q] - lam * Y[q];
    ms_residual(g, W, G);
    const double gnorm = sqrt(dot(N, G, G));
    if (0.5 * gnorm * gnorm <= 0.5 * f0 * f0 + lam * alpha * initslope) {
      memcpy(X, W, sizeof(double) * N);
      memcpy(F, G, sizeof(double) * N);
      *fnorm = gnorm;
      *ynorm_out = lam * ynorm;
      return 1;
    }
    double lamtemp;
    if (it == 0) {
      lamtemp = -initslope / (gnorm * gnorm - f0 * f0 - 2.0 * lam * initslope);
    } else {
      const double t1 = 0.5 * (gnorm * gnorm - f0 * f0) - lam * initslope;
      const double t2 = 0.5 * (gprev * gprev - f0 * f0) - lamprev * initslope;
      const double a = (t1 / (lam * lam) - t2 / (lamprev * lamprev)) / (lam - lamprev);
      const double b = (-lamprev * t1 / (lam * lam) + lam * t2 / (lamprev * lamprev)) / (lam - lamprev);
      const double d = fmax(b * b - 3.0 * a * initslope, 0.0);
      lamtemp = a == 0.0 ? -initslope / (2.0 * b) : (-b + sqrt(d)) / (3.0 * a);
    }
    lamprev = lam;
    gprev = gnorm;
    lam = lamtemp > 0.5 * lam ? 0.5 * lam : (lamtemp <= 0.1 * lam ? 0.1 * lam : lamtemp);
  }
  return 0;
}

static int levels_to_3(int m) {
  int l = 1;
  while (m > 3 && (m - 1) % 2 == 0) {
    m = (m - 1) / 2 + 1;
    l++;
  }
  return l;
}

int ms_nk_solve(const ms_grid *g0, int grid_sequence, double rtol, double ksp_rtol, double *u_out, ms_nk_report *rep) {
  memset(rep, 0, sizeof(*rep));
  if (grid_sequence < 0 || grid_sequence > 15) return -1;
  ms_grid g = *g0;
  long N = (long)g.mx * g.my;
  double *X = (double *)malloc(sizeof(double) * N);
  if (!X) return -2;
  ms_initial(&g, X);
  int rc = 0;
  for (int lev = 0; lev <= grid_sequence && !rc; lev++) {
    N = (long)g.mx * g.my;
    double *F = malloc(sizeof(double) * N), *Y = malloc(sizeof(double) * N), *W = malloc(sizeof(double) * N);
    double *G = malloc(sizeof(double) * N), *JY = malloc(sizeof(double) * N), *w = malloc(sizeof(double) * 9 * N);
    double *work = malloc(sizeof(double) * 8 * N);
    or_opts o;
    or_opts_default(&o);
    o.grid.dim = 2;
    o.grid.mx = g.mx;
    o.grid.my = g.my;
    o.grid.mz = 1;
    o.grid.Lx = o.grid.Ly = o.grid.Lz = 1.0;
    o.grid.cx = o.grid.cy = o.grid.cz = 1.0;
    o.grid.problem = OR_ZERO;
    o.pc_type = OR_PC_MG;
    o.smooth_type = OR_SMOOTH_CHEBYSHEV;
    o.smooth_its = 2;
    o.mg_levels = levels_to_3(g.mx);
    o.mg_cycles = 1;
    void *mg = or_mg_new(&o);
    if (!F || !Y || !W || !G || !JY || !w || !work || !mg) rc = -2;
    if (!rc) {
      ms_residual(&g, X, F);
      double fnorm = sqrt(dot(N, F, F));
      const double ttol = rtol * fnorm;
      int reason = 0, its = 0;
      if (isnan(fnorm)) reason = -4;
      else if (fnorm < 1e-50) reason = 2;
      while (!reason) {
        ms_row_weights(&g, X, w);
        rep->ksp_its += bicgstab(&g, w, mg, F, Y, ksp_rtol, 10000, work);
        double ynorm = 0.0;
        const int ok = line_search(&g, X, F, &fnorm, Y, w, W, G, JY, &ynorm);
        its++;
        if (!ok) {
          reason = -6;
          break;
        }
        const double xnorm = sqrt(dot(N, X, X));
        if (isnan(fnorm)) reason = -4;
        else if (fnorm < 1e-50) reason = 2;
        else if (fnorm <= ttol) reason = 3;
        else if (ynorm < 1e-8 * xnorm) reason = 4;
        else if (its >= 50) reason = -5;
      }
      rep->m[lev] = g.mx;
      rep->its[lev] = its;
      rep->reason[lev] = reason;
      rep->fnorm_last = fnorm;
      rep->ngrids = lev + 1;
      if (reason < 0) rc = -3;
    }
    or_mg_free(mg);
    free(F); free(Y); free(W); free(G); free(JY); free(w); free(work);
    if (!rc && lev < grid_sequence) {
      ms_grid gf = g;
      gf.mx = 2 * g.mx - 1;
      gf.my = 2 * g.my - 1;
      double *Xf = (double *)malloc(sizeof(double) * (long)gf.mx * gf.my);
      if (!Xf) {
        rc = -2;
        break;
      }
      ms_interpolate(&g, X, &gf, Xf);
      free(X);
      X = Xf;
      g = gf;
    }
  }
  rep->errinf = -1.0;
  if (!rc && g.problem == MS_CATENOID && g.q == -0.5) {
    N = (long)g.mx * g.my;
    double *E = (double *)malloc(sizeof(double) * N);
    ms_exact(&g, E);
    double e = 0.0;
    for (long q = 0; q < N; q++) e = fmax(e, fabs(X[q] - E[q]));
    rep->errinf = e;
    free(E);
  }
  if (u_out && !rc) memcpy(u_out, X, sizeof(double) * (long)g.mx * g.my);
  free(X);
  return rc;
}
