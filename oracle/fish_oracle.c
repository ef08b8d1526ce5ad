/*
 * fish_oracle.c -- CPU restatement of the fish.c / poissonfunctions.c path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Nothing in the GPU library links,
 * loads or calls this file.  Every function names the reference lines it
 * restates (paths inside bueler/p4pdes).  Loops are OpenMP-parallel so the
 * same code serves as the timed CPU baseline; dot products are reduced in a
 * fixed order (per line/plane partials summed serially) so results do not
 * depend on the thread count.
 *
 * PETSc solver semantics restated here (PETSc is not in the reference tree;
 * these follow PETSc's documented algorithms for the options fish uses):
 *   - SNESKSPONLY: one linear solve J y = F(u0) from y = 0, then u = u0 - y.
 *   - KSPCG, preconditioned (default) or unpreconditioned norm; converged when
 *     ||r_k|| <= max(rtol*||r_0||, atol); diverged when ||r_k|| >= dtol*||r_0||;
 *     iteration cap max_it; beta == 0 stops as converged-atol.
 *   - PCMG multiplicative cycles on the DMDA hierarchy (m_c = (m_f-1)/2+1),
 *     rediscretised level operators, Q1 interpolation P, restriction P^T,
 *     exact coarse solve, pre- and post-smoothing with the same smoother
 *     (nonzero initial guess), V (1 recursion) or W (2 recursions).
 *   - KSPCHEBYSHEV (first kind) with PCJACOBI on the interval [emin,emax]
 *     of D^{-1}A, `its` iterations; KSPRICHARDSON with PCJACOBI.
 *   - PCILU level 0, natural ordering (used only to replay fish.test runs
 *     that rely on PETSc's one-rank default preconditioner).
 *   Eigenvalue bounds: PETSc estimates lambda_max(D^{-1}A) with a short
 *   Krylov run; this restatement uses the exact lambda_max of the
 *   Jacobi-scaled constant-coefficient stencil (closed form below) with the
 *   same default transform emin = 0.1*lmax, emax = 1.1*lmax.
 */
#include "fish_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(g, i, j, k) ((((size_t)(k)) * (size_t)(g)->my + (size_t)(j)) * (size_t)(g)->mx + (size_t)(i))

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

long long or_nodes(const or_grid *g) { return (long long)g->mx * g->my * g->mz; }

void or_spacing(const or_grid *g, double h[3]) {
  /* DMDASetUniformCoordinates(0,Lx,0,Ly,0,Lz) then h = L/(m-1):
     poissonfunctions.c:34-36, :72-75, fish.c:220 */
  h[0] = g->Lx / (g->mx - 1);
  h[1] = g->dim >= 2 ? g->Ly / (g->my - 1) : 1.0;
  h[2] = g->dim >= 3 ? g->Lz / (g->mz - 1) : 1.0;
}

/* ---- problem functions: fish.c:15-82, tables fish.c:115-123 ---- */

double or_gfun(const or_grid *g, double x, double y, double z) {
  switch (g->problem) {
  case OR_MANUPOLY:
    if (g->dim == 1) return x * x * (1.0 - x * x);                      /* fish.c:15-17 */
    if (g->dim == 2) return x * x * (1.0 - x * x) * y * y * (y * y - 1.0); /* :19-21 */
    return x * x * (1.0 - x * x) * y * y * (y * y - 1.0) * z * z * (z * z - 1.0); /* :23-25 */
  case OR_MANUEXP:
    if (g->dim == 1) return -exp(x);      /* fish.c:27-29 */
    if (g->dim == 2) return -x * exp(y);  /* :31-33 */
    return -x * exp(y + z);               /* :35-37 */
  default:
    return 0.0;                           /* fish.c:39-41 */
  }
}

double or_ffun(const or_grid *g, double x, double y, double z) {
  switch (g->problem) {
  case OR_MANUPOLY:
    if (g->dim == 1) return g->cx * 12.0 * x * x - 2.0; /* fish.c:45-48 */
    {
      double aa = x * x * (1.0 - x * x), bb = y * y * (y * y - 1.0);
      double ddaa = 2.0 * (1.0 - 6.0 * x * x), ddbb = 2.0 * (6.0 * y * y - 1.0);
      if (g->dim == 2) return -(g->cx * ddaa * bb + g->cy * aa * ddbb); /* :50-58 */
      double cc = z * z * (z * z - 1.0), ddcc = 2.0 * (6.0 * z * z - 1.0);
      return -(g->cx * ddaa * bb * cc + g->cy * aa * ddbb * cc + g->cz * aa * bb * ddcc); /* :60-70 */
    }
  case OR_MANUEXP:
    if (g->dim == 1) return exp(x);          /* fish.c:72-74 */
    if (g->dim == 2) return x * exp(y);      /* :76-78 */
    return 2.0 * x * exp(y + z);             /* :80-82 */
  default:
    return 0.0;
  }
}

static inline double gval(const or_grid *g, int i, int j, int k, const double h[3]) {
  if (g->problem == OR_USER) return g->g_user[IDX(g, i, j, k)];
  return or_gfun(g, i * h[0], j * h[1], k * h[2]);
}
static inline double fval(const or_grid *g, int i, int j, int k, const double h[3]) {
  if (g->problem == OR_USER) return g->f_user[IDX(g, i, j, k)];
  return or_ffun(g, i * h[0], j * h[1], k * h[2]);
}

/* stencil weights: sc[d] = c_d * vol / h_d^2, scdiag = 2*sum(sc), vol = prod h.
   1D: poissonfunctions.c:122-131 (cx/h, 2cx/h); 2D: :35-40; 3D: :76-82 */
static void weights(const or_grid *g, double sc[3], double *scdiag, double *vol) {
  double h[3];
  or_spacing(g, h);
  if (g->dim == 1) {
    sc[0] = g->cx / h[0]; sc[1] = sc[2] = 0.0;
    *vol = h[0];
    *scdiag = g->cx * (2.0 / h[0]);
  } else if (g->dim == 2) {
    sc[0] = g->cx * h[1] / h[0]; sc[1] = g->cy * h[0] / h[1]; sc[2] = 0.0;
    *vol = h[0] * h[1];
    *scdiag = 2.0 * (sc[0] + sc[1]);
  } else {
    double dvol = h[0] * h[1] * h[2];
    sc[0] = g->cx * dvol / (h[0] * h[0]);
    sc[1] = g->cy * dvol / (h[1] * h[1]);
    sc[2] = g->cz * dvol / (h[2] * h[2]);
    *vol = dvol;
    *scdiag = 2.0 * (sc[0] + sc[1] + sc[2]);
  }
}

static inline int is_bdry(const or_grid *g, int i, int j, int k) {
  if (i == 0 || i == g->mx - 1) return 1;
  if (g->dim >= 2 && (j == 0 || j == g->my - 1)) return 1;
  if (g->dim >= 3 && (k == 0 || k == g->mz - 1)) return 1;
  return 0;
}

/* ---- residual: Poisson{1,2,3}DFunctionLocal, poissonfunctions.c:4-115 ---- */
void or_residual(const or_grid *g, const double *u, double *F) {
  double h[3], sc[3], scdiag, vol;
  or_spacing(g, h);
  weights(g, sc, &scdiag, &vol);
  const int mx = g->mx, my = g->my, mz = g->mz, dim = g->dim;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < mz; k++) {
    for (int j = 0; j < my; j++) {
      for (int i = 0; i < mx; i++) {
        size_t n = IDX(g, i, j, k);
        if (is_bdry(g, i, j, k)) {
          /* 1D :10-12, 2D :43-47, 3D :86-91 */
          if (dim == 1) {
            F[n] = u[n] - gval(g, i, j, k, h);
            F[n] *= g->cx * (2.0 / h[0]);
          } else {
            F[n] = u[n] - gval(g, i, j, k, h);
            F[n] *= scdiag;
          }
          continue;
        }
        /* neighbours on the boundary read g there: 1D :14-17, 2D :48-56, 3D :92-104 */
        double ue = (i + 1 == mx - 1) ? gval(g, i + 1, j, k, h) : u[n + 1];
        double uw = (i - 1 == 0) ? gval(g, i - 1, j, k, h) : u[n - 1];
        if (dim == 1) {
          F[n] = g->cx * (2.0 * u[n] - uw - ue) / h[0] - h[0] * fval(g, i, j, k, h); /* :18-19 */
          continue;
        }
        size_t sy = (size_t)mx;
        double un = (j + 1 == my - 1) ? gval(g, i, j + 1, k, h) : u[n + sy];
        double us = (j - 1 == 0) ? gval(g, i, j - 1, k, h) : u[n - sy];
        if (dim == 2) {
          F[n] = scdiag * u[n] - sc[0] * (uw + ue) - sc[1] * (us + un)
                 - vol * fval(g, i, j, k, h); /* :57-59 */
          continue;
        }
        size_t sz = (size_t)mx * my;
        double uu = (k + 1 == mz - 1) ? gval(g, i, j, k + 1, h) : u[n + sz];
        double ud = (k - 1 == 0) ? gval(g, i, j, k - 1, h) : u[n - sz];
        F[n] = scdiag * u[n] - sc[0] * (uw + ue) - sc[1] * (us + un) - sc[2] * (uu + ud)
               - vol * fval(g, i, j, k, h); /* :104-106 */
      }
    }
  }
}

/* ---- Jacobian, matrix-free: Poisson{1,2,3}DJacobianLocal, poissonfunctions.c:117-258.
   Boundary rows: scdiag on the diagonal only.  Interior rows: scdiag, and -sc_d for
   each neighbour that is NOT a boundary node (boundary columns eliminated). ---- */
void or_apply(const or_grid *g, const double *p, double *q) {
  double sc[3], scdiag, vol;
  weights(g, sc, &scdiag, &vol);
  const int mx = g->mx, my = g->my, mz = g->mz, dim = g->dim;
  const size_t sy = (size_t)mx, sz = (size_t)mx * my;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < mz; k++) {
    for (int j = 0; j < my; j++) {
      for (int i = 0; i < mx; i++) {
        size_t n = IDX(g, i, j, k);
        double v = scdiag * p[n];
        if (!is_bdry(g, i, j, k)) {
          double sx = 0.0;
          if (i - 1 > 0) sx += p[n - 1];
          if (i + 1 < mx - 1) sx += p[n + 1];
          v -= sc[0] * sx;
          if (dim >= 2) {
            double s2 = 0.0;
            if (j - 1 > 0) s2 += p[n - sy];
            if (j + 1 < my - 1) s2 += p[n + sy];
            v -= sc[1] * s2;
          }
          if (dim >= 3) {
            double s3 = 0.0;
            if (k - 1 > 0) s3 += p[n - sz];
            if (k + 1 < mz - 1) s3 += p[n + sz];
            v -= sc[2] * s3;
          }
        }
        q[n] = v;
      }
    }
  }
}

/* ---- Form{1,2,3}DUExact: fish.c:288-340 ---- */
void or_exact_fill(const or_grid *g, double *u) {
  double h[3];
  or_spacing(g, h);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < g->mz; k++)
    for (int j = 0; j < g->my; j++)
      for (int i = 0; i < g->mx; i++) u[IDX(g, i, j, k)] = gval(g, i, j, k, h);
}

/* splitmix64: the build's own generator for -fsh_initial_type random
   (PETSc's PetscRandom stream is not reproducible here) */
static inline unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

/* ---- InitialState: poissonfunctions.c:260-346 ---- */
void or_initial_state(const or_grid *g, int type, int gbdry, unsigned long long seed, double *u) {
  double h[3];
  or_spacing(g, h);
  long long N = or_nodes(g);
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++)
    u[n] = type == 1 ? (double)(splitmix64(seed ^ (unsigned long long)n) >> 11) * 0x1.0p-53 : 0.0;
  if (!gbdry) return;
  for (int k = 0; k < g->mz; k++)
    for (int j = 0; j < g->my; j++)
      for (int i = 0; i < g->mx; i++)
        if (is_bdry(g, i, j, k)) u[IDX(g, i, j, k)] = gval(g, i, j, k, h);
}

/* ---- error report: fish.c:254-276 ---- */
void or_errnorms(const or_grid *g, const double *u, double *errinf, double *err2h) {
  double h[3];
  or_spacing(g, h);
  double emax = 0.0, s2 = 0.0;
  for (int k = 0; k < g->mz; k++) {
    double pl2 = 0.0;
    for (int j = 0; j < g->my; j++)
      for (int i = 0; i < g->mx; i++) {
        double e = u[IDX(g, i, j, k)] - gval(g, i, j, k, h);
        if (fabs(e) > emax) emax = fabs(e);
        pl2 += e * e;
      }
    s2 += pl2;
  }
  double normconst = (double)(g->mx - 1);
  if (g->dim >= 2) normconst *= (double)(g->my - 1);
  if (g->dim >= 3) normconst *= (double)(g->mz - 1);
  *errinf = emax;
  *err2h = sqrt(s2) / sqrt(normconst);
}

/* deterministic dot: one partial per (j,k) line, summed serially */
double or_dot(const or_grid *g, const double *a, const double *b) {
  const int nl = g->my * g->mz, mx = g->mx;
  double *part = (double *)malloc(sizeof(double) * (size_t)nl);
#pragma omp parallel for schedule(static)
  for (int l = 0; l < nl; l++) {
    const double *pa = a + (size_t)l * mx, *pb = b + (size_t)l * mx;
    double s = 0.0;
    for (int i = 0; i < mx; i++) s += pa[i] * pb[i];
    part[l] = s;
  }
  double s = 0.0;
  for (int l = 0; l < nl; l++) s += part[l];
  free(part);
  return s;
}

static void vcopy(long long N, const double *a, double *b) {
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++) b[n] = a[n];
}
static void vzero(long long N, double *a) {
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++) a[n] = 0.0;
}

/* ---- grid transfers: DMDA Q1 interpolation P (vertex-centred, ratio 2) and
   restriction P^T, applied to every node including boundary nodes ---- */
void or_prolong_add(const or_grid *f, const or_grid *c, const double *xc, double *xf) {
  const int dim = f->dim;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < f->mz; k++) {
    for (int j = 0; j < f->my; j++) {
      for (int i = 0; i < f->mx; i++) {
        int i0 = i >> 1, i1 = (i & 1) ? i0 + 1 : i0;
        int j0 = j >> 1, j1 = (dim >= 2 && (j & 1)) ? j0 + 1 : j0;
        int k0 = k >> 1, k1 = (dim >= 3 && (k & 1)) ? k0 + 1 : k0;
        double wi = (i & 1) ? 0.5 : 1.0, wj = (dim >= 2 && (j & 1)) ? 0.5 : 1.0,
               wk = (dim >= 3 && (k & 1)) ? 0.5 : 1.0;
        double v = 0.0;
        int ni = (i & 1) ? 2 : 1, nj = (dim >= 2 && (j & 1)) ? 2 : 1, nk = (dim >= 3 && (k & 1)) ? 2 : 1;
        for (int c3 = 0; c3 < nk; c3++)
          for (int c2 = 0; c2 < nj; c2++)
            for (int c1 = 0; c1 < ni; c1++) {
              int I = c1 ? i1 : i0, J = c2 ? j1 : j0, K = c3 ? k1 : k0;
              v += wi * wj * wk * xc[IDX(c, I, J, K)];
            }
        xf[IDX(f, i, j, k)] += v;
      }
    }
  }
}

void or_restrict(const or_grid *f, const or_grid *c, const double *rf, double *bc) {
  const int dim = f->dim;
  const int dk = dim >= 3 ? 1 : 0, dj = dim >= 2 ? 1 : 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int K = 0; K < c->mz; K++) {
    for (int J = 0; J < c->my; J++) {
      for (int I = 0; I < c->mx; I++) {
        double v = 0.0;
        for (int a = -dk; a <= dk; a++) {
          int k = 2 * K + a;
          if (k < 0 || k >= f->mz) continue;
          double wk = a ? 0.5 : 1.0;
          for (int b = -dj; b <= dj; b++) {
            int j = 2 * J + b;
            if (j < 0 || j >= f->my) continue;
            double wj = b ? 0.5 : 1.0;
            for (int e = -1; e <= 1; e++) {
              int i = 2 * I + e;
              if (i < 0 || i >= f->mx) continue;
              double wi = e ? 0.5 : 1.0;
              v += wi * wj * wk * rf[IDX(f, i, j, k)];
            }
          }
        }
        bc[IDX(c, I, J, K)] = v;
      }
    }
  }
}

/* ---- smoothers ---- */

/* exact spectrum ends of D^{-1}A for the constant-diagonal stencil:
   1 -+ sum_d (2 sc_d/scdiag) cos(pi/(m_d-1)); boundary rows contribute 1 */
static void spectrum(const or_grid *g, double *lmin, double *lmax) {
  double sc[3], scdiag, vol;
  weights(g, sc, &scdiag, &vol);
  int m[3] = {g->mx, g->my, g->mz};
  int interior = 1;
  for (int d = 0; d < g->dim; d++)
    if (m[d] < 3) interior = 0;
  double s = 0.0;
  if (interior)
    for (int d = 0; d < g->dim; d++) s += 2.0 * sc[d] / scdiag * cos(M_PI / (m[d] - 1));
  *lmax = 1.0 + s;
  *lmin = 1.0 - s;
  if (*lmax < 1.0) *lmax = 1.0;
  if (*lmin > 1.0) *lmin = 1.0;
}

void or_cheb_bounds(const or_grid *g, const double esteig[4], double *emin, double *emax) {
  double lmin, lmax;
  spectrum(g, &lmin, &lmax);
  *emin = esteig[0] * lmin + esteig[1] * lmax;
  *emax = esteig[2] * lmin + esteig[3] * lmax;
}

/* Chebyshev semi-iteration (first kind) preconditioned by Jacobi, nonzero
   initial guess, `its` iterations; PETSc KSPCHEBYSHEV semantics.
   w1, w2, w3: work vectors. */
void or_chebyshev(const or_grid *g, double emin, double emax, int its,
                  const double *b, double *x, double *w1, double *w2, double *w3) {
  double sc[3], scdiag, vol;
  weights(g, sc, &scdiag, &vol);
  const long long N = or_nodes(g);
  const double dinv = 1.0 / scdiag;
  const double scale = 2.0 / (emax + emin);
  const double alpha = 1.0 - scale * emin;
  const double mu = 1.0 / alpha, omegaprod = 2.0 / alpha;
  double ckm1 = 1.0, ck = mu;
  double *pkm1 = x, *pk = w1, *pkp1 = w2, *r = w3;
  if (its <= 0) return;
  or_apply(g, pkm1, r);
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++) {
    double rn = b[n] - r[n];
    pk[n] = pkm1[n] + scale * (rn * dinv);
  }
  for (int it = 1; it < its; it++) {
    double ckp1 = 2.0 * mu * ck - ckm1;
    double omega = omegaprod * ck / ckp1;
    or_apply(g, pk, r);
#pragma omp parallel for schedule(static)
    for (long long n = 0; n < N; n++) {
      double z = (b[n] - r[n]) * dinv;
      pkp1[n] = (1.0 - omega) * pkm1[n] + omega * pk[n] + omega * scale * z;
    }
    double *t = pkm1; pkm1 = pk; pk = pkp1; pkp1 = t;
    ckm1 = ck; ck = ckp1;
  }
  if (pk != x) vcopy(N, pk, x);
}

static void richardson(const or_grid *g, double scale, int its, const double *b, double *x, double *r) {
  double sc[3], scdiag, vol;
  weights(g, sc, &scdiag, &vol);
  const long long N = or_nodes(g);
  for (int it = 0; it < its; it++) {
    or_apply(g, x, r);
#pragma omp parallel for schedule(static)
    for (long long n = 0; n < N; n++) x[n] += scale * ((b[n] - r[n]) / scdiag);
  }
}

/* ---- exact solve by sine-transform diagonalisation ----
   Interior block: J = sum_d sc_d T_d (T = tridiag(-1,2,-1) on m_d-2 points), whose
   eigenvectors are S_{ik} = sqrt(2/(n+1)) sin(ik pi/(n+1)), eigenvalues
   2 - 2cos(k pi/(n+1)), n = m_d - 2.  Boundary rows: x = b/scdiag. */
static void sine_matrix(int n, double *S) {
  double a = sqrt(2.0 / (n + 1));
  for (int i = 1; i <= n; i++)
    for (int k = 1; k <= n; k++) S[(i - 1) * n + (k - 1)] = a * sin(M_PI * (double)i * k / (n + 1));
}

/* apply S (symmetric) along dimension d of an interior array of shape n[0..2] */
static void transform_dim(const int n[3], int d, const double *S, double *a) {
  const int n0 = n[0], n1 = n[1], n2 = n[2], nd = n[d];
  const size_t st[3] = {1, (size_t)n0, (size_t)n0 * n1};
  const size_t total = (size_t)n0 * n1 * n2;
  const size_t lines = total / nd;
#pragma omp parallel
  {
    double *tmp = (double *)malloc(sizeof(double) * nd);
#pragma omp for schedule(static)
    for (size_t l = 0; l < lines; l++) {
      /* base index of line l along dimension d */
      size_t base;
      if (d == 0) base = l * n0;
      else if (d == 1) base = (l / n0) * (size_t)n0 * n1 + (l % n0);
      else base = l;
      for (int i = 0; i < nd; i++) {
        double s = 0.0;
        for (int k = 0; k < nd; k++) s += S[i * nd + k] * a[base + k * st[d]];
        tmp[i] = s;
      }
      for (int i = 0; i < nd; i++) a[base + i * st[d]] = tmp[i];
    }
    free(tmp);
  }
}

int or_exact_solve(const or_grid *g, const double *b, double *x) {
  double sc[3], scdiag, vol;
  weights(g, sc, &scdiag, &vol);
  const int dim = g->dim;
  int m[3] = {g->mx, g->my, g->mz};
  int n[3] = {1, 1, 1};
  for (int d = 0; d < dim; d++) n[d] = m[d] - 2;
  const long long N = or_nodes(g);
  /* boundary rows (and everything, if there is no interior) */
  for (long long q = 0; q < N; q++) x[q] = b[q] / scdiag;
  for (int d = 0; d < dim; d++)
    if (n[d] < 1) return 0;
  size_t ni = (size_t)n[0] * n[1] * n[2];
  double *a = (double *)malloc(sizeof(double) * ni);
  double *S[3] = {NULL, NULL, NULL};
  double *lam[3] = {NULL, NULL, NULL};
  if (!a) return -1;
  for (int d = 0; d < dim; d++) {
    S[d] = (double *)malloc(sizeof(double) * n[d] * n[d]);
    lam[d] = (double *)malloc(sizeof(double) * n[d]);
    sine_matrix(n[d], S[d]);
    for (int k = 1; k <= n[d]; k++) lam[d][k - 1] = sc[d] * (2.0 - 2.0 * cos(M_PI * k / (n[d] + 1)));
  }
  const int oj = dim >= 2 ? 1 : 0, ok = dim >= 3 ? 1 : 0;
  for (int k = 0; k < n[2]; k++)
    for (int j = 0; j < n[1]; j++)
      for (int i = 0; i < n[0]; i++)
        a[((size_t)k * n[1] + j) * n[0] + i] = b[IDX(g, i + 1, j + oj, k + ok)];
  for (int d = 0; d < dim; d++) transform_dim(n, d, S[d], a);
  for (int k = 0; k < n[2]; k++)
    for (int j = 0; j < n[1]; j++)
      for (int i = 0; i < n[0]; i++) {
        double l = lam[0][i];
        if (dim >= 2) l += lam[1][j];
        if (dim >= 3) l += lam[2][k];
        a[((size_t)k * n[1] + j) * n[0] + i] /= l;
      }
  for (int d = 0; d < dim; d++) transform_dim(n, d, S[d], a);
  for (int k = 0; k < n[2]; k++)
    for (int j = 0; j < n[1]; j++)
      for (int i = 0; i < n[0]; i++)
        x[IDX(g, i + 1, j + oj, k + ok)] = a[((size_t)k * n[1] + j) * n[0] + i];
  for (int d = 0; d < dim; d++) { free(S[d]); free(lam[d]); }
  free(a);
  return 0;
}

/* ---- multigrid preconditioner ---- */
typedef struct {
  or_grid g;
  double *b, *x, *r, *w1, *w2, *w3;
  double emin, emax;
} mg_level;

typedef struct {
  int nlev;
  mg_level *lev; /* lev[0] coarsest ... lev[nlev-1] finest */
  const or_opts *o;
} mg_ctx;

static int mg_setup(const or_opts *o, mg_ctx *mg) {
  int L = o->mg_levels;
  if (L < 1) return -1;
  mg->nlev = L;
  mg->o = o;
  mg->lev = (mg_level *)calloc((size_t)L, sizeof(mg_level));
  or_grid g = o->grid;
  for (int l = L - 1; l >= 0; l--) {
    mg_level *lv = &mg->lev[l];
    lv->g = g;
    lv->g.problem = OR_ZERO; /* level operators only; data enters through b */
    long long N = or_nodes(&g);
    lv->b = (double *)calloc((size_t)N, sizeof(double));
    lv->x = (double *)calloc((size_t)N, sizeof(double));
    lv->r = (double *)calloc((size_t)N, sizeof(double));
    lv->w1 = (double *)calloc((size_t)N, sizeof(double));
    lv->w2 = (double *)calloc((size_t)N, sizeof(double));
    lv->w3 = (double *)calloc((size_t)N, sizeof(double));
    or_cheb_bounds(&lv->g, o->esteig, &lv->emin, &lv->emax);
    if (l > 0) {
      int m[3] = {g.mx, g.my, g.mz};
      for (int d = 0; d < g.dim; d++) {
        if ((m[d] - 1) % 2 != 0 || m[d] < 3) return -2; /* cannot coarsen */
        m[d] = (m[d] - 1) / 2 + 1;
      }
      g.mx = m[0]; g.my = m[1]; g.mz = m[2];
    }
  }
  return 0;
}

static void mg_free(mg_ctx *mg) {
  for (int l = 0; l < mg->nlev; l++) {
    mg_level *lv = &mg->lev[l];
    free(lv->b); free(lv->x); free(lv->r); free(lv->w1); free(lv->w2); free(lv->w3);
  }
  free(mg->lev);
}

static void mg_smooth(mg_ctx *mg, mg_level *lv) {
  const or_opts *o = mg->o;
  if (o->smooth_type == OR_SMOOTH_CHEBYSHEV)
    or_chebyshev(&lv->g, lv->emin, lv->emax, o->smooth_its, lv->b, lv->x, lv->w1, lv->w2, lv->w3);
  else
    richardson(&lv->g, o->richardson_scale, o->smooth_its, lv->b, lv->x, lv->r);
}

static void mg_cycle(mg_ctx *mg, int l) {
  mg_level *lv = &mg->lev[l];
  if (l == 0) {
    or_exact_solve(&lv->g, lv->b, lv->x);
    return;
  }
  mg_level *lc = &mg->lev[l - 1];
  long long N = or_nodes(&lv->g);
  mg_smooth(mg, lv);                          /* pre-smooth */
  or_apply(&lv->g, lv->x, lv->r);             /* r = b - A x */
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++) lv->r[n] = lv->b[n] - lv->r[n];
  or_restrict(&lv->g, &lc->g, lv->r, lc->b);  /* b_c = P^T r */
  vzero(or_nodes(&lc->g), lc->x);
  for (int c = 0; c < mg->o->mg_cycles; c++) mg_cycle(mg, l - 1);
  or_prolong_add(&lv->g, &lc->g, lc->x, lv->x); /* x += P x_c */
  mg_smooth(mg, lv);                          /* post-smooth */
}

static void mg_apply(mg_ctx *mg, const double *r, double *z) {
  mg_level *top = &mg->lev[mg->nlev - 1];
  long long N = or_nodes(&top->g);
  vcopy(N, r, top->b);
  vzero(N, top->x);
  mg_cycle(mg, mg->nlev - 1);
  vcopy(N, top->x, z);
}

/* The multigrid V-cycle as a preconditioner object for other oracle solvers
   (the minimal-surface Newton-Krylov baseline): the hierarchy of o->grid with
   o's smoother options; the options are copied. */
typedef struct {
  or_opts o;
  mg_ctx mg;
} or_mg;

void *or_mg_new(const or_opts *o) {
  or_mg *m = (or_mg *)calloc(1, sizeof(or_mg));
  if (!m) return NULL;
  m->o = *o;
  if (mg_setup(&m->o, &m->mg) != 0) {
    free(m);
    return NULL;
  }
  return m;
}

void or_mg_apply(void *m, const double *r, double *z) { mg_apply(&((or_mg *)m)->mg, r, z); }

void or_mg_free(void *m) {
  if (!m) return;
  mg_free(&((or_mg *)m)->mg);
  free(m);
}

/* ---- ILU(0), natural ordering, on the Jacobian pattern ---- */
typedef struct {
  or_grid g;
  double *d; /* modified pivots */
  double sc[3], scdiag;
} ilu_ctx;

static void ilu_setup(const or_grid *g, ilu_ctx *il) {
  double vol;
  il->g = *g;
  weights(g, il->sc, &il->scdiag, &vol);
  long long N = or_nodes(g);
  il->d = (double *)malloc(sizeof(double) * (size_t)N);
  const size_t st[3] = {1, (size_t)g->mx, (size_t)g->mx * g->my};
  for (int k = 0; k < g->mz; k++)
    for (int j = 0; j < g->my; j++)
      for (int i = 0; i < g->mx; i++) {
        size_t n = IDX(g, i, j, k);
        double dn = il->scdiag;
        if (!is_bdry(g, i, j, k)) {
          int c[3] = {i, j, k};
          for (int d = 0; d < g->dim; d++)
            if (c[d] - 1 > 0) dn -= il->sc[d] * il->sc[d] / il->d[n - st[d]];
        }
        il->d[n] = dn;
      }
}

static void ilu_apply(const ilu_ctx *il, const double *r, double *z) {
  const or_grid *g = &il->g;
  const size_t st[3] = {1, (size_t)g->mx, (size_t)g->mx * g->my};
  long long N = or_nodes(g);
  for (int k = 0; k < g->mz; k++) /* forward: (D + L) v = r */
    for (int j = 0; j < g->my; j++)
      for (int i = 0; i < g->mx; i++) {
        size_t n = IDX(g, i, j, k);
        double s = r[n];
        if (!is_bdry(g, i, j, k)) {
          int c[3] = {i, j, k};
          for (int d = 0; d < g->dim; d++)
            if (c[d] - 1 > 0) s += il->sc[d] * z[n - st[d]];
        }
        z[n] = s / il->d[n];
      }
  for (long long q = N - 1; q >= 0; q--) { /* backward: (I + D^{-1}U) z = v */
    size_t n = (size_t)q;
    int i = (int)(n % g->mx), j = (int)((n / g->mx) % g->my), k = (int)(n / ((size_t)g->mx * g->my));
    if (is_bdry(g, i, j, k)) continue;
    int c[3] = {i, j, k}, m[3] = {g->mx, g->my, g->mz};
    double s = 0.0;
    for (int d = 0; d < g->dim; d++)
      if (c[d] + 1 < m[d] - 1) s += il->sc[d] * z[n + st[d]];
    z[n] += s / il->d[n];
  }
}

/* ---- preconditioner dispatch ---- */
typedef struct {
  int type;
  or_grid g;
  double scdiag;
  mg_ctx mg;
  ilu_ctx ilu;
} pc_ctx;

static void pc_apply(pc_ctx *pc, const double *r, double *z) {
  long long N = or_nodes(&pc->g);
  switch (pc->type) {
  case OR_PC_JACOBI:
#pragma omp parallel for schedule(static)
    for (long long n = 0; n < N; n++) z[n] = r[n] / pc->scdiag;
    break;
  case OR_PC_MG: mg_apply(&pc->mg, r, z); break;
  case OR_PC_ILU: ilu_apply(&pc->ilu, r, z); break;
  default: vcopy(N, r, z);
  }
}

/* KSPConvergedDefault semantics; returns the reason (0 = keep iterating) */
static int converged(const or_opts *o, int it, double rnorm, double *ttol, double *rnorm0) {
  if (it == 0) {
    *rnorm0 = rnorm;
    *ttol = fmax(o->rtol * rnorm, o->atol);
  }
  if (isnan(rnorm) || isinf(rnorm)) return OR_DIVERGED_NANORINF;
  if (rnorm <= *ttol) return rnorm < o->atol ? OR_CONVERGED_ATOL : OR_CONVERGED_RTOL;
  if (rnorm >= o->dtol * *rnorm0 && it > 0) return OR_DIVERGED_DTOL;
  return 0;
}

/* KSPCG from y = 0 (guess zero), PETSc cg.c algorithm restated */
int or_ksp_solve(const or_opts *o, const double *bvec, double *y, or_report *rep) {
  const or_grid *g = &o->grid;
  long long N = or_nodes(g);
  pc_ctx pc;
  memset(&pc, 0, sizeof(pc));
  pc.type = o->pc_type;
  pc.g = *g;
  {
    double sc[3], vol;
    weights(g, sc, &pc.scdiag, &vol);
  }
  if (pc.type == OR_PC_MG && mg_setup(o, &pc.mg) != 0) return -1;
  if (pc.type == OR_PC_ILU) ilu_setup(g, &pc.ilu);
  double *r = (double *)malloc(sizeof(double) * N), *z = (double *)malloc(sizeof(double) * N);
  double *p = (double *)malloc(sizeof(double) * N), *w = (double *)malloc(sizeof(double) * N);
  vzero(N, y);
  vcopy(N, bvec, r); /* r = b (x = 0) */
  double dp, beta = 0.0, betaold = 1.0, dpi = 0.0, dpiold, ttol = 0.0, rnorm0 = 0.0;
  int reason = 0, its = 0, nh = 0;
  if (o->norm_type == OR_NORM_PRECONDITIONED) {
    pc_apply(&pc, r, z);
    dp = sqrt(or_dot(g, z, z));
  } else {
    dp = sqrt(or_dot(g, r, r));
  }
  if (rep->hist) rep->hist[nh] = dp;
  nh++;
  reason = converged(o, 0, dp, &ttol, &rnorm0);
  if (!reason) {
    if (o->norm_type != OR_NORM_PRECONDITIONED) pc_apply(&pc, r, z);
    beta = or_dot(g, z, r);
    int i = 0;
    do {
      its = i + 1;
      if (beta == 0.0) { reason = OR_CONVERGED_ATOL; break; }
      if (i > 0 && beta * betaold < 0.0) { reason = OR_DIVERGED_INDEFINITE_PC; break; }
      if (i == 0) {
        vcopy(N, z, p);
      } else {
        double bb = beta / betaold;
#pragma omp parallel for schedule(static)
        for (long long n = 0; n < N; n++) p[n] = z[n] + bb * p[n];
      }
      dpiold = dpi;
      or_apply(g, p, w);
      dpi = or_dot(g, p, w);
      betaold = beta;
      if (dpi == 0.0 || (i > 0 && dpi * dpiold < 0.0)) { reason = OR_DIVERGED_INDEFINITE_MAT; break; }
      double a = beta / dpi;
#pragma omp parallel for schedule(static)
      for (long long n = 0; n < N; n++) {
        y[n] += a * p[n];
        r[n] -= a * w[n];
      }
      if (o->norm_type == OR_NORM_PRECONDITIONED) {
        pc_apply(&pc, r, z);
        dp = sqrt(or_dot(g, z, z));
      } else {
        dp = sqrt(or_dot(g, r, r));
      }
      if (rep->hist) rep->hist[nh] = dp;
      nh++;
      reason = converged(o, i + 1, dp, &ttol, &rnorm0);
      if (reason) break;
      if (o->norm_type != OR_NORM_PRECONDITIONED) pc_apply(&pc, r, z);
      beta = or_dot(g, z, r);
      i++;
    } while (i < o->max_it);
    if (!reason && i >= o->max_it) reason = OR_DIVERGED_ITS;
  }
  rep->its = its;
  rep->reason = reason;
  rep->nhist = nh;
  free(r); free(z); free(p); free(w);
  if (pc.type == OR_PC_MG) mg_free(&pc.mg);
  if (pc.type == OR_PC_ILU) free(pc.ilu.d);
  return 0;
}

/* fish.c:237-280 with SNESKSPONLY: F(u0), solve J y = F, u = u0 - y, report */
int or_fish_solve(const or_opts *o, double *u, or_report *rep) {
  const or_grid *g = &o->grid;
  long long N = or_nodes(g);
  double *F = (double *)malloc(sizeof(double) * N), *y = (double *)malloc(sizeof(double) * N);
  if (!F || !y) return -1;
  or_initial_state(g, o->initial_type, o->initial_gonboundary, o->seed, u);
  or_residual(g, u, F);
  rep->fnorm0 = sqrt(or_dot(g, F, F));
  int rc = or_ksp_solve(o, F, y, rep);
  if (rc) { free(F); free(y); return rc; }
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < N; n++) u[n] -= y[n];
  or_residual(g, u, F);
  rep->fnorm1 = sqrt(or_dot(g, F, F));
  or_errnorms(g, u, &rep->errinf, &rep->err2h);
  free(F); free(y);
  return 0;
}

/* ---- options, with fish's spellings ---- */
void or_opts_default(or_opts *o) {
  memset(o, 0, sizeof(*o));
  o->grid.dim = 2;                 /* fish.c:140 */
  o->grid.problem = OR_MANUEXP;    /* fish.c:141 */
  o->grid.Lx = o->grid.Ly = o->grid.Lz = 1.0;
  o->grid.cx = o->grid.cy = o->grid.cz = 1.0;
  o->initial_type = 0;
  o->initial_gonboundary = 1;
  o->rtol = 1e-5; o->atol = 1e-50; o->dtol = 1e5; o->max_it = 10000; /* KSP defaults */
  o->norm_type = OR_NORM_PRECONDITIONED;
  o->pc_type = OR_PC_ILU;          /* PETSc's one-rank default */
  o->mg_levels = 0;
  o->mg_cycles = 1;
  o->smooth_type = OR_SMOOTH_CHEBYSHEV;
  o->smooth_its = 2;
  o->esteig[0] = 0.0; o->esteig[1] = 0.1; o->esteig[2] = 0.0; o->esteig[3] = 1.1;
  o->richardson_scale = 1.0;
  o->seed = 0;
}

static int parse_bool(const char *s) {
  if (!s) return 1;
  if (!strcmp(s, "0") || !strcasecmp(s, "false") || !strcasecmp(s, "no")) return 0;
  return 1;
}

int or_opts_parse(or_opts *o, int argc, const char **argv, int *da_refine_out) {
  int refine = 0, base[3] = {3, 3, 3}, levels = 0;
  for (int a = 0; a < argc; a++) {
    const char *k = argv[a];
    const char *v = (a + 1 < argc) ? argv[a + 1] : NULL;
    int hasv = v && (v[0] != '-' || (v[1] >= '0' && v[1] <= '9') || v[1] == '.');
#define TAKE() (a++, v)
    if (!strcmp(k, "-fsh_dim") && hasv) o->grid.dim = atoi(TAKE());
    else if (!strcmp(k, "-fsh_problem") && hasv) {
      const char *s = TAKE();
      if (!strcmp(s, "manupoly")) o->grid.problem = OR_MANUPOLY;
      else if (!strcmp(s, "manuexp")) o->grid.problem = OR_MANUEXP;
      else if (!strcmp(s, "zero")) o->grid.problem = OR_ZERO;
      else return 62;
    } else if (!strcmp(k, "-fsh_cx") && hasv) o->grid.cx = atof(TAKE());
    else if (!strcmp(k, "-fsh_cy") && hasv) o->grid.cy = atof(TAKE());
    else if (!strcmp(k, "-fsh_cz") && hasv) o->grid.cz = atof(TAKE());
    else if (!strcmp(k, "-fsh_Lx") && hasv) o->grid.Lx = atof(TAKE());
    else if (!strcmp(k, "-fsh_Ly") && hasv) o->grid.Ly = atof(TAKE());
    else if (!strcmp(k, "-fsh_Lz") && hasv) o->grid.Lz = atof(TAKE());
    else if (!strcmp(k, "-fsh_initial_type") && hasv) {
      const char *s = TAKE();
      o->initial_type = !strcmp(s, "random") ? 1 : 0;
    } else if (!strcmp(k, "-fsh_initial_gonboundary")) {
      if (v && v[0] != '-') o->initial_gonboundary = parse_bool(TAKE());
      else o->initial_gonboundary = 1;
    } else if (!strcmp(k, "-da_refine") && hasv) refine = atoi(TAKE());
    else if (!strcmp(k, "-da_grid_x") && hasv) base[0] = atoi(TAKE());
    else if (!strcmp(k, "-da_grid_y") && hasv) base[1] = atoi(TAKE());
    else if (!strcmp(k, "-da_grid_z") && hasv) base[2] = atoi(TAKE());
    else if (!strcmp(k, "-ksp_rtol") && hasv) o->rtol = atof(TAKE());
    else if (!strcmp(k, "-ksp_atol") && hasv) o->atol = atof(TAKE());
    else if (!strcmp(k, "-ksp_divtol") && hasv) o->dtol = atof(TAKE());
    else if (!strcmp(k, "-ksp_max_it") && hasv) o->max_it = atoi(TAKE());
    else if (!strcmp(k, "-ksp_norm_type") && hasv) {
      const char *s = TAKE();
      o->norm_type = !strcmp(s, "unpreconditioned") ? OR_NORM_UNPRECONDITIONED : OR_NORM_PRECONDITIONED;
    } else if (!strcmp(k, "-pc_type") && hasv) {
      const char *s = TAKE();
      if (!strcmp(s, "mg")) o->pc_type = OR_PC_MG;
      else if (!strcmp(s, "jacobi")) o->pc_type = OR_PC_JACOBI;
      else if (!strcmp(s, "none")) o->pc_type = OR_PC_NONE;
      else if (!strcmp(s, "ilu")) o->pc_type = OR_PC_ILU;
      else return 56;
    } else if (!strcmp(k, "-pc_mg_levels") && hasv) levels = atoi(TAKE());
    else if (!strcmp(k, "-pc_mg_cycle_type") && hasv) o->mg_cycles = !strcmp(TAKE(), "w") ? 2 : 1;
    else if (!strcmp(k, "-mg_levels_ksp_type") && hasv) {
      const char *s = TAKE();
      o->smooth_type = !strcmp(s, "richardson") ? OR_SMOOTH_RICHARDSON : OR_SMOOTH_CHEBYSHEV;
    } else if (!strcmp(k, "-mg_levels_ksp_max_it") && hasv) o->smooth_its = atoi(TAKE());
    else if (!strcmp(k, "-mg_levels_ksp_richardson_scale") && hasv) o->richardson_scale = atof(TAKE());
    else if (!strcmp(k, "-mg_levels_ksp_chebyshev_esteig") && hasv) {
      const char *s = TAKE();
      if (sscanf(s, "%lf,%lf,%lf,%lf", &o->esteig[0], &o->esteig[1], &o->esteig[2], &o->esteig[3]) != 4)
        return 62;
    } else if (!strcmp(k, "-fsh_seed") && hasv) o->seed = strtoull(TAKE(), NULL, 10);
#undef TAKE
  }
  int dim = o->grid.dim;
  if (dim < 1 || dim > 3) return 1;                                    /* fish.c:214-216 */
  if (o->grid.cx <= 0.0 || o->grid.cy <= 0.0 || o->grid.cz <= 0.0) return 2; /* fish.c:188-190 */
  if (o->grid.problem == OR_MANUEXP && (o->grid.cx != 1.0 || o->grid.cy != 1.0 || o->grid.cz != 1.0))
    return 3;                                                          /* fish.c:191-193 */
  int m[3] = {1, 1, 1};
  for (int d = 0; d < dim; d++) m[d] = (base[d] - 1) * (1 << refine) + 1;
  o->grid.mx = m[0]; o->grid.my = m[1]; o->grid.mz = m[2];
  o->mg_levels = levels > 0 ? levels : refine + 1;
  if (da_refine_out) *da_refine_out = refine;
  return 0;
}

static const char *reason_name(int r) {
  switch (r) {
  case OR_CONVERGED_RTOL: return "CONVERGED_RTOL";
  case OR_CONVERGED_ATOL: return "CONVERGED_ATOL";
  case OR_DIVERGED_ITS: return "DIVERGED_ITS";
  case OR_DIVERGED_DTOL: return "DIVERGED_DTOL";
  case OR_DIVERGED_INDEFINITE_PC: return "DIVERGED_INDEFINITE_PC";
  case OR_DIVERGED_NANORINF: return "DIVERGED_NANORINF";
  case OR_DIVERGED_INDEFINITE_MAT: return "DIVERGED_INDEFINITE_MAT";
  default: return "CONVERGED_ITERATING";
  }
}

static void print_snes_norm(int it, double f) {
  if (f > 1.e-9) printf("%3d SNES Function norm %g\n", it, f);
  else if (f > 1.e-11) printf("%3d SNES Function norm %5.3e\n", it, f);
  else printf("%3d SNES Function norm < 1.e-11\n", it);
}

int or_fish_main(int argc, const char **argv) {
  or_opts o;
  or_opts_default(&o);
  int rc = or_opts_parse(&o, argc, argv, NULL);
  if (rc) { fprintf(stderr, "fish oracle: invalid options (code %d)\n", rc); return rc; }
  int snes_mon = 0, reason = 0, kspmon = 0;
  for (int a = 0; a < argc; a++) {
    if (!strcmp(argv[a], "-snes_monitor_short") || !strcmp(argv[a], "-snes_monitor")) snes_mon = 1;
    if (!strcmp(argv[a], "-ksp_converged_reason")) reason = 1;
    if (!strcmp(argv[a], "-ksp_monitor")) kspmon = 1;
  }
  long long N = or_nodes(&o.grid);
  double *u = (double *)malloc(sizeof(double) * N);
  double *hist = (double *)malloc(sizeof(double) * (o.max_it + 2));
  or_report rep;
  memset(&rep, 0, sizeof(rep));
  rep.hist = hist;
  rc = or_fish_solve(&o, u, &rep);
  if (rc) { fprintf(stderr, "fish oracle: solve failed (%d)\n", rc); return 70; }
  if (snes_mon) print_snes_norm(0, rep.fnorm0);
  if (kspmon)
    for (int i = 0; i < rep.nhist; i++) printf("    %d KSP Residual norm %g\n", i, rep.hist[i]);
  if (reason) {
    if (rep.reason > 0)
      printf("    Linear solve converged due to %s iterations %d\n", reason_name(rep.reason), rep.its);
    else
      printf("    Linear solve did not converge due to %s iterations %d\n", reason_name(rep.reason), rep.its);
  }
  if (snes_mon) print_snes_norm(1, rep.fnorm1);
  static const char *pn[] = {"manupoly", "manuexp", "zero"};
  char gridstr[99];
  if (o.grid.dim == 1) snprintf(gridstr, 99, "%d point 1D", o.grid.mx);
  else if (o.grid.dim == 2) snprintf(gridstr, 99, "%d x %d point 2D", o.grid.mx, o.grid.my);
  else snprintf(gridstr, 99, "%d x %d x %d point 3D", o.grid.mx, o.grid.my, o.grid.mz);
  printf("problem %s on %s grid:\n  error |u-uexact|_inf = %.3e, |u-uexact|_h = %.3e\n",
         pn[o.grid.problem], gridstr, rep.errinf, rep.err2h);
  fflush(stdout);
  free(u); free(hist);
  return 0;
}
