/* minimal_oracle.c -- CPU restatement of the minimal-surface equation of
 * c/ch7/minimal.c for parity tests (TEST INFRASTRUCTURE; the GPU library
 * never calls it).
 *
 *   -div( (1 + |grad u|^2)^q grad u ) = 0 on the unit square, u = g on the
 *   boundary; q = -1/2 is the minimal surface equation.
 *
 * Each function cites the reference lines it restates.  The Jacobian is not
 * in the reference (it uses finite-difference colouring or matrix-free
 * differencing of F): ms_jv / ms_jacobian_csr are the exact derivative of
 * ms_residual, checked against differences of F by the tests.
 */
#include "minimal_oracle.h"

#include <math.h>
#include <stdlib.h>

/* boundary data, minimal.c:27-42 */
double ms_g(const ms_grid *g, double x, double y) {
  if (g->problem == MS_TENT) {
    if (x < 1.0e-8) return 2.0 * g->tent_H * (y < 0.5 ? y : 1.0 - y);
    return 0.0;
  }
  const double c = g->catenoid_c;
  return c * cosh(x / c) * sin(acos((y / c) / cosh(x / c)));
}

static int on_bdry(const ms_grid *g, int i, int j) {
  return i == 0 || j == 0 || i == g->mx - 1 || j == g->my - 1;
}

/* InitialState(ZEROS, gonboundary = TRUE), c/ch6/poissonfunctions.c:260-346 as
   called at minimal.c:155-157 */
void ms_initial(const ms_grid *g, double *u) {
  const double hx = 1.0 / (g->mx - 1), hy = 1.0 / (g->my - 1);
  for (int j = 0; j < g->my; j++)
    for (int i = 0; i < g->mx; i++)
      u[(long)j * g->mx + i] = on_bdry(g, i, j) ? ms_g(g, i * hx, j * hy) : 0.0;
}

/* FormExactFromG, minimal.c:193-208 */
void ms_exact(const ms_grid *g, double *u) {
  const double hx = 1.0 / (g->mx - 1), hy = 1.0 / (g->my - 1);
  for (int j = 0; j < g->my; j++)
    for (int i = 0; i < g->mx; i++) u[(long)j * g->mx + i] = ms_g(g, i * hx, j * hy);
}

/* The eight neighbour values of interior node (i,j): the array value, or g
   (evaluated at x +- hx, y +- hy as minimal.c:227-255 does) when the
   neighbour is a boundary node.  Order: e w n s ne nw se sw. */
static void neighbours(const ms_grid *g, const double *u, int i, int j, double v[8]) {
  const int mx = g->mx, my = g->my;
  const double hx = 1.0 / (mx - 1), hy = 1.0 / (my - 1), x = i * hx, y = j * hy;
  const int di[8] = {1, -1, 0, 0, 1, -1, 1, -1}, dj[8] = {0, 0, 1, -1, 1, 1, -1, -1};
  for (int q = 0; q < 8; q++) {
    const int a = i + di[q], b = j + dj[q];
    v[q] = on_bdry(g, a, b) ? ms_g(g, x + di[q] * hx, y + dj[q] * hy) : u[(long)b * mx + a];
  }
}

/* FormFunctionLocal, minimal.c:210-282 */
void ms_residual(const ms_grid *g, const double *u, double *F) {
  const int mx = g->mx, my = g->my;
  const double hx = 1.0 / (mx - 1), hy = 1.0 / (my - 1), hxhy = hx / hy, hyhx = hy / hx;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const long n = (long)j * mx + i;
      if (on_bdry(g, i, j)) {
        F[n] = u[n] - ms_g(g, i * hx, j * hy);
        continue;
      }
      double v[8];
      neighbours(g, u, i, j, v);
      const double uc = u[n], ue = v[0], uw = v[1], un = v[2], us = v[3];
      const double une = v[4], unw = v[5], use = v[6], usw = v[7];
      double dx, dy;
      dx = (ue - uc) / hx;
      dy = (un + une - us - use) / (4.0 * hy);
      const double De = pow(1.0 + dx * dx + dy * dy, g->q);
      dx = (uc - uw) / hx;
      dy = (unw + un - usw - us) / (4.0 * hy);
      const double Dw = pow(1.0 + dx * dx + dy * dy, g->q);
      dx = (ue + une - uw - unw) / (4.0 * hx);
      dy = (un - uc) / hy;
      const double Dn = pow(1.0 + dx * dx + dy * dy, g->q);
      dx = (ue + use - uw - usw) / (4.0 * hx);
      dy = (uc - us) / hy;
      const double Ds = pow(1.0 + dx * dx + dy * dy, g->q);
      F[n] = -hyhx * (De * (ue - uc) - Dw * (uc - uw)) - hxhy * (Dn * (un - uc) - Ds * (uc - us));
    }
}

/* Linearisation of one half-point flux D(W) * (difference):
     delta[D(W) d] = (D + K dn/hn) delta d + (K dt/(4 ht)) delta(transverse sum)
   with K = 2 q (1+W)^(q-1) d, d the normal difference, dn = d/hn the normal
   derivative, dt the transverse derivative.  A = D + K dn/hn, Q = K dt/(4 ht). */
static void half_point(double q, double d, double hn, double dt, double ht, double *A, double *Q) {
  const double dn = d / hn, W = dn * dn + dt * dt;
  const double D = pow(1.0 + W, q);
  const double K = 2.0 * q * pow(1.0 + W, q - 1.0) * d;
  *A = D + K * dn / hn;
  *Q = K * dt / (4.0 * ht);
}

/* A and Q of the four half-points of interior node n, order e w n s */
static void node_coefs(const ms_grid *g, const double *u, int i, int j, double A[4], double Q[4]) {
  const double hx = 1.0 / (g->mx - 1), hy = 1.0 / (g->my - 1);
  double v[8];
  neighbours(g, u, i, j, v);
  const double uc = u[(long)j * g->mx + i], ue = v[0], uw = v[1], un = v[2], us = v[3];
  const double une = v[4], unw = v[5], use = v[6], usw = v[7];
  half_point(g->q, ue - uc, hx, (un + une - us - use) / (4.0 * hy), hy, &A[0], &Q[0]);
  half_point(g->q, uc - uw, hx, (unw + un - usw - us) / (4.0 * hy), hy, &A[1], &Q[1]);
  half_point(g->q, un - uc, hy, (ue + une - uw - unw) / (4.0 * hx), hx, &A[2], &Q[2]);
  half_point(g->q, uc - us, hy, (ue + use - uw - usw) / (4.0 * hx), hx, &A[3], &Q[3]);
}

/* Column weights of interior row (i,j) over the 3x3 block, index
   (dj+1)*3 + (di+1), before dropping boundary neighbours. */
static void row_weights(const ms_grid *g, const double A[4], const double Q[4], double w[9]) {
  const double hx = 1.0 / (g->mx - 1), hy = 1.0 / (g->my - 1), a = hy / hx, b = hx / hy;
  const double Ae = A[0], Aw = A[1], An = A[2], As = A[3], Qe = Q[0], Qw = Q[1], Qn = Q[2], Qs = Q[3];
  w[4] = a * (Ae + Aw) + b * (An + As);      /* centre */
  w[5] = -a * Ae - b * (Qn - Qs);           /* e  */
  w[3] = -a * Aw + b * (Qn - Qs);           /* w  */
  w[7] = -a * (Qe - Qw) - b * An;           /* n  */
  w[1] = a * (Qe - Qw) - b * As;            /* s  */
  w[8] = -a * Qe - b * Qn;                  /* ne */
  w[2] = a * Qe + b * Qs;                   /* se */
  w[6] = a * Qw + b * Qn;                   /* nw */
  w[0] = -a * Qw - b * Qs;                  /* sw */
}

/* the nine column weights of every row (ms_jv's, once per linearisation
   point): w[9 n + (dj+1)*3 + di+1]; boundary rows get w[9n+4] = 1 and zeros */
void ms_row_weights(const ms_grid *g, const double *u, double *w) {
  const int mx = g->mx, my = g->my;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const long n = (long)j * mx + i;
      double *wn = w + 9 * n;
      if (on_bdry(g, i, j)) {
        for (int q = 0; q < 9; q++) wn[q] = q == 4 ? 1.0 : 0.0;
        continue;
      }
      double A[4], Q[4];
      node_coefs(g, u, i, j, A, Q);
      row_weights(g, A, Q, wn);
      for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++)
          if (on_bdry(g, i + di, j + dj)) wn[(dj + 1) * 3 + di + 1] = 0.0;
    }
}

void ms_jv(const ms_grid *g, const double *u, const double *v, double *out) {
  const int mx = g->mx, my = g->my;
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const long n = (long)j * mx + i;
      if (on_bdry(g, i, j)) {
        out[n] = v[n];
        continue;
      }
      double A[4], Q[4], w[9], s = 0.0;
      node_coefs(g, u, i, j, A, Q);
      row_weights(g, A, Q, w);
      for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++)
          if (!on_bdry(g, i + di, j + dj)) s += w[(dj + 1) * 3 + di + 1] * v[n + (long)dj * mx + di];
      out[n] = s;
    }
}

int ms_jacobian_csr(const ms_grid *g, const double *u, int *rowptr, int *col, double *val) {
  const int mx = g->mx, my = g->my;
  int nz = 0;
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      const int n = j * mx + i;
      rowptr[n] = nz;
      if (on_bdry(g, i, j)) {
        col[nz] = n;
        val[nz++] = 1.0;
        continue;
      }
      double A[4], Q[4], w[9];
      node_coefs(g, u, i, j, A, Q);
      row_weights(g, A, Q, w);
      for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++)
          if (!on_bdry(g, i + di, j + dj)) {
            col[nz] = n + dj * mx + di;
            val[nz++] = w[(dj + 1) * 3 + di + 1];
          }
    }
  rowptr[mx * my] = nz;
  return nz;
}

/* MSEMonitor, minimal.c:286-362: area of the Q1 surface and min/max of the
   diffusivity at the Gauss-Legendre points of every cell */
void ms_area(const ms_grid *g, const double *u, int degree, double *area, double *Dmin, double *Dmax) {
  static const double xi1[1] = {0.0}, w1[1] = {2.0};
  static const double xi2[2] = {-0.57735026918962576451, 0.57735026918962576451}, w2[2] = {1.0, 1.0};
  static const double xi3[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};
  static const double w3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  const double *xi = degree == 1 ? xi1 : degree == 2 ? xi2 : xi3;
  const double *wq = degree == 1 ? w1 : degree == 2 ? w2 : w3;
  const int nq = degree < 1 ? 1 : degree > 3 ? 3 : degree;
  const int mx = g->mx;
  const double hx = 1.0 / (g->mx - 1), hy = 1.0 / (g->my - 1);
  double a = 0.0, dmin = INFINITY, dmax = 0.0;
  for (int j = 1; j < g->my; j++) {
    const double yj = j * hy;
    for (int i = 1; i < mx; i++) {
      const double xi_ = i * hx;
      const double u00 = u[(long)(j - 1) * mx + i - 1], u10 = u[(long)(j - 1) * mx + i];
      const double u01 = u[(long)j * mx + i - 1], u11 = u[(long)j * mx + i];
      for (int r = 0; r < nq; r++) {
        const double x = xi_ - hx + hx * 0.5 * (xi[r] + 1.0);
        for (int s = 0; s < nq; s++) {
          const double y = yj - hy + hy * 0.5 * (xi[s] + 1.0);
          const double ux = ((u11 - u01) * (y - (yj - hy)) + (u10 - u00) * (yj - y)) / (hx * hy);
          const double uy = ((u11 - u10) * (x - (xi_ - hx)) + (u01 - u00) * (xi_ - x)) / (hx * hy);
          const double W = ux * ux + uy * uy, D = pow(1.0 + W, g->q);
          if (D < dmin) dmin = D;
          if (D > dmax) dmax = D;
          a += wq[r] * wq[s] * sqrt(1.0 + W);
        }
      }
    }
  }
  *area = a * hx * hy / 4.0;
  *Dmin = dmin;
  *Dmax = dmax;
}

/* DMDA Q1 interpolation, ratio 2 (the grid-sequencing initial iterate) */
void ms_interpolate(const ms_grid *c, const double *uc, const ms_grid *f, double *uf) {
  for (int J = 0; J < f->my; J++)
    for (int I = 0; I < f->mx; I++) {
      const int i0 = I / 2, j0 = J / 2, i1 = i0 + I % 2, j1 = j0 + J % 2;  /* odd: average with the next */
      const double a = uc[(long)j0 * c->mx + i0], b = uc[(long)j0 * c->mx + i1];
      const double d = uc[(long)j1 * c->mx + i0], e = uc[(long)j1 * c->mx + i1];
      uf[(long)J * f->mx + I] = 0.25 * (a + b + d + e);
    }
}
