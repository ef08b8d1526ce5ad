/* bratu_oracle.c -- CPU restatement of the Liouville-Bratu equation
 *   -Laplace(u) - lambda e^u = 0 on the unit square, u = g on the boundary,
 * of c/ch7/solns/bratu2D.c for parity tests (TEST INFRASTRUCTURE; the GPU
 * library never calls it).  The Jacobian is the exact derivative of the
 * residual (the reference uses the Poisson Jacobian, FD colouring, or FAS). */
#include "bratu_oracle.h"

#include <math.h>

/* g_zero / g_liouville, bratu2D.c:58-68 */
double lb_g(const lb_grid *g, double x, double y) {
  if (!g->exact) return 0.0;
  const double r2 = (x + 1.0) * (x + 1.0) + (y + 1.0) * (y + 1.0), qq = r2 * r2 + 1.0, omega = r2 / (qq * qq);
  return log(32.0 * omega);
}

/* FormUExact, bratu2D.c:160-182 */
void lb_exact(const lb_grid *g, double *u) {
  const double hx = 1.0 / (double)(g->mx - 1), hy = 1.0 / (double)(g->my - 1);
  for (int j = 0; j < g->my; j++)
    for (int i = 0; i < g->mx; i++) u[(long)j * g->mx + i] = lb_g(g, i * hx, j * hy);
}

static int bdry(const lb_grid *g, int i, int j) { return i == 0 || j == 0 || i == g->mx - 1 || j == g->my - 1; }

/* FormFunctionLocal, bratu2D.c:188-217 */
void lb_residual(const lb_grid *g, const double *u, double *F) {
  const int mx = g->mx;
  const double hx = 1.0 / (double)(g->mx - 1), hy = 1.0 / (double)(g->my - 1);
  const double darea = hx * hy, hxhy = hx / hy, hyhx = hy / hx;
  for (int j = 0; j < g->my; j++)
    for (int i = 0; i < mx; i++) {
      const long n = (long)j * mx + i;
      if (bdry(g, i, j)) {
        F[n] = u[n] - lb_g(g, i * hx, j * hy);
      } else {
        F[n] = hyhx * (2.0 * u[n] - u[n - 1] - u[n + 1]) + hxhy * (2.0 * u[n] - u[n - mx] - u[n + mx]) -
               darea * g->lambda * exp(u[n]);
      }
    }
}

int lb_jacobian_csr(const lb_grid *g, const double *u, int *rowptr, int *col, double *val) {
  const int mx = g->mx;
  const double hx = 1.0 / (double)(g->mx - 1), hy = 1.0 / (double)(g->my - 1);
  const double darea = hx * hy, hxhy = hx / hy, hyhx = hy / hx;
  int nz = 0;
  for (int j = 0; j < g->my; j++)
    for (int i = 0; i < mx; i++) {
      const int n = j * mx + i;
      rowptr[n] = nz;
      if (bdry(g, i, j)) {
        col[nz] = n;
        val[nz++] = 1.0;
        continue;
      }
      col[nz] = n - mx; val[nz++] = -hxhy;
      col[nz] = n - 1;  val[nz++] = -hyhx;
      col[nz] = n;      val[nz++] = 2.0 * (hyhx + hxhy) - darea * g->lambda * exp(u[n]);
      col[nz] = n + 1;  val[nz++] = -hyhx;
      col[nz] = n + mx; val[nz++] = -hxhy;
    }
  rowptr[mx * g->my] = nz;
  return nz;
}
