/* bratu_oracle.h -- CPU restatement of the Liouville-Bratu residual of
 * c/ch7/solns/bratu2D.c (TEST INFRASTRUCTURE: only tests/, smoke() and
 * bench.py's CPU leg use it).  Grid: mx x my nodes on the unit square,
 * index j*mx + i. */
#ifndef BRATU_ORACLE_H
#define BRATU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int mx, my;
  double lambda;
  int exact; /* 1: Liouville boundary data (lambda = 1), 0: u = 0 on the boundary */
} lb_grid;

double lb_g(const lb_grid *g, double x, double y);
void lb_exact(const lb_grid *g, double *u);
void lb_residual(const lb_grid *g, const double *u, double *F);
int lb_jacobian_csr(const lb_grid *g, const double *u, int *rowptr, int *col, double *val);

#ifdef __cplusplus
}
#endif
#endif
