/* minimal_oracle.h -- CPU restatement of the minimal-surface residual of
 * c/ch7/minimal.c (TEST INFRASTRUCTURE: only tests/, smoke() and bench.py's
 * CPU leg use it; the GPU library never does).
 *
 * Grid: mx x my nodes on the unit square (minimal.c:131-136: DMDA box
 * stencil, DMDASetUniformCoordinates(0,1,0,1)), array index j*mx + i.
 */
#ifndef MINIMAL_ORACLE_H
#define MINIMAL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { MS_TENT = 0, MS_CATENOID = 1 };

typedef struct {
  int mx, my;
  int problem;       /* MS_TENT / MS_CATENOID */
  double q;          /* exponent of the diffusivity (1 + |grad u|^2)^q */
  double catenoid_c; /* catenoid parameter c >= 1 */
  double tent_H;     /* tent door height */
} ms_grid;

double ms_g(const ms_grid *g, double x, double y);
/* u = g on the boundary, 0 inside (InitialState ZEROS with g on the boundary) */
void ms_initial(const ms_grid *g, double *u);
/* u = g at every node (FormExactFromG) */
void ms_exact(const ms_grid *g, double *u);
/* F(u), FormFunctionLocal */
void ms_residual(const ms_grid *g, const double *u, double *F);
/* the row weights of J at u, 9 per node (see minimal_oracle.c) */
void ms_row_weights(const ms_grid *g, const double *u, double *w);
/* J v, the exact derivative of F at u applied to v */
void ms_jv(const ms_grid *g, const double *u, const double *v, double *out);
/* the same Jacobian in CSR form (9 entries per interior row, 1 per boundary row);
   rowptr has mx*my+1 entries, col/val at least 9*mx*my */
int ms_jacobian_csr(const ms_grid *g, const double *u, int *rowptr, int *col, double *val);
/* surface area and diffusivity bounds by Q1 + Gauss-Legendre (MSEMonitor) */
void ms_area(const ms_grid *g, const double *u, int degree, double *area, double *Dmin, double *Dmax);
/* DMDA Q1 interpolation coarse -> fine (fine = 2*coarse - 1 nodes per side) */
void ms_interpolate(const ms_grid *c, const double *uc, const ms_grid *f, double *uf);

#ifdef __cplusplus
}
#endif
#endif
