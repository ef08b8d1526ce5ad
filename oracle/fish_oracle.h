/*
 * fish_oracle.h -- CPU restatement of the fish.c / poissonfunctions.c path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU library
 * (libfishgpu.so): only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The GPU library never links or calls it.
 *
 * What it restates (reference paths are inside bueler/p4pdes):
 *   - manufactured exact solutions and right-hand sides  c/ch6/fish.c:15-82
 *   - residuals Poisson{1,2,3}DFunctionLocal              c/ch6/poissonfunctions.c:4-115
 *   - Jacobians Poisson{1,2,3}DJacobianLocal (applied     c/ch6/poissonfunctions.c:117-258
 *     matrix-free, same entries as the assembled matrix)
 *   - InitialState                                        c/ch6/poissonfunctions.c:260-346
 *   - Form{1,2,3}DUExact and the error report             c/ch6/fish.c:237-340
 *   - the PETSc solver stack fish selects (SNESKSPONLY + KSPCG + PCMG with
 *     Chebyshev/Richardson level smoothers, Jacobi, ILU(0)) restated from
 *     PETSc's documented algorithms; PETSc itself is not in the reference tree.
 * Plus an independent exact direct solve of the same discrete system by
 * sine-transform diagonalisation (no solver tolerance involved).
 *
 * Arrays are dense, x fastest: index = (k*my + j)*mx + i.
 */
#ifndef FISH_ORACLE_H_
#define FISH_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_MANUPOLY = 0, OR_MANUEXP = 1, OR_ZERO = 2, OR_USER = 3 };
enum { OR_PC_NONE = 0, OR_PC_JACOBI = 1, OR_PC_MG = 2, OR_PC_ILU = 3 };
enum { OR_SMOOTH_CHEBYSHEV = 0, OR_SMOOTH_RICHARDSON = 1 };
enum { OR_NORM_PRECONDITIONED = 0, OR_NORM_UNPRECONDITIONED = 1 };

/* reasons, same numeric values as PETSc's KSPConvergedReason */
enum {
  OR_CONVERGED_RTOL = 2, OR_CONVERGED_ATOL = 3, OR_CONVERGED_ITERATING = 0,
  OR_DIVERGED_ITS = -3, OR_DIVERGED_DTOL = -4, OR_DIVERGED_INDEFINITE_PC = -8,
  OR_DIVERGED_NANORINF = -9, OR_DIVERGED_INDEFINITE_MAT = -10
};

typedef struct {
  int dim;                 /* 1, 2 or 3 */
  int mx, my, mz;          /* nodes per direction; unused directions are 1 */
  double Lx, Ly, Lz;       /* domain [0,Lx]x[0,Ly]x[0,Lz] */
  double cx, cy, cz;       /* -cx u_xx - cy u_yy - cz u_zz = f */
  int problem;             /* OR_MANUPOLY / OR_MANUEXP / OR_ZERO / OR_USER */
  const double *f_user;    /* OR_USER: f at every node */
  const double *g_user;    /* OR_USER: g at every node (boundary entries used) */
} or_grid;

typedef struct {
  or_grid grid;
  int initial_type;        /* 0 zeros, 1 random (own generator, not PETSc's) */
  int initial_gonboundary; /* 1: u0 = g on the boundary */
  double rtol, atol, dtol;
  int max_it;
  int norm_type;           /* OR_NORM_* */
  int pc_type;             /* OR_PC_* */
  int mg_levels;           /* number of levels incl. finest */
  int mg_cycles;           /* 1 = V, 2 = W */
  int smooth_type;         /* OR_SMOOTH_* */
  int smooth_its;          /* -mg_levels_ksp_max_it */
  double esteig[4];        /* emin = a*lmin + b*lmax, emax = c*lmin + d*lmax */
  double richardson_scale;
  unsigned long long seed; /* for initial_type random */
} or_opts;

typedef struct {
  int its;                 /* KSP iterations */
  int reason;              /* OR_CONVERGED_* / OR_DIVERGED_* */
  int nhist;               /* entries in hist (its+1 when converged) */
  double *hist;            /* caller-provided, length >= max_it+1 (may be NULL) */
  double fnorm0, fnorm1;   /* ||F(u0)||_2, ||F(u)||_2 */
  double errinf, err2h;    /* fish.c:254-276 */
} or_report;

/* pointwise problem functions (fish.c:15-82) */
double or_gfun(const or_grid *g, double x, double y, double z);
double or_ffun(const or_grid *g, double x, double y, double z);

long long or_nodes(const or_grid *g);
void or_spacing(const or_grid *g, double h[3]);

/* discrete operators */
void or_residual(const or_grid *g, const double *u, double *F);
void or_apply(const or_grid *g, const double *p, double *q);
void or_exact_fill(const or_grid *g, double *u);
void or_initial_state(const or_grid *g, int type, int gbdry,
                      unsigned long long seed, double *u);
void or_errnorms(const or_grid *g, const double *u, double *errinf, double *err2h);
double or_dot(const or_grid *g, const double *a, const double *b);

/* multigrid pieces on a level pair (fine grid f, coarse grid c) */
void or_restrict(const or_grid *f, const or_grid *c, const double *rf, double *bc);
void or_prolong_add(const or_grid *f, const or_grid *c, const double *xc, double *xf);
void or_cheb_bounds(const or_grid *g, const double esteig[4], double *emin, double *emax);
void or_chebyshev(const or_grid *g, double emin, double emax, int its,
                  const double *b, double *x, double *w1, double *w2, double *w3);

/* exact direct solve of J x = b (sine-transform diagonalisation) */
int or_exact_solve(const or_grid *g, const double *b, double *x);

/* KSP solve J y = b from y = 0 with the selected PC; returns 0 or -1 (bad args) */
int or_ksp_solve(const or_opts *o, const double *b, double *y, or_report *rep);
/* one V-cycle of the multigrid preconditioner of o (pc mg, o's smoother
   options) as an object: z = B r on o->grid */
void *or_mg_new(const or_opts *o);
void or_mg_apply(void *mg, const double *r, double *z);
void or_mg_free(void *mg);

/* the whole fish flow: u0, F(u0), KSP, u = u0 - y, errors.  u: output. */
int or_fish_solve(const or_opts *o, double *u, or_report *rep);

/* option parsing with fish's flag spellings; returns 0 or a nonzero code */
void or_opts_default(or_opts *o);
int or_opts_parse(or_opts *o, int argc, const char **argv, int *da_refine_out);

/* run like the reference program: parse, solve, print fish's lines to stdout */
int or_fish_main(int argc, const char **argv);

/* threads used by the OpenMP loops */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
