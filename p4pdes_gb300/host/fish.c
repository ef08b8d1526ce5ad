/*
 * fish.c -- command-line driver of libfishgpu.so with the reference's flags
 * and report lines (the host side of c/ch6/fish.c:128-286).
 *
 *   ./fish -fsh_dim 3 -fsh_problem manupoly -da_refine 8 -pc_type mg \
 *          -mg_levels_ksp_type chebyshev -mg_levels_pc_type jacobi -ksp_rtol 1e-10
 *
 * Additional flags: -fsh_precision fp64|mixed, -log_view (prints the solve
 * time and DOF/s).  Exit status is the library status (0 on success).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fishgpu.h"

static void print_snes_norm(int it, double f) {
  /* -snes_monitor_short formatting */
  if (f > 1.e-9) printf("%3d SNES Function norm %g\n", it, f);
  else if (f > 1.e-11) printf("%3d SNES Function norm %5.3e\n", it, f);
  else printf("%3d SNES Function norm < 1.e-11\n", it);
}

int main(int argc, char **argv) {
  fishgpu_opts o;
  fishgpu_report rep;
  int rc, log_view = 0;
  fishgpu_opts_default(&o);
  rc = fishgpu_opts_parse(&o, argc - 1, (const char *const *)(argv + 1));
  if (rc) {
    fprintf(stderr, "fish: %s\n", fishgpu_strerror(rc));
    return rc;
  }
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "-log_view")) log_view = 1;
    if (!strcmp(argv[a], "-pc_mg_galerkin"))
      fprintf(stderr, "fish: -pc_mg_galerkin ignored (level operators are rediscretised)\n");
  }
  const int dim = o.ctx.dim;
  const size_t N = (size_t)o.mx * (dim >= 2 ? o.my : 1) * (dim >= 3 ? o.mz : 1);
  double *u = (double *)malloc(sizeof(double) * N);
  if (!u) return FISHGPU_ERR_NOMEM;
  rc = fishgpu_solve_host(&o, NULL, NULL, u, &rep);
  if (rc && rc != FISHGPU_ERR_NOT_CONVERGED) {
    fprintf(stderr, "fish: %s\n", fishgpu_strerror(rc));
    free(u);
    return rc;
  }
  if (o.snes_monitor) print_snes_norm(0, rep.fnorm0);
  if (o.monitor) {
    int n = rep.nhist < FISHGPU_MAX_HIST ? rep.nhist : FISHGPU_MAX_HIST;
    if (o.precision == FISHGPU_MIXED) /* refinement steps: FP64 true residual and inner CG iterations */
      for (int i = 0; i < n; i++)
        printf("    %d refinement residual norm %g (inner iterations %d)\n", i, rep.hist[i],
               i > 0 && i - 1 < FISHGPU_MAX_OUTER ? rep.inner_its[i - 1] : 0);
    else
      for (int i = 0; i < n; i++) printf("    %d KSP Residual norm %g\n", i, rep.hist[i]);
  }
  if (o.converged_reason) {
    if (rep.reason > 0)
      printf("    Linear solve converged due to %s iterations %d\n", fishgpu_reason_name(rep.reason), rep.its);
    else
      printf("    Linear solve did not converge due to %s iterations %d\n", fishgpu_reason_name(rep.reason),
             rep.its);
  }
  if (o.snes_monitor) print_snes_norm(1, rep.fnorm1);
  static const char *names[] = {"manupoly", "manuexp", "zero"};
  char gridstr[99];
  if (dim == 1) snprintf(gridstr, 99, "%d point 1D", o.mx);
  else if (dim == 2) snprintf(gridstr, 99, "%d x %d point 2D", o.mx, o.my);
  else snprintf(gridstr, 99, "%d x %d x %d point 3D", o.mx, o.my, o.mz);
  printf("problem %s on %s grid:\n  error |u-uexact|_inf = %.3e, |u-uexact|_h = %.3e\n",
         names[o.ctx.problem], gridstr, rep.errinf, rep.err2h);
  if (log_view)
    printf("solve time (incl. host copies) %.6f s, %.4e DOF/s, iterations %d, outer %d\n",
           rep.solve_ms * 1e-3, (double)rep.dofs / (rep.solve_ms * 1e-3), rep.its, rep.outer_its);
  for (int a = 1; a + 1 < argc; a++)  /* -snes_view_solution binary:FILE (PETSc binary Vec, natural order) */
    if (!strcmp(argv[a], "-snes_view_solution") && !strncmp(argv[a + 1], "binary:", 7)) {
      const int wrc = fishgpu_petsc_vec_write(argv[a + 1] + 7, 0, u, (long long)N);
      if (wrc) fprintf(stderr, "fish: cannot write %s\n", argv[a + 1] + 7);
    }
  free(u);
  return rc;
}
