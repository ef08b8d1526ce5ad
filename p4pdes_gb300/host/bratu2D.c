/*
 * bratu2D.c -- command-line driver of the GPU Newton solver for the
 * Liouville-Bratu equation -Laplace(u) - lambda e^u = 0 with the reference's
 * flags and report lines (the host side of c/ch7/solns/bratu2D.c:73-157).
 *
 *   ./bratu2D -lb_exact -snes_converged_reason -snes_monitor -da_refine 8 -snes_rtol 1e-10
 *
 * Newton with the exact Jacobian and FP32 BiCGStab + Poisson multigrid inner
 * solves (PETSc's FAS / nonlinear Gauss-Seidel options are not offered).
 * Exit status is the library status (0 on success).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fishgpu.h"

static void indent(int n) {
  for (int k = 0; k < n; k++) putchar(' ');
}

static void print_snes_norm(int tab, int it, double f) {
  indent(tab);
  if (f > 1.e-9) printf("%3d SNES Function norm %g\n", it, f);
  else if (f > 1.e-11) printf("%3d SNES Function norm %5.3e\n", it, f);
  else printf("%3d SNES Function norm < 1.e-11\n", it);
}

int main(int argc, char **argv) {
  fishgpu_ms_opts o;
  fishgpu_ms_report *rep = (fishgpu_ms_report *)calloc(1, sizeof(fishgpu_ms_report));
  int showcounts = 0, log_view = 0;
  if (!rep) return FISHGPU_ERR_NOMEM;
  fishgpu_bratu_opts_default(&o);
  int rc = fishgpu_ms_opts_parse(&o, argc - 1, (const char *const *)(argv + 1));
  if (rc) {
    fprintf(stderr, "bratu2D: %s\n", fishgpu_strerror(rc));
    free(rep);
    return rc;
  }
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "-lb_showcounts")) showcounts = 1;
    if (!strcmp(argv[a], "-log_view")) log_view = 1;
  }
  int mx = o.mx, my = o.my;
  for (int k = 0; k < o.grid_sequence; k++) {
    mx = 2 * mx - 1;
    my = 2 * my - 1;
  }
  double *u = (double *)malloc(sizeof(double) * (size_t)mx * my);
  if (!u) return FISHGPU_ERR_NOMEM;
  rc = fishgpu_ms_solve(&o, u, rep);
  if (rc && rc != FISHGPU_ERR_NOT_CONVERGED) {
    fprintf(stderr, "bratu2D: %s\n", fishgpu_strerror(rc));
    free(rep);
    free(u);
    return rc;
  }
  for (int k = 0; k < rep->ngrids; k++) {
    const int tab = 2 * (rep->ngrids - 1 - k);
    for (int it = 0; it <= rep->its[k]; it++) {
      if (o.snes_monitor) print_snes_norm(tab, it, rep->fnorm[k][it]);
      if (o.ksp_converged_reason && it < rep->its[k]) {
        indent(tab + 4);
        printf("Linear solve %s due to %s iterations %d\n", rep->ksp_reason[k][it] > 0 ? "converged" : "did not converge",
               fishgpu_reason_name(rep->ksp_reason[k][it]), rep->ksp_its[k][it]);
      }
    }
    if (o.converged_reason) {
      indent(tab);
      printf("Nonlinear solve %s due to %s iterations %d\n", rep->reason[k] > 0 ? "converged" : "did not converge",
             fishgpu_snes_reason_name(rep->reason[k]), rep->its[k]);
    }
  }
  if (showcounts)  /* residual calls as the reference counts them; no nonlinear Gauss-Seidel here */
    printf("flops = %.3e,  residual calls = %lld,  NGS calls = %d\n", 12.0 * (double)mx * my * (double)rep->nfuncs,
           rep->nfuncs, 0);
  const int last = rep->ngrids - 1;
  if (rep->errinf >= 0.0)
    printf("done on %d x %d grid:   error |u-uexact|_inf = %.3e\n", rep->m[last], rep->m[last], rep->errinf);
  else
    printf("done on %d x %d grid ...\n", rep->m[last], rep->m[last]);
  if (log_view)
    printf("solve time %.6f s, %.4e DOF/s, Newton iterations %d, inner iterations %lld\n", rep->solve_ms * 1e-3,
           (double)rep->dofs / (rep->solve_ms * 1e-3), rep->its[last], rep->total_ksp_its);
  for (int a = 1; a + 1 < argc; a++)
    if (!strcmp(argv[a], "-snes_view_solution") && !strncmp(argv[a + 1], "binary:", 7))
      if (fishgpu_petsc_vec_write(argv[a + 1] + 7, 0, u, (long long)mx * my))
        fprintf(stderr, "bratu2D: cannot write %s\n", argv[a + 1] + 7);
  free(rep);
  free(u);
  return rc;
}
