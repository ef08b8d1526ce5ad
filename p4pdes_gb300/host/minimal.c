/*
 * minimal.c -- command-line driver of the GPU minimal-surface solver with the
 * reference's flags and report lines (the host side of c/ch7/minimal.c:56-191).
 *
 *   ./minimal -snes_converged_reason -snes_grid_sequence 2 -ms_monitor -ms_quaddegree 2
 *   ./minimal -da_refine 9 -snes_rtol 1e-10 -log_view
 *
 * With grid sequencing, the reports of coarser grids are indented two spaces
 * per remaining refinement, as PETSc's tabbed viewers print them.  Exit
 * status is the library status (0 on success).
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
  int log_view = 0;
  if (!rep) return FISHGPU_ERR_NOMEM;
  fishgpu_ms_opts_default(&o);
  int rc = fishgpu_ms_opts_parse(&o, argc - 1, (const char *const *)(argv + 1));
  if (rc) {
    fprintf(stderr, "minimal: %s\n", fishgpu_strerror(rc));
    return rc;
  }
  for (int a = 1; a < argc; a++)
    if (!strcmp(argv[a], "-log_view")) log_view = 1;
  int mx = o.mx, my = o.my;
  for (int k = 0; k < o.grid_sequence; k++) {
    mx = 2 * mx - 1;
    my = 2 * my - 1;
  }
  double *u = (double *)malloc(sizeof(double) * (size_t)mx * my);
  if (!u) return FISHGPU_ERR_NOMEM;
  rc = fishgpu_ms_solve(&o, u, rep);
  if (rc && rc != FISHGPU_ERR_NOT_CONVERGED) {
    fprintf(stderr, "minimal: %s\n", fishgpu_strerror(rc));
    free(rep);
    free(u);
    return rc;
  }
  for (int k = 0; k < rep->ngrids; k++) {
    const int tab = 2 * (rep->ngrids - 1 - k);
    for (int it = 0; it <= rep->its[k]; it++) {
      if (o.snes_monitor) print_snes_norm(tab, it, rep->fnorm[k][it]);
      if (o.monitor_degree > 0) {
        indent(tab);
        printf("area = %.8f; %.4f <= D <= %.4f\n", rep->area[k][it][0], rep->area[k][it][1], rep->area[k][it][2]);
      }
      if (o.ksp_converged_reason && it < rep->its[k]) {
        indent(tab + 4);
        if (rep->ksp_reason[k][it] > 0)
          printf("Linear solve converged due to %s iterations %d\n", fishgpu_reason_name(rep->ksp_reason[k][it]),
                 rep->ksp_its[k][it]);
        else
          printf("Linear solve did not converge due to %s iterations %d\n",
                 fishgpu_reason_name(rep->ksp_reason[k][it]), rep->ksp_its[k][it]);
      }
    }
    if (o.converged_reason) {
      indent(tab + 2);
      if (rep->reason[k] > 0)
        printf("Nonlinear solve converged due to %s iterations %d\n", fishgpu_snes_reason_name(rep->reason[k]),
               rep->its[k]);
      else
        printf("Nonlinear solve did not converge due to %s iterations %d\n",
               fishgpu_snes_reason_name(rep->reason[k]), rep->its[k]);
    }
  }
  const int last = rep->ngrids - 1;
  printf("done on %d x %d grid and problem %s", rep->m[last], rep->m[last],
         o.ctx.problem == FISHGPU_MS_CATENOID ? "catenoid" : "tent");
  if (rep->errinf >= 0.0) printf(":  error |u-uexact|_inf = %.5e\n", rep->errinf);
  else printf(" ...\n");
  if (log_view)
    printf("solve time %.6f s, %.4e DOF/s, Newton iterations %d, inner iterations %lld\n", rep->solve_ms * 1e-3,
           (double)rep->dofs / (rep->solve_ms * 1e-3), rep->its[last], rep->total_ksp_its);
  for (int a = 1; a + 1 < argc; a++)  /* -snes_view_solution binary:FILE (PETSc binary Vec, natural order) */
    if (!strcmp(argv[a], "-snes_view_solution") && !strncmp(argv[a + 1], "binary:", 7)) {
      const int wrc = fishgpu_petsc_vec_write(argv[a + 1] + 7, 0, u, (long long)mx * my);
      if (wrc) fprintf(stderr, "minimal: cannot write %s\n", argv[a + 1] + 7);
    }
  free(rep);
  free(u);
  return rc;
}
