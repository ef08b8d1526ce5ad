/*
 * obstacle.c -- command-line driver of the GPU obstacle-problem solver with
 * the reference's flags and report lines (the host side of
 * c/ch12/obstacle.c:51-183): -Laplace(u) = 0 on (-2,2)^2, u >= psi, reduced-
 * space active-set Newton (SNESVINEWTONRSLS semantics) with FP32 BiCGStab +
 * Poisson multigrid inner solves on the inactive set.
 *
 *   ./obstacle -da_refine 2 -snes_monitor_short -ksp_converged_reason
 *   ./obstacle -snes_grid_sequence 3 -snes_converged_reason -obs_dump_binary u.dat
 *
 * Exit status is the library status (0 on success).
 */
#include <math.h>
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

/* the obstacle psi of obstacle.c:15-25, for the binary dump of the lower bound */
static double psi(double x, double y) {
  const double r = sqrt(x * x + y * y), r0 = 0.9, psi0 = sqrt(1.0 - r0 * r0), dpsi0 = -r0 / psi0;
  return r <= r0 ? sqrt(1.0 - r * r) : psi0 + dpsi0 * (r - r0);
}

int main(int argc, char **argv) {
  fishgpu_ms_opts o;
  fishgpu_ms_report *rep = (fishgpu_ms_report *)calloc(1, sizeof(fishgpu_ms_report));
  const char *dump = NULL;
  int log_view = 0;
  if (!rep) return FISHGPU_ERR_NOMEM;
  fishgpu_obstacle_opts_default(&o);
  int rc = fishgpu_ms_opts_parse(&o, argc - 1, (const char *const *)(argv + 1));
  if (rc) {
    fprintf(stderr, "obstacle: %s\n", fishgpu_strerror(rc));
    free(rep);
    return rc;
  }
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "-obs_dump_binary") && a + 1 < argc) dump = argv[a + 1];
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
    fprintf(stderr, "obstacle: %s\n", fishgpu_strerror(rc));
    free(rep);
    free(u);
    return rc;
  }
  const int last = rep->ngrids - 1;
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
      indent(tab + 2);
      printf("Nonlinear solve %s due to %s iterations %d\n", rep->reason[k] > 0 ? "converged" : "did not converge",
             fishgpu_snes_reason_name(rep->reason[k]), rep->its[k]);
    }
  }
  if (dump) {  /* obstacle.c:138-145: u, then the lower bound psi */
    printf("writing u,psi in binary format to %s ...\n", dump);
    double *lo = (double *)malloc(sizeof(double) * (size_t)mx * my);
    if (lo) {
      const double dx = 4.0 / (mx - 1), dy = 4.0 / (my - 1);
      for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) lo[(size_t)j * mx + i] = psi(-2.0 + i * dx, -2.0 + j * dy);
      if (fishgpu_petsc_vec_write(dump, 0, u, (long long)mx * my) ||
          fishgpu_petsc_vec_write(dump, 1, lo, (long long)mx * my))
        fprintf(stderr, "obstacle: cannot write %s\n", dump);
      free(lo);
    }
  }
  if (rep->reason[last] <= 0) printf("WARNING: SNES not converged ... use -snes_converged_reason to check\n");
  printf("done on %d x %d grid ... %s, SNES iters = %d, last KSP iters = %d\n", rep->m[last], rep->m[last],
         fishgpu_snes_reason_name(rep->reason[last]), rep->its[last],
         rep->its[last] > 0 ? rep->ksp_its[last][rep->its[last] - 1] : 0);
  printf("errors: av |u-uexact| = %.3e, |u-uexact|_inf = %.3e, active area error = %.3f%%\n", rep->err1,
         rep->errinf, 100.0 * rep->active_area_err);
  if (log_view)
    printf("solve time %.6f s, %.4e DOF/s, Newton iterations %d, inner iterations %lld\n", rep->solve_ms * 1e-3,
           (double)rep->dofs / (rep->solve_ms * 1e-3), rep->its[last], rep->total_ksp_its);
  free(rep);
  free(u);
  return rc;
}
