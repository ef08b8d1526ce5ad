// common.cu -- geometry, launch shapes, per-device scratch, option parsing
// and status strings of libfishgpu.so.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>


#include <cudaTypedefs.h>

#include "common.cuh"
#include "tma.cuh"

namespace fg {

// cuTensorMapEncodeTiled, looked up once through the runtime (the library
// links the runtime only)
static PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    else
      cudaGetLastError();
  });
  return fn;
}

bool tma_map_3d(CUtensorMap *map, const void *base, CUtensorMapDataType dtype, long long nx, long long ny,
                long long nz, long long row_bytes, long long plane_bytes, int bx, int by, int bz) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)row_bytes, (cuuint64_t)plane_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, dtype, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

Geom make_geom_box(int dim, int mx, int my, int mz, const double xmin[3], const double xmax[3],
                   double cx, double cy, double cz) {
  Geom g;
  memset(&g, 0, sizeof(g));
  g.dim = dim;
  g.mx = mx;
  g.my = dim >= 2 ? my : 1;
  g.mz = dim >= 3 ? mz : 1;
  g.pitch = g.mx;
  g.plane = (long long)g.mx * g.my;
  for (int d = 0; d < 3; d++) {
    g.x0[d] = d < dim ? xmin[d] : 0.0;
    g.h[d] = 1.0;
  }
  g.h[0] = (xmax[0] - xmin[0]) / (mx - 1);
  if (dim >= 2) g.h[1] = (xmax[1] - xmin[1]) / (my - 1);
  if (dim >= 3) g.h[2] = (xmax[2] - xmin[2]) / (mz - 1);
  if (dim == 1) {  // poissonfunctions.c:117-131
    g.sc[0] = cx / g.h[0];
    g.scdiag = cx * (2.0 / g.h[0]);
    g.vol = g.h[0];
  } else if (dim == 2) {  // poissonfunctions.c:35-40
    g.sc[0] = cx * g.h[1] / g.h[0];
    g.sc[1] = cy * g.h[0] / g.h[1];
    g.scdiag = 2.0 * (g.sc[0] + g.sc[1]);
    g.vol = g.h[0] * g.h[1];
  } else {  // poissonfunctions.c:72-82
    double dvol = g.h[0] * g.h[1] * g.h[2];
    g.sc[0] = cx * dvol / (g.h[0] * g.h[0]);
    g.sc[1] = cy * dvol / (g.h[1] * g.h[1]);
    g.sc[2] = cz * dvol / (g.h[2] * g.h[2]);
    g.scdiag = 2.0 * (g.sc[0] + g.sc[1] + g.sc[2]);
    g.vol = dvol;
  }
  for (int d = 0; d < 3; d++) g.scf[d] = (float)g.sc[d];
  g.scdiagf = (float)g.scdiag;
  return g;
}

Geom make_geom(int dim, int mx, int my, int mz, double Lx, double Ly, double Lz, double cx,
               double cy, double cz) {
  const double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {Lx, Ly, Lz};
  return make_geom_box(dim, mx, my, mz, lo, hi, cx, cy, cz);
}

static int g_nsm = 0;

int sm_count() {
  if (g_nsm > 0) return g_nsm;
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
  g_nsm = n;
  return n;
}

Launch launch_box(int dim, int nx, int ny, int nz) {
  Launch L;
  const int maxb = std::min(MAX_BLOCKS, sm_count() * 8);
  long long tiles;
  if (dim == 1) {
    L.block = dim3(256, 1, 1);
    L.tm = Tiles{(nx + 255) / 256, 1, 1, 1};
    tiles = L.tm.tx;
  } else {
    L.block = dim3(32, 8, 1);
    int tx = (nx + 31) / 32, ty = (ny + 7) / 8, zc = 1, tz = nz;
    if (dim == 3) {
      const long long cols = (long long)tx * ty, want = 8LL * maxb;
      zc = (int)std::max(1LL, (cols * nz + want - 1) / want);
      tz = (nz + zc - 1) / zc;
    }
    L.tm = Tiles{tx, ty, tz, zc};
    tiles = (long long)tx * ty * tz;
  }
  L.grid = dim3((unsigned)std::max(1LL, std::min(tiles, (long long)maxb)), 1, 1);
  return L;
}

}  // namespace fg

// ------------------------------------------------------------------ C ABI
extern "C" const char *fishgpu_strerror(int code) {
  switch (code) {
  case FISHGPU_OK: return "ok";
  case FISHGPU_ERR_ARG: return "invalid argument";
  case FISHGPU_ERR_CUDA: return "CUDA runtime error";
  case FISHGPU_ERR_NOMEM: return "out of device memory";
  case FISHGPU_ERR_NOT_CONVERGED: return "linear solve did not converge";
  case FISHGPU_ERR_NONFINITE: return "non-finite value in the solve";
  case FISHGPU_ERR_TIMEOUT: return "device-side wait timed out";
  case FISHGPU_ERR_UNSUPPORTED: return "option not supported by the GPU library";
  case FISHGPU_ERR_NODEVICE: return "no usable CUDA device";
  default: return "unknown status";
  }
}

extern "C" const char *fishgpu_reason_name(int r) {
  switch (r) {
  case 2: return "CONVERGED_RTOL";
  case 3: return "CONVERGED_ATOL";
  case -3: return "DIVERGED_ITS";
  case -4: return "DIVERGED_DTOL";
  case -8: return "DIVERGED_INDEFINITE_PC";
  case -9: return "DIVERGED_NANORINF";
  case -10: return "DIVERGED_INDEFINITE_MAT";
  default: return "CONVERGED_ITERATING";
  }
}

extern "C" int fishgpu_opts_default(fishgpu_opts *o) {
  if (!o) return FISHGPU_ERR_ARG;
  memset(o, 0, sizeof(*o));
  o->ctx.dim = 2;                      // fish.c:140
  o->ctx.problem = FISHGPU_MANUEXP;    // fish.c:141
  o->ctx.Lx = o->ctx.Ly = o->ctx.Lz = 1.0;  // fish.c:148-150
  o->ctx.cx = o->ctx.cy = o->ctx.cz = 1.0;  // fish.c:151-153
  o->mx = o->my = o->mz = 3;           // DMDACreate{1,2,3}d with 3 nodes per side, fish.c:199-213
  o->my = 3;
  o->initial_type = FISHGPU_INITIAL_ZEROS;
  o->initial_gonboundary = 1;
  o->rtol = 1e-5;                      // PETSc KSP defaults
  o->atol = 1e-50;
  o->dtol = 1e5;
  o->max_it = 10000;
  o->norm_type = FISHGPU_NORM_PRECONDITIONED;
  o->pc_type = FISHGPU_PC_MG;
  o->mg_levels = 0;
  o->mg_cycles = 1;
  o->smooth_type = FISHGPU_SMOOTH_CHEBYSHEV;
  o->smooth_its = 2;                   // PCMG default smoothing steps
  o->esteig[0] = 0.0;
  o->esteig[1] = 0.1;
  o->esteig[2] = 0.0;
  o->esteig[3] = 1.1;
  o->richardson_scale = 1.0;
  o->precision = FISHGPU_FP64;
  o->inner_rtol = 1e-6;
  o->inner_max_it = 100;
  o->outer_max_it = 30;
  o->graph_iters = 0;
  o->fuse_smooth = 0;
  o->device_loop = 1;
  o->first_floor_scale = 0.3;
  o->inner_accurate = -1;
  o->fuse_restrict = 0;
  o->tma_apply = 0;
  o->vtail = 1;
  o->persist = -1;
  o->fuse_cgr = 1;
  o->coop_tail = 0;
  o->pair_y = 1;
  return FISHGPU_OK;
}

static int parse_bool(const char *s) {
  if (!strcmp(s, "0") || !strcasecmp(s, "false") || !strcasecmp(s, "no")) return 0;
  return 1;
}

static int is_value(const char *v) {
  if (!v) return 0;
  if (v[0] != '-') return 1;
  return (v[1] >= '0' && v[1] <= '9') || v[1] == '.';
}

extern "C" int fishgpu_opts_parse(fishgpu_opts *o, int argc, const char *const *argv) {
  if (!o || argc < 0 || (argc > 0 && !argv)) return FISHGPU_ERR_ARG;
  int refine = 0, base[3] = {3, 3, 3}, levels = 0;
  for (int a = 0; a < argc; a++) {
    const char *k = argv[a];
    const char *v = (a + 1 < argc) ? argv[a + 1] : NULL;
    const int hv = is_value(v);
    if (!k) return FISHGPU_ERR_ARG;
#define NEEDV() \
  if (!hv) return FISHGPU_ERR_ARG; \
  a++;
    if (!strcmp(k, "-fsh_dim")) { NEEDV(); o->ctx.dim = atoi(v); }
    else if (!strcmp(k, "-fsh_problem")) {
      NEEDV();
      if (!strcmp(v, "manupoly")) o->ctx.problem = FISHGPU_MANUPOLY;
      else if (!strcmp(v, "manuexp")) o->ctx.problem = FISHGPU_MANUEXP;
      else if (!strcmp(v, "zero")) o->ctx.problem = FISHGPU_ZERO;
      else return FISHGPU_ERR_ARG;
    }
    else if (!strcmp(k, "-fsh_cx")) { NEEDV(); o->ctx.cx = atof(v); }
    else if (!strcmp(k, "-fsh_cy")) { NEEDV(); o->ctx.cy = atof(v); }
    else if (!strcmp(k, "-fsh_cz")) { NEEDV(); o->ctx.cz = atof(v); }
    else if (!strcmp(k, "-fsh_Lx")) { NEEDV(); o->ctx.Lx = atof(v); }
    else if (!strcmp(k, "-fsh_Ly")) { NEEDV(); o->ctx.Ly = atof(v); }
    else if (!strcmp(k, "-fsh_Lz")) { NEEDV(); o->ctx.Lz = atof(v); }
    else if (!strcmp(k, "-fsh_initial_type")) {
      NEEDV();
      if (!strcmp(v, "zeros")) o->initial_type = FISHGPU_INITIAL_ZEROS;
      else if (!strcmp(v, "random")) o->initial_type = FISHGPU_INITIAL_RANDOM;
      else return FISHGPU_ERR_ARG;
    }
    else if (!strcmp(k, "-fsh_initial_gonboundary")) {
      if (v && v[0] != '-') { o->initial_gonboundary = parse_bool(v); a++; }
      else o->initial_gonboundary = 1;
    }
    else if (!strcmp(k, "-fsh_seed")) { NEEDV(); o->seed = strtoull(v, NULL, 10); }
    else if (!strcmp(k, "-fsh_precision")) {
      NEEDV();
      if (!strcmp(v, "fp64")) o->precision = FISHGPU_FP64;
      else if (!strcmp(v, "mixed")) o->precision = FISHGPU_MIXED;
      else return FISHGPU_ERR_ARG;
    }
    else if (!strcmp(k, "-fsh_inner_rtol")) { NEEDV(); o->inner_rtol = atof(v); }
    else if (!strcmp(k, "-fsh_inner_max_it")) { NEEDV(); o->inner_max_it = atoi(v); }
    else if (!strcmp(k, "-fsh_outer_max_it")) { NEEDV(); o->outer_max_it = atoi(v); }
    else if (!strcmp(k, "-fsh_graph_iters")) { NEEDV(); o->graph_iters = atoi(v); }
    else if (!strcmp(k, "-fsh_fuse_smooth")) { NEEDV(); o->fuse_smooth = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_device_loop")) { NEEDV(); o->device_loop = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_loop_cap")) { NEEDV(); o->loop_cap = atoi(v); }
    else if (!strcmp(k, "-fsh_first_floor")) { NEEDV(); o->first_floor_scale = atof(v); }
    else if (!strcmp(k, "-fsh_fuse_restrict")) { NEEDV(); o->fuse_restrict = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_tma_apply")) { NEEDV(); o->tma_apply = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_vtail")) { NEEDV(); o->vtail = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_vtail_points")) { NEEDV(); o->vtail_points = atoi(v); }
    else if (!strcmp(k, "-fsh_persist")) { NEEDV(); o->persist = atoi(v) < 0 ? -1 : atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_persist_points")) { NEEDV(); o->persist_points = atoi(v); }
    else if (!strcmp(k, "-fsh_persist_tail")) { NEEDV(); o->persist_tail = atoi(v); }
    else if (!strcmp(k, "-fsh_fuse_cgr")) { NEEDV(); o->fuse_cgr = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_coop_tail")) { NEEDV(); o->coop_tail = atoi(v); }
    else if (!strcmp(k, "-fsh_pair_y")) { NEEDV(); o->pair_y = atoi(v) != 0; }
    else if (!strcmp(k, "-fsh_inner_accurate")) { NEEDV(); o->inner_accurate = atoi(v) < 0 ? -1 : atoi(v) != 0; }
    else if (!strcmp(k, "-da_refine")) { NEEDV(); refine = atoi(v); }
    else if (!strcmp(k, "-da_grid_x")) { NEEDV(); base[0] = atoi(v); }
    else if (!strcmp(k, "-da_grid_y")) { NEEDV(); base[1] = atoi(v); }
    else if (!strcmp(k, "-da_grid_z")) { NEEDV(); base[2] = atoi(v); }
    else if (!strcmp(k, "-ksp_rtol")) { NEEDV(); o->rtol = atof(v); }
    else if (!strcmp(k, "-ksp_atol")) { NEEDV(); o->atol = atof(v); }
    else if (!strcmp(k, "-ksp_divtol")) { NEEDV(); o->dtol = atof(v); }
    else if (!strcmp(k, "-ksp_max_it")) { NEEDV(); o->max_it = atoi(v); }
    else if (!strcmp(k, "-ksp_type")) { NEEDV(); if (strcmp(v, "cg")) return FISHGPU_ERR_UNSUPPORTED; }
    else if (!strcmp(k, "-ksp_norm_type")) {
      NEEDV();
      if (!strcmp(v, "preconditioned")) o->norm_type = FISHGPU_NORM_PRECONDITIONED;
      else if (!strcmp(v, "unpreconditioned")) o->norm_type = FISHGPU_NORM_UNPRECONDITIONED;
      else return FISHGPU_ERR_UNSUPPORTED;
    }
    else if (!strcmp(k, "-pc_type")) {
      NEEDV();
      if (!strcmp(v, "mg")) o->pc_type = FISHGPU_PC_MG;
      else if (!strcmp(v, "jacobi")) o->pc_type = FISHGPU_PC_JACOBI;
      else if (!strcmp(v, "none")) o->pc_type = FISHGPU_PC_NONE;
      else return FISHGPU_ERR_UNSUPPORTED;
    }
    else if (!strcmp(k, "-pc_mg_levels")) { NEEDV(); levels = atoi(v); }
    else if (!strcmp(k, "-pc_mg_cycle_type")) {
      NEEDV();
      if (!strcmp(v, "v")) o->mg_cycles = 1;
      else if (!strcmp(v, "w")) o->mg_cycles = 2;
      else return FISHGPU_ERR_ARG;
    }
    else if (!strcmp(k, "-mg_levels_ksp_type")) {
      NEEDV();
      if (!strcmp(v, "chebyshev")) o->smooth_type = FISHGPU_SMOOTH_CHEBYSHEV;
      else if (!strcmp(v, "richardson")) o->smooth_type = FISHGPU_SMOOTH_RICHARDSON;
      else return FISHGPU_ERR_UNSUPPORTED;
    }
    else if (!strcmp(k, "-mg_levels_pc_type")) { NEEDV(); if (strcmp(v, "jacobi")) return FISHGPU_ERR_UNSUPPORTED; }
    else if (!strcmp(k, "-mg_levels_ksp_max_it")) { NEEDV(); o->smooth_its = atoi(v); }
    else if (!strcmp(k, "-mg_levels_ksp_richardson_scale")) { NEEDV(); o->richardson_scale = atof(v); }
    else if (!strcmp(k, "-mg_levels_ksp_chebyshev_esteig")) {
      NEEDV();
      if (sscanf(v, "%lf,%lf,%lf,%lf", &o->esteig[0], &o->esteig[1], &o->esteig[2], &o->esteig[3]) != 4)
        return FISHGPU_ERR_ARG;
    }
    else if (!strcmp(k, "-ksp_monitor")) o->monitor = 1;
    else if (!strcmp(k, "-ksp_converged_reason")) o->converged_reason = 1;
    else if (!strcmp(k, "-snes_monitor") || !strcmp(k, "-snes_monitor_short")) o->snes_monitor = 1;
#undef NEEDV
  }
  const int dim = o->ctx.dim;
  if (dim < 1 || dim > 3) return FISHGPU_ERR_ARG;                               // fish.c:214-216
  if (o->ctx.cx <= 0.0 || o->ctx.cy <= 0.0 || o->ctx.cz <= 0.0) return FISHGPU_ERR_ARG;  // fish.c:188-190
  if (o->ctx.problem == FISHGPU_MANUEXP && (o->ctx.cx != 1.0 || o->ctx.cy != 1.0 || o->ctx.cz != 1.0))
    return FISHGPU_ERR_ARG;                                                      // fish.c:191-193
  if (refine < 0 || refine > 20 || o->smooth_its < 1 || o->max_it < 0) return FISHGPU_ERR_ARG;
  int m[3] = {1, 1, 1};
  for (int d = 0; d < dim; d++) {
    if (base[d] < 2) return FISHGPU_ERR_ARG;
    long long md = (long long)(base[d] - 1) * (1LL << refine) + 1;
    if (md > (1LL << 30)) return FISHGPU_ERR_ARG;
    m[d] = (int)md;
  }
  o->mx = m[0];
  o->my = m[1];
  o->mz = m[2];
  o->da_refine = refine;
  o->mg_levels = levels > 0 ? levels : refine + 1;
  return FISHGPU_OK;
}
