// callbacks.cu -- the drop-in DMDA local call-backs of libfishgpu.so:
// residual (Poisson{1,2,3}DFunctionLocal), matrix-free Jacobian apply,
// exact solution, initial state and the error report, all FP64.
#include <math.h>

#include "common.cuh"

namespace fg {

static int check_info(const fishgpu_info *info, int dim) {
  if (!info || info->dim != dim) return FISHGPU_ERR_ARG;
  const int m[3] = {info->mx, info->my, info->mz};
  const int s[3] = {info->xs, info->ys, info->zs};
  const int w[3] = {info->xm, info->ym, info->zm};
  for (int d = 0; d < dim; d++) {
    if (m[d] < 2) return FISHGPU_ERR_ARG;
    if (s[d] < 0 || w[d] < 0 || s[d] + w[d] > m[d]) return FISHGPU_ERR_ARG;
    if (!(info->xmax[d] > info->xmin[d])) return FISHGPU_ERR_ARG;
  }
  for (int d = dim; d < 3; d++)
    if (m[d] != 1 || s[d] != 0 || w[d] != 1) return FISHGPU_ERR_ARG;
  return FISHGPU_OK;
}

static int make_prob(const fishgpu_ctx *user, int dim, Prob *pb) {
  if (!user) return FISHGPU_ERR_ARG;
  if (user->problem < FISHGPU_MANUPOLY || user->problem > FISHGPU_USER) return FISHGPU_ERR_ARG;
  if (user->problem == FISHGPU_USER && (!user->f || !user->g)) return FISHGPU_ERR_ARG;
  if (!(user->cx > 0.0) || !(user->cy > 0.0) || !(user->cz > 0.0)) return FISHGPU_ERR_ARG;
  pb->problem = user->problem;
  pb->dim = dim;
  pb->cx = user->cx;
  pb->cy = user->cy;
  pb->cz = user->cz;
  pb->f = user->f;
  pb->g = user->g;
  pb->upitch = 0;  // set from the grid by the caller
  pb->uplane = 0;
  return FISHGPU_OK;
}

static Geom info_geom(const fishgpu_info *info, const fishgpu_ctx *user) {
  return make_geom_box(info->dim, info->mx, info->my, info->mz, info->xmin, info->xmax, user->cx,
                       user->cy, user->cz);
}

static Range info_range(const fishgpu_info *info) {
  return Range{info->xs, info->ys, info->zs, info->xs + info->xm, info->ys + info->ym,
               info->zs + info->zm};
}

// F on the owned range.  Boundary rows scdiag*(u - g); interior rows read g
// at boundary neighbours (c/ch6/poissonfunctions.c:10-19, :43-59, :86-106).
// USERP: FISHGPU_USER f and g read directly (the problem-generic accessors
// would carry the built-in problems' FP64 transcendentals into the loop).
template <int DIM, bool USERP>
__global__ void __launch_bounds__(256) k_funclocal(Geom g, Range R, Tiles tm, Prob pb,
                                                   const double *__restrict__ u,
                                                   double *__restrict__ F) {
  auto fa = [&](int i, int j, int k) -> double {
    if constexpr (USERP) return pb.f[uidx(pb, i, j, k)];
    else return f_at(pb, g, i, j, k);
  };
  auto ga = [&](int i, int j, int k) -> double {
    if constexpr (USERP) return pb.g[uidx(pb, i, j, k)];
    else return g_at(pb, g, i, j, k);
  };
  FG_POINT_LOOP_BEGIN(R)
  const double uc = u[n];
  if (on_bdry<DIM>(g, i, j, k)) {
    double v = uc - ga(i, j, k);
    F[n] = v * g.scdiag;
  } else {
    const double ue = (i + 1 == g.mx - 1) ? ga(i + 1, j, k) : u[n + 1];
    const double uw = (i - 1 == 0) ? ga(i - 1, j, k) : u[n - 1];
    if (DIM == 1) {
      F[n] = pb.cx * (2.0 * uc - uw - ue) / g.h[0] - g.h[0] * fa(i, j, k);
    } else {
      const double un = (j + 1 == g.my - 1) ? ga(i, j + 1, k) : u[n + g.pitch];
      const double us = (j - 1 == 0) ? ga(i, j - 1, k) : u[n - g.pitch];
      if (DIM == 2) {
        F[n] = g.scdiag * uc - g.sc[0] * (uw + ue) - g.sc[1] * (us + un) - g.vol * fa(i, j, k);
      } else {
        const double uu = (k + 1 == g.mz - 1) ? ga(i, j, k + 1) : u[n + g.plane];
        const double ud = (k - 1 == 0) ? ga(i, j, k - 1) : u[n - g.plane];
        F[n] = g.scdiag * uc - g.sc[0] * (uw + ue) - g.sc[1] * (us + un) - g.sc[2] * (uu + ud) -
               g.vol * fa(i, j, k);
      }
    }
  }
  FG_POINT_LOOP_END
}

template <int DIM>
__global__ void __launch_bounds__(256) k_uexact(Geom g, Range R, Tiles tm, Prob pb,
                                                double *__restrict__ u) {
  FG_POINT_LOOP_BEGIN(R)
  u[n] = g_at(pb, g, i, j, k);
  FG_POINT_LOOP_END
}

// splitmix64 of (seed ^ dense index), mapped to [0,1) with 53 bits
__device__ __forceinline__ double uniform01(unsigned long long seed, unsigned long long idx) {
  unsigned long long x = (seed ^ idx) + 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return (double)(x >> 11) * 0x1.0p-53;
}

template <int DIM>
__global__ void __launch_bounds__(256) k_initial(Geom g, Range R, Tiles tm, Prob pb, int type,
                                                 int gbdry, unsigned long long seed,
                                                 double *__restrict__ u) {
  FG_POINT_LOOP_BEGIN(R)
  const unsigned long long dense = ((unsigned long long)k * g.my + j) * g.mx + i;
  double v = type == FISHGPU_INITIAL_RANDOM ? uniform01(seed, dense) : 0.0;
  if (gbdry && on_bdry<DIM>(g, i, j, k)) v = g_at(pb, g, i, j, k);
  u[n] = v;
  FG_POINT_LOOP_END
}

// sum of (u - uexact)^2 reduced; max |u - uexact| by an atomic max on the
// bit pattern (non-negative doubles order like their bit patterns)
template <int DIM>
__global__ void __launch_bounds__(256) k_errnorm(Geom g, Range R, Tiles tm, Prob pb,
                                                 const double *__restrict__ u, Reducer red,
                                                 double *out, unsigned long long *maxbits) {
  double s = 0.0, mx = 0.0;
  FG_POINT_LOOP_BEGIN(R)
  const double e = u[n] - g_at(pb, g, i, j, k);
  s = fma(e, e, s);
  mx = fmax(mx, fabs(e));
  FG_POINT_LOOP_END
  __shared__ double bmax[32];
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  double wm = warp_max(mx);
  if ((tid & 31) == 0) bmax[tid >> 5] = wm;
  __syncthreads();
  if (tid == 0) {
    double b = 0.0;
    for (int q = 0; q < (int)((blockDim.x * blockDim.y + 31) / 32); q++) b = fmax(b, bmax[q]);
    atomicMax(maxbits, (unsigned long long)__double_as_longlong(b));
  }
  double v1[1] = {s};
  reduce_and_finalize<1>(v1, red, 0, nullptr, FIN_STORE, out);
}

#define FG_DIM_SWITCH(dim, CALL) \
  switch (dim) {                 \
  case 1: { constexpr int D = 1; CALL; } break; \
  case 2: { constexpr int D = 2; CALL; } break; \
  default: { constexpr int D = 3; CALL; } break; \
  }

template <int DIM>
static int funclocal(const fishgpu_info *info, const double *au, double *aF, const fishgpu_ctx *user,
                     void *stream) {
  int rc = check_info(info, DIM);
  if (rc) return rc;
  Prob pb;
  if ((rc = make_prob(user, DIM, &pb))) return rc;
  if (!au || !aF) return FISHGPU_ERR_ARG;
  if (info->xm * info->ym * info->zm == 0) return FISHGPU_OK;
  const Geom g = info_geom(info, user);
  pb.upitch = g.pitch;
  pb.uplane = g.plane;
  const Range R = info_range(info);
  const Launch L = launch_box(DIM, info->xm, info->ym, info->zm);
  if (pb.problem == FISHGPU_USER)
    k_funclocal<DIM, true><<<L.grid, L.block, 0, (cudaStream_t)stream>>>(g, R, L.tm, pb, au, aF);
  else
    k_funclocal<DIM, false><<<L.grid, L.block, 0, (cudaStream_t)stream>>>(g, R, L.tm, pb, au, aF);
  return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
}

// Reduction scratch for one call: partials + ticket, stream-ordered.
static int scratch_alloc(cudaStream_t s, int nblocks, int nv, Reducer *red, double **extra,
                         int nextra) {
  const size_t part = sizeof(double) * (size_t)nv * nblocks;
  const size_t bytes = part + 64 + sizeof(double) * (size_t)nextra;
  char *p = nullptr;
  if (cudaMallocAsync((void **)&p, bytes, s) != cudaSuccess) return FISHGPU_ERR_NOMEM;
  red->partials = (double *)p;
  red->tickets = (unsigned int *)(p + part);
  red->cap = nblocks;
  red->tcap = 1;
  if (extra) *extra = (double *)(p + part + 64);
  if (cudaMemsetAsync(p + part, 0, 64 + sizeof(double) * (size_t)nextra, s) != cudaSuccess)
    return FISHGPU_ERR_CUDA;
  return FISHGPU_OK;
}

template <int DIM>
static int opapply(const fishgpu_info *info, const double *p, double *q, double *pq_dot,
                   const fishgpu_ctx *user, void *stream) {
  int rc = check_info(info, DIM);
  if (rc) return rc;
  Prob pb;
  if ((rc = make_prob(user, DIM, &pb))) return rc;
  if (!p || !q) return FISHGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const Geom g = info_geom(info, user);
  pb.upitch = g.pitch;
  pb.uplane = g.plane;
  const Range R = info_range(info);
  const Launch L = launch_box(DIM, info->xm, info->ym, info->zm);
  if (info->xm * info->ym * info->zm == 0) {
    if (pq_dot && cudaMemsetAsync(pq_dot, 0, sizeof(double), s) != cudaSuccess) return FISHGPU_ERR_CUDA;
    return FISHGPU_OK;
  }
  if (!pq_dot) {
    k_apply<DIM, double, false><<<L.grid, L.block, 0, s>>>(g, R, L.tm, nullptr, p, q, Reducer{}, 0,
                                                          FIN_STORE, nullptr);
    return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  }
  Reducer red;
  if ((rc = scratch_alloc(s, (int)L.grid.x, 1, &red, nullptr, 0))) return rc;
  k_apply<DIM, double, true><<<L.grid, L.block, 0, s>>>(g, R, L.tm, nullptr, p, q, red, 0, FIN_STORE,
                                                       pq_dot);
  rc = cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  if (cudaFreeAsync(red.partials, s) != cudaSuccess) rc = FISHGPU_ERR_CUDA;
  return rc;
}

}  // namespace fg

using namespace fg;

extern "C" int Poisson1DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                                          const fishgpu_ctx *user, void *stream) {
  return funclocal<1>(info, au, aF, user, stream);
}
extern "C" int Poisson2DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                                          const fishgpu_ctx *user, void *stream) {
  return funclocal<2>(info, au, aF, user, stream);
}
extern "C" int Poisson3DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                                          const fishgpu_ctx *user, void *stream) {
  return funclocal<3>(info, au, aF, user, stream);
}
extern "C" int Poisson1DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                                          double *pq_dot, const fishgpu_ctx *user, void *stream) {
  return opapply<1>(info, p, q, pq_dot, user, stream);
}
extern "C" int Poisson2DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                                          double *pq_dot, const fishgpu_ctx *user, void *stream) {
  return opapply<2>(info, p, q, pq_dot, user, stream);
}
extern "C" int Poisson3DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                                          double *pq_dot, const fishgpu_ctx *user, void *stream) {
  return opapply<3>(info, p, q, pq_dot, user, stream);
}

extern "C" int FormUExact_gpu(const fishgpu_info *info, double *u, const fishgpu_ctx *user,
                              void *stream) {
  if (!info || !u) return FISHGPU_ERR_ARG;
  int rc = check_info(info, info->dim);
  if (rc) return rc;
  Prob pb;
  if ((rc = make_prob(user, info->dim, &pb))) return rc;
  if (info->xm * info->ym * info->zm == 0) return FISHGPU_OK;
  const Geom g = info_geom(info, user);
  pb.upitch = g.pitch;
  pb.uplane = g.plane;
  const Range R = info_range(info);
  const Launch L = launch_box(info->dim, info->xm, info->ym, info->zm);
  cudaStream_t s = (cudaStream_t)stream;
  FG_DIM_SWITCH(info->dim, (k_uexact<D><<<L.grid, L.block, 0, s>>>(g, R, L.tm, pb, u)));
  return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
}

extern "C" int InitialState_gpu(const fishgpu_info *info, int initial_type, int gbdry,
                                unsigned long long seed, double *u, const fishgpu_ctx *user,
                                void *stream) {
  if (!info || !u) return FISHGPU_ERR_ARG;
  if (initial_type != FISHGPU_INITIAL_ZEROS && initial_type != FISHGPU_INITIAL_RANDOM)
    return FISHGPU_ERR_ARG;  // poissonfunctions.c:371-372
  int rc = check_info(info, info->dim);
  if (rc) return rc;
  Prob pb;
  if ((rc = make_prob(user, info->dim, &pb))) return rc;
  if (info->xm * info->ym * info->zm == 0) return FISHGPU_OK;
  const Geom g = info_geom(info, user);
  pb.upitch = g.pitch;
  pb.uplane = g.plane;
  const Range R = info_range(info);
  const Launch L = launch_box(info->dim, info->xm, info->ym, info->zm);
  cudaStream_t s = (cudaStream_t)stream;
  FG_DIM_SWITCH(info->dim,
                (k_initial<D><<<L.grid, L.block, 0, s>>>(g, R, L.tm, pb, initial_type, gbdry, seed, u)));
  return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
}

extern "C" int ErrorNorms_gpu(const fishgpu_info *info, const double *u, const fishgpu_ctx *user,
                              double *errinf, double *err2h, void *stream) {
  if (!info || !u || !errinf || !err2h) return FISHGPU_ERR_ARG;
  int rc = check_info(info, info->dim);
  if (rc) return rc;
  Prob pb;
  if ((rc = make_prob(user, info->dim, &pb))) return rc;
  const Geom g = info_geom(info, user);
  pb.upitch = g.pitch;
  pb.uplane = g.plane;
  const Range R = info_range(info);
  const Launch L = launch_box(info->dim, info->xm, info->ym, info->zm);
  cudaStream_t s = (cudaStream_t)stream;
  Reducer red;
  double *extra = nullptr;
  if ((rc = scratch_alloc(s, (int)L.grid.x, 1, &red, &extra, 2))) return rc;
  FG_DIM_SWITCH(info->dim, (k_errnorm<D><<<L.grid, L.block, 0, s>>>(
                               g, R, L.tm, pb, u, red, extra, (unsigned long long *)(extra + 1))));
  double h[2] = {0.0, 0.0};
  rc = cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  if (!rc && cudaMemcpyAsync(h, extra, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = FISHGPU_ERR_CUDA;
  if (cudaFreeAsync(red.partials, s) != cudaSuccess) rc = FISHGPU_ERR_CUDA;
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = FISHGPU_ERR_CUDA;
  if (rc) return rc;
  double normconst = (double)(info->mx - 1);  // fish.c:260-276
  if (info->dim >= 2) normconst *= (double)(info->my - 1);
  if (info->dim >= 3) normconst *= (double)(info->mz - 1);
  *errinf = h[1];  // the slot holds the bit pattern of the largest |e|
  *err2h = sqrt(h[0]) / sqrt(normconst);
  return FISHGPU_OK;
}
