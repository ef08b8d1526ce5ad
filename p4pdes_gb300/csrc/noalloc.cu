// noalloc.cu -- PoissonOperatorApplyNoAlloc_gpu: the matrix-free Jacobian
// apply with its p.q dot product, using a static device array for the
// reduction scratch instead of a per-call allocation.
//
// Who needs it: callers that may not enter the CUDA allocator once they are
// running -- for example a serving loop that reserves its whole HBM budget up
// front and admits work against it, a host framework whose own pool owns all
// device memory, or latency-critical code where an allocation could fail,
// block or synchronise.  The ordinary Poisson{1,2,3}DOperatorApply_gpu takes
// its partial-sum scratch from cudaMallocAsync on every call; this entry point
// takes it from `g_apply_scratch` below and calls no allocating routine.
//
// Limits and sharing:
//   * the array holds the partial sums of at most NOALLOC_MAX_BLOCKS blocks
//     (4096 doubles = 32 KiB) plus a 256-byte ticket area; the launch used
//     here never has more blocks (its kernel strides over tiles), and a
//     launch that would is rejected with FISHGPU_ERR_ARG;
//   * every GPU that loads the library holds the array until process exit;
//   * all calls on one device share the array: calls that overlap on the GPU
//     (different streams without ordering between them) race on it and give
//     wrong dot products.  The ticket is cleared before every launch; the
//     partial sums need no clearing (each block writes its own slot before the
//     last block reads it);
//   * every call looks the array's device address up with
//     cudaGetSymbolAddress on the current device (cheap, allocates nothing),
//     so the address stays right after a device reset; the first call on a
//     device may load the library's device code there, so make it before any
//     stream capture on that device;
//   * the stream must belong to the current device (the array's address is
//     that device's); a stream of another device is rejected with
//     FISHGPU_ERR_ARG.
#include "common.cuh"

namespace fg {

constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr size_t NOALLOC_TICKET_BYTES = 256;
constexpr size_t NOALLOC_BYTES = sizeof(double) * NOALLOC_MAX_BLOCKS + NOALLOC_TICKET_BYTES;
// launch_box caps every grid at MAX_BLOCKS blocks; the array must hold that many partial sums
static_assert(MAX_BLOCKS <= NOALLOC_MAX_BLOCKS, "the scratch array holds fewer partial sums than a launch may need");

// Host code must not use this name as an address: it is a host-side stand-in.
static __device__ __align__(256) unsigned char g_apply_scratch[NOALLOC_BYTES];

// Device address of g_apply_scratch on the current device, after checking
// that `s` belongs to that device (the legacy and per-thread default streams
// belong to whichever device is current).
static int noalloc_scratch(cudaStream_t s, unsigned char **out) {
  int dev = 0, sdev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return FISHGPU_ERR_NODEVICE;
  }
  if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
    cudaGetLastError();
    return FISHGPU_ERR_ARG;
  }
  if (sdev != dev) return FISHGPU_ERR_ARG;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_apply_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return FISHGPU_ERR_CUDA;
  }
  *out = (unsigned char *)p;
  return FISHGPU_OK;
}

template <int DIM>
static int apply_noalloc(const fishgpu_info *info, const double *p, double *q, double *pq_dot,
                         const fishgpu_ctx *user, cudaStream_t s) {
  const int m[3] = {info->mx, info->my, info->mz};
  const int st[3] = {info->xs, info->ys, info->zs};
  const int w[3] = {info->xm, info->ym, info->zm};
  for (int d = 0; d < DIM; d++) {
    if (m[d] < 2 || st[d] < 0 || w[d] < 0 || st[d] + w[d] > m[d]) return FISHGPU_ERR_ARG;
    if (!(info->xmax[d] > info->xmin[d])) return FISHGPU_ERR_ARG;
  }
  for (int d = DIM; d < 3; d++)
    if (m[d] != 1 || st[d] != 0 || w[d] != 1) return FISHGPU_ERR_ARG;
  if (!(user->cx > 0.0) || !(user->cy > 0.0) || !(user->cz > 0.0)) return FISHGPU_ERR_ARG;
  const Geom g = make_geom_box(DIM, info->mx, info->my, info->mz, info->xmin, info->xmax, user->cx, user->cy,
                               user->cz);
  const Range R{info->xs, info->ys, info->zs, info->xs + info->xm, info->ys + info->ym, info->zs + info->zm};
  if (info->xm * info->ym * info->zm == 0) {
    if (pq_dot && cudaMemsetAsync(pq_dot, 0, sizeof(double), s) != cudaSuccess) return FISHGPU_ERR_CUDA;
    return FISHGPU_OK;
  }
  const Launch L = launch_box(DIM, info->xm, info->ym, info->zm);
  if (!pq_dot) {
    k_apply<DIM, double, false><<<L.grid, L.block, 0, s>>>(g, R, L.tm, nullptr, p, q, Reducer{}, 0, FIN_STORE,
                                                          nullptr);
    return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  }
  if ((int)L.grid.x > NOALLOC_MAX_BLOCKS) return FISHGPU_ERR_ARG;  // more partial sums than the array holds
  unsigned char *base = nullptr;
  int rc = noalloc_scratch(s, &base);
  if (rc) return rc;
  Reducer red;
  red.partials = (double *)base;
  red.tickets = (unsigned int *)(base + sizeof(double) * NOALLOC_MAX_BLOCKS);
  red.cap = (int)L.grid.x;
  red.tcap = 1;
  if (cudaMemsetAsync(red.tickets, 0, NOALLOC_TICKET_BYTES, s) != cudaSuccess) return FISHGPU_ERR_CUDA;
  k_apply<DIM, double, true><<<L.grid, L.block, 0, s>>>(g, R, L.tm, nullptr, p, q, red, 0, FIN_STORE, pq_dot);
  return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
}

}  // namespace fg

extern "C" int PoissonOperatorApplyNoAlloc_gpu(const fishgpu_info *info, const double *p, double *q,
                                               double *pq_dot, const fishgpu_ctx *user, void *stream) {
  if (!info || !p || !q || !user) return FISHGPU_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  switch (info->dim) {
  case 1: return fg::apply_noalloc<1>(info, p, q, pq_dot, user, s);
  case 2: return fg::apply_noalloc<2>(info, p, q, pq_dot, user, s);
  case 3: return fg::apply_noalloc<3>(info, p, q, pq_dot, user, s);
  default: return FISHGPU_ERR_ARG;
  }
}
