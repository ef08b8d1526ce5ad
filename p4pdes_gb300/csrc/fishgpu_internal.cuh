// fishgpu_internal.cuh -- shared device/host definitions of libfishgpu.so.
//
// Layout: every level vector is a dense array a[(k*my + j)*mx + i] (x fastest)
// over ALL nodes, boundary nodes included, exactly like the DMDA global vectors
// of the reference.  Kernels index with (i,j,k), never flat, so a level may
// carry a padded row pitch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fishgpu.h"

namespace fg {

// ---------------------------------------------------------------- geometry
// Stencil weights as the reference computes them:
//   1D  poissonfunctions.c:122-131  sc = cx/h,             diag = cx*(2/h)
//   2D  poissonfunctions.c:35-40    sc = cx*hy/hx, cy*hx/hy, diag = 2(scx+scy)
//   3D  poissonfunctions.c:76-82    sc = c*dvol/h^2,       diag = 2(scx+scy+scz)
struct Geom {
  int dim;
  int mx, my, mz;
  int pitch;        // elements between (j) rows
  long long plane;  // elements between (k) planes
  double x0[3];     // coordinates of node (0,0,0)
  double h[3];
  double sc[3];
  double scdiag;
  double vol;       // cell volume multiplying f in the residual
  // sc and scdiag rounded to FP32 once on the host: the FP32 kernels read
  // these instead of converting the FP64 values, a conversion the compiler
  // may repeat inside a loop (it rematerialises kernel parameters rather than
  // keep them in registers), and that runs on the FP64 pipe
  float scf[3];
  float scdiagf;
};

Geom make_geom(int dim, int mx, int my, int mz, double Lx, double Ly, double Lz,
               double cx, double cy, double cz);

__host__ __device__ inline long long gidx(const Geom &g, int i, int j, int k) {
  return (long long)k * g.plane + (long long)j * g.pitch + i;
}

// ---------------------------------------------------------------- KSP state
// Lives in device memory; kernels of a CG iteration read alpha/beta from it
// and the last block of each reduction kernel updates it (so a whole
// iteration can be captured in a CUDA graph with no host round trip).
enum {
  R_ITERATING = 0, R_CONVERGED_RTOL = 2, R_CONVERGED_ATOL = 3,
  R_DIVERGED_ITS = -3, R_DIVERGED_DTOL = -4, R_DIVERGED_INDEFINITE_PC = -8,
  R_DIVERGED_NANORINF = -9, R_DIVERGED_INDEFINITE_MAT = -10
};

enum Fin {
  FIN_STORE = 0,      // acc[q] = sum_q
  FIN_INIT_RR,        // unpreconditioned initial norm: dp = sqrt(rr), test n=0
  FIN_INIT_ZZZR,      // after B r0: (precond) dp = ||z||, test n=0; beta = z.r
  FIN_PW,             // dpi = p.w, alpha = beta/dpi
  FIN_RR,             // unpreconditioned: dp = ||r||, test n=i+1
  FIN_ZZZR,           // after B r: (precond) dp = ||z||, test; beta = z.r; i++
  FIN_PW_DEFER        // FIN_PW after a direction update that left y alone: the
                      // owed update (alpha, pend) moves to (alpha2, pend2)
};

struct KspState {
  double rtol, atol, dtol;
  int max_it, norm_type;
  int i;       // completed iterations of the CG loop
  int its;     // PETSc ksp->its
  int reason;
  int done;    // nonzero: every kernel of the iteration returns at once
  int nhist;
  int pend;    // y += alpha p deferred: 0 none, 1 in p buffer 0, 2 in p buffer 1
  int pend2;   // an older deferred y += alpha2 p (applied first), in the other buffer
  unsigned int loops;  // bodies run by the device-side solve loop (graph_loop.cuh)
  double dp, rnorm0, ttol, beta, betaold, dpi, dpiold, alpha;
  double bratio;  // beta / betaold for the next direction update (one division, in the finaliser)
  double alpha2;  // the step of the update owed in pend2
  // Mixed form, solution accumulated in FP64: the inner solve's updates go
  // straight into the outer FP64 solution as y64 += (yscale * alpha) p, with
  // yscale the refinement step's residual norm; yfresh: y64 holds nothing yet
  // (the first refinement step), so the first update writes it without reading
  double yscale;
  int yfresh;
  double acc[4];
  unsigned int *ndone;  // batches: incremented once when this instance stops
  double hist[FISHGPU_MAX_HIST];
};

// Reduction scratch: partials[slot*cap + block] and one ticket per slot.
struct Reducer {
  double *partials;
  unsigned int *tickets;
  int cap;   // capacity per value
  int tcap;  // tickets per slot (batched reductions: one per plane)
};

// ---------------------------------------------------------------- problems
// Manufactured solutions and right-hand sides of c/ch6/fish.c:15-82.
__host__ __device__ inline double prob_g(int problem, int dim, double x, double y, double z) {
  if (problem == FISHGPU_MANUPOLY) {
    double a = x * x * (1.0 - x * x);
    if (dim == 1) return a;
    double b = y * y * (y * y - 1.0);
    if (dim == 2) return a * b;
    return a * b * (z * z * (z * z - 1.0));
  }
  if (problem == FISHGPU_MANUEXP) {
    if (dim == 1) return -exp(x);
    if (dim == 2) return -x * exp(y);
    return -x * exp(y + z);
  }
  return 0.0;
}

__host__ __device__ inline double prob_f(int problem, int dim, double cx, double cy, double cz,
                                         double x, double y, double z) {
  if (problem == FISHGPU_MANUPOLY) {
    if (dim == 1) return cx * 12.0 * x * x - 2.0;
    double aa = x * x * (1.0 - x * x), bb = y * y * (y * y - 1.0);
    double ddaa = 2.0 * (1.0 - 6.0 * x * x), ddbb = 2.0 * (6.0 * y * y - 1.0);
    if (dim == 2) return -(cx * ddaa * bb + cy * aa * ddbb);
    double cc = z * z * (z * z - 1.0), ddcc = 2.0 * (6.0 * z * z - 1.0);
    return -(cx * ddaa * bb * cc + cy * aa * ddbb * cc + cz * aa * bb * ddcc);
  }
  if (problem == FISHGPU_MANUEXP) {
    if (dim == 1) return exp(x);
    if (dim == 2) return x * exp(y);
    return 2.0 * x * exp(y + z);
  }
  return 0.0;
}

// Problem description passed by value to kernels.  FISHGPU_USER arrays are
// dense (x fastest) with their own strides, whatever the pitch of the grid
// being computed on.
struct Prob {
  int problem, dim;
  double cx, cy, cz;
  const double *f, *g;  // FISHGPU_USER arrays
  long long upitch, uplane;
};

__device__ inline long long uidx(const Prob &p, int i, int j, int k) {
  return (long long)k * p.uplane + (long long)j * p.upitch + i;
}

__device__ inline double g_at(const Prob &p, const Geom &gm, int i, int j, int k) {
  if (p.problem == FISHGPU_USER) return p.g[uidx(p, i, j, k)];
  return prob_g(p.problem, p.dim, gm.x0[0] + i * gm.h[0], gm.x0[1] + j * gm.h[1],
                gm.x0[2] + k * gm.h[2]);
}
__device__ inline double f_at(const Prob &p, const Geom &gm, int i, int j, int k) {
  if (p.problem == FISHGPU_USER) return p.f[uidx(p, i, j, k)];
  return prob_f(p.problem, p.dim, p.cx, p.cy, p.cz, gm.x0[0] + i * gm.h[0],
                gm.x0[1] + j * gm.h[1], gm.x0[2] + k * gm.h[2]);
}

// ---------------------------------------------------------------- reductions
template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block sum into thread 0 (fixed tree: deterministic).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double red_sm[NV][32];
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, wid = tid >> 5, nw = (nt + 31) >> 5;
  warp_sum<NV>(v);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) red_sm[q][wid] = v[q];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = lane < nw ? red_sm[q][lane] : 0.0;
    warp_sum<NV>(v);
  }
  __syncthreads();
}

// KSPConvergedDefault: n = iteration number, rnorm = monitored norm.
__device__ inline int ksp_test(KspState *st, int n, double rnorm) {
  if (n == 0) {
    st->rnorm0 = rnorm;
    st->ttol = fmax(st->rtol * rnorm, st->atol);
  }
  if (isnan(rnorm) || isinf(rnorm)) return R_DIVERGED_NANORINF;
  if (rnorm <= st->ttol) return rnorm < st->atol ? R_CONVERGED_ATOL : R_CONVERGED_RTOL;
  if (n > 0 && rnorm >= st->dtol * st->rnorm0) return R_DIVERGED_DTOL;
  return 0;
}

__device__ inline void ksp_push(KspState *st, double dp) {
  st->dp = dp;
  if (st->nhist < FISHGPU_MAX_HIST) st->hist[st->nhist] = dp;
  st->nhist++;
}

__device__ inline void ksp_stop(KspState *st, int reason) {
  st->reason = reason;
  st->done = 1;
  if (st->ndone) atomicAdd(st->ndone, 1u);
}

// Scalar part of one KSPCG step (the PETSc cg.c algorithm), run by one thread
// of the last block of the reduction that produced `tot`.
// Not inlined: one thread runs it once per launch, and keeping its switch out
// of the stencil kernels leaves their registers to the z-march.
static __device__ __noinline__ void ksp_finalize(KspState *st, Fin fin, const double *tot, int nv, double *out) {
  if (fin == FIN_STORE) {
    if (out)
      for (int q = 0; q < nv; q++) out[q] = tot[q];
    return;
  }
  const bool precond = st->norm_type == FISHGPU_NORM_PRECONDITIONED;
  switch (fin) {
  case FIN_INIT_RR: {  // unpreconditioned: dp = ||r0||
    double dp = sqrt(tot[0]);
    ksp_push(st, dp);
    int r = ksp_test(st, 0, dp);
    if (r) { st->its = 0; ksp_stop(st, r); }
    break;
  }
  case FIN_INIT_ZZZR: {  // z0 = B r0 done: tot = {z.z, z.r}
    if (precond) {
      double dp = sqrt(tot[0]);
      ksp_push(st, dp);
      int r = ksp_test(st, 0, dp);
      if (r) { st->its = 0; ksp_stop(st, r); break; }
    }
    st->beta = tot[1];
    st->i = 0;
    if (isnan(st->beta) || isinf(st->beta)) { st->its = 1; ksp_stop(st, R_DIVERGED_NANORINF); break; }
    if (st->beta == 0.0) { st->its = 1; ksp_stop(st, R_CONVERGED_ATOL); }
    break;
  }
  case FIN_PW:
  case FIN_PW_DEFER: {  // w = A p done: tot = {p.w}; the previous y update was applied (FIN_PW) or is still owed
    if (fin == FIN_PW_DEFER) {
      st->alpha2 = st->alpha;
      st->pend2 = st->pend;
    } else {
      st->pend2 = 0;
    }
    double dpi = tot[0];
    st->its = st->i + 1;
    st->betaold = st->beta;
    st->pend = 0;
    if (isnan(dpi) || isinf(dpi)) { ksp_stop(st, R_DIVERGED_NANORINF); break; }
    if (dpi == 0.0 || (st->i > 0 && ((dpi > 0.0) != (st->dpi > 0.0)))) {
      ksp_stop(st, R_DIVERGED_INDEFINITE_MAT);
      break;
    }
    st->dpi = dpi;
    st->alpha = st->beta / dpi;
    // iteration i wrote its direction to p buffer 1 - (i & 1); y += alpha p is now owed
    st->pend = 2 - (st->i & 1);
    break;
  }
  case FIN_RR: {  // unpreconditioned norm after x += a p, r -= a w
    double dp = sqrt(tot[0]);
    ksp_push(st, dp);
    int r = ksp_test(st, st->i + 1, dp);
    if (r) ksp_stop(st, r);
    break;
  }
  case FIN_ZZZR: {  // z = B r done: tot = {z.z, z.r}
    if (precond) {
      double dp = sqrt(tot[0]);
      ksp_push(st, dp);
      int r = ksp_test(st, st->i + 1, dp);
      if (r) { ksp_stop(st, r); break; }
    }
    st->beta = tot[1];
    st->bratio = st->beta / st->betaold;
    st->i += 1;
    if (st->i >= st->max_it) { ksp_stop(st, R_DIVERGED_ITS); break; }
    if (isnan(st->beta) || isinf(st->beta)) { st->its = st->i + 1; ksp_stop(st, R_DIVERGED_NANORINF); break; }
    if (st->beta == 0.0) { st->its = st->i + 1; ksp_stop(st, R_CONVERGED_ATOL); break; }
    if (st->beta * st->betaold < 0.0) { st->its = st->i + 1; ksp_stop(st, R_DIVERGED_INDEFINITE_PC); }
    break;
  }
  default:
    break;
  }
}

// Every block stores its partial; the last block to arrive sums all partials in
// block order (deterministic) and runs the finalizer.
template <int NV>
__device__ __forceinline__ void reduce_and_finalize(double (&v)[NV], Reducer red, int slot,
                                                    KspState *st, Fin fin, double *out) {
  __shared__ bool am_last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  block_sum<NV>(v);
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) red.partials[(slot * NV + q) * red.cap + bid] = v[q];
    __threadfence();
    unsigned int t = atomicAdd(&red.tickets[(size_t)slot * (red.tcap > 1 ? red.tcap : 1)], 1u);
    am_last = (t == (unsigned)(nb - 1));
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) {
    s[q] = 0.0;
    for (int b = tid; b < nb; b += nt) s[q] += __ldcg(&red.partials[(slot * NV + q) * red.cap + b]);
  }
  block_sum<NV>(s);
  if (tid == 0) {
    red.tickets[(size_t)slot * (red.tcap > 1 ? red.tcap : 1)] = 0u;
    if (st || fin == FIN_STORE) ksp_finalize(st, fin, s, NV, out);
  }
}

// ---------------------------------------------------------------- launches
// Tiles of (32 x 8) columns (256 x 1 in 1D) by zc planes; kernels loop over
// tiles with a grid-stride loop, so gridDim.x never exceeds MAX_BLOCKS and the
// reduction scratch has a fixed capacity.
struct Tiles {
  int tx, ty, tz, zc;
};
constexpr int MAX_BLOCKS = 4096;

struct Launch {
  Tiles tm;
  dim3 grid, block;
};

// Launch shape for the box [0,nx) x [0,ny) x [0,nz) of a dim-D grid.
Launch launch_box(int dim, int nx, int ny, int nz);
inline Launch launch_for(const Geom &g) { return launch_box(g.dim, g.mx, g.my, g.mz); }

#define FG_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return FISHGPU_ERR_CUDA;    \
  } while (0)

}  // namespace fg
