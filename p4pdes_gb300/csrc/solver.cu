// solver.cu -- device-resident CG + geometric multigrid for the fish solve.
//
// Replaces the PETSc stack fish selects (c/ch6/fish.c:223-239: SNESKSPONLY,
// KSPCG, -pc_type mg) with project code:
//   * KSP: CG with PETSc's cg.c semantics (preconditioned or unpreconditioned
//     norm, KSPConvergedDefault test), all scalars on the device;
//   * PC: multiplicative V/W cycles over the DMDA hierarchy
//     (m_c = (m_f-1)/2+1), rediscretised level operators (fish.c:7),
//     Q1 interpolation P and restriction P^T, Chebyshev/Jacobi or
//     Richardson/Jacobi smoothing with a nonzero initial guess, exact
//     coarse solve (single block);
//   * the KSP set-up and one CG iteration are captured once as CUDA graphs.
// Forms: FISHGPU_FP64 (everything FP64; the twin of the CPU oracle) and
// FISHGPU_MIXED (FP64 iterative refinement: FP64 true residual, norms and
// solution update; FP32 inner CG with an FP32 V-cycle).
//
// Internal vectors use the padded layout of vkernels.cuh (row pitch a
// multiple of 4, zero padding); the caller's u is dense and is packed /
// unpacked at the ends of a solve.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "graph_loop.cuh"
#include "mg_hooks.cuh"
#include "vblock.cuh"
#include "vkernels.cuh"

namespace fg {

constexpr int MAX_LEVELS = 24;
constexpr int ZC = 32;            // k-planes per block in the 3D stencil kernels
constexpr int FLAT_BLOCKS = 4096; // grid cap of the pointwise kernels

template <typename T>
struct Level {
  Post2Z pz{};     // launch shape of the fused two-step post-smoother (3D FP32)
  Geom g;      // padded pitch
  Slots sl;    // pointwise kernels and grid transfers
  Slots st;    // stencils: sl, or the 2D row march for batches
  T *b = nullptr, *r = nullptr;
  T *X[3] = {nullptr, nullptr, nullptr};  // rotating iterate buffers
  int cur = 0;                            // buffer holding the iterate (enqueue time)
  double emin = 0.0, emax = 0.0;
  // coarsest level only
  T *S[3] = {nullptr, nullptr, nullptr};
  T *ilam = nullptr, *work = nullptr;
  int n[3] = {1, 1, 1};
};

template <typename T>
struct Hier {
  int nlev = 0;
  Level<T> lev[MAX_LEVELS];
  T *zbuf = nullptr;  // z for the Jacobi / none preconditioners
  T *z = nullptr;     // where the preconditioner leaves z (fixed per option set)
  TailLevel<T> *tail = nullptr;  // device: levels 0 .. tail_top of the one-block V-cycle tail
  int tail_top = 0;              // 0: no tail
  int tail_threads = 0;
  size_t tail_smem = 0;    // dynamic shared memory of k_vtail: the coarse solve's scratch and the tail's copy
  size_t tail_coarse = 0;  // the coarse solve's scratch (0: its work area in global memory)
  int tail_copy = -1;      // offset of the tail's copy (-1: the tail works in global memory)
  // the persistent solve (k_ksp_persist): every level, the fine one's b the KSP residual
  TailLevel<T> *plev = nullptr;  // device, levels 0 .. nlev-1; null: no persistent solve
  int pbtop = 0;                 // levels pbtop .. 0 in block 0
  size_t psmem = 0;              // dynamic shared memory of the persistent solve (coarse scratch, tail copy)
  size_t pcoarse = 0;            // the coarse solve's scratch (0: its work area in global memory)
  int pcopy = -1;                // offset of block 0's tail copy (-1: none)
  // the cooperative V-cycle tail (k_vtail_coop): levels 0 .. ctail_top in one launch
  int ctail_top = 0;  // 0: none
  int ctail_blocks = 0;
  size_t ctail_smem = 0;
  PersistArgs<T> ctail{};  // its level table, coarse solve and barrier (no KSP vectors)
};

// Threads per block of the slot kernels of a level: 128 on 2D grids (twice
// the blocks of 256, spreading the FP64 kernels of a 257^2 .. 1025^2 grid over
// more SMs: measured 1.50 -> 1.35 ms at 257^2, 3.33 -> 3.13 ms at 1025^2 for
// the FP64 solve, the mixed form unchanged; 64 and 32 were no better)
static int level_chunk(const Geom &g, int batch) {
  return g.dim == 2 && !batch ? 128 : 256;
}

static Geom padded(Geom g) {
  g.pitch = (g.mx + 3) / 4 * 4;
  g.plane = (long long)g.pitch * g.my;
  return g;
}

// Whether the inner FP32 solves of the mixed form use the accurate form
// (v_cgp_apply's ACC): asked for (1, 0), or, by default (-1), when the
// standard form cannot finish in two refinement steps: its first step stops
// near 0.3 kappa 2^-24 and a second one reduces by inner_rtol at best.
static bool inner_accurate_for(int choice, double rtol, double inner_rtol, double kappa) {
  if (choice >= 0) return choice != 0;
  return rtol < 0.3 * kappa * 0x1.0p-24 * inner_rtol;
}

// Exact spectrum ends of D^{-1}A for the constant-diagonal stencil:
// 1 -+ sum_d (2 sc_d / scdiag) cos(pi/(m_d-1)); boundary rows give 1.
static void spectrum(const Geom &g, double *lmin, double *lmax) {
  const int m[3] = {g.mx, g.my, g.mz};
  bool interior = true;
  for (int d = 0; d < g.dim; d++)
    if (m[d] < 3) interior = false;
  double s = 0.0;
  if (interior)
    for (int d = 0; d < g.dim; d++) s += 2.0 * g.sc[d] / g.scdiag * cos(M_PI / (m[d] - 1));
  *lmax = fmax(1.0, 1.0 + s);
  *lmin = fmin(1.0, 1.0 - s);
}

static Geom coarsen(const Geom &f, const fishgpu_ctx &c) {
  return padded(make_geom(f.dim, (f.mx - 1) / 2 + 1, f.dim >= 2 ? (f.my - 1) / 2 + 1 : 1,
                          f.dim >= 3 ? (f.mz - 1) / 2 + 1 : 1, c.Lx, c.Ly, c.Lz, c.cx, c.cy, c.cz));
}

static size_t nelem(const Geom &g) { return (size_t)g.plane * g.mz; }

static unsigned flat_grid(long long tot4) {
  long long b = (tot4 + 255) / 256;
  if (b > FLAT_BLOCKS) b = FLAT_BLOCKS;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace fg

using namespace fg;

struct fishgpu_solver_s {
  fishgpu_opts o;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Geom fine;       // padded
  Geom dense;      // the caller's layout (pitch = mx)
  Slots sf;        // slots of the fine level
  Slots sfst;      // stencil slots of the fine level (sf, or the fine level's row march)
  Launch Lf;       // scalar launch over the fine grid
  unsigned gfl = 1;  // grid of the pointwise kernels on the fine level
  Prob prob;
  KspState *st = nullptr;    // device
  KspState *st_h = nullptr;  // pinned host mirror
  Reducer red;
  double *dval = nullptr;    // device scalars for FIN_STORE results
  double *hval = nullptr;    // pinned host copy
  Hier<double> h64;
  Hier<float> h32;
  // FP64 vectors (padded): u, KSP vectors (FP64 form) / outer vectors (mixed)
  double *u64 = nullptr, *r64 = nullptr, *p64 = nullptr, *q64 = nullptr, *w64 = nullptr, *y64 = nullptr;
  double *b64 = nullptr;
  double *beff = nullptr;    // F(u) = A u - beff (vol*f plus the boundary data of the eliminated columns)
  bool beff_ready = false;   // built-in problems: computed once
  // FP32 inner KSP vectors (mixed form)
  float *r32 = nullptr, *p32 = nullptr, *q32 = nullptr, *w32 = nullptr, *y32 = nullptr;
  float *r32b = nullptr;   // second CG residual buffer of the FP32 inner solves (fuse_cgr_ok)
  cudaGraphExec_t gexec = nullptr;       // giters CG iterations
  cudaGraphExec_t gloop = nullptr;       // the same repeated on the device until the solve stops
  bool loop_refused = false;             // the driver refused the device loop: poll from the host
  long long n_loop = 0;                  // kernel nodes of one body of gloop
  cudaGraphExec_t gexec_init = nullptr;  // the KSP set-up sequence
  cudaGraphExec_t gexec_init64[2] = {nullptr, nullptr};  // the same from b64 / r64 (mixed form)
  long long n_init = 0, n_iter = 0;      // kernel nodes of the two graphs
  long long launches = 0;                // kernels launched by the current solve
  int giters = 1;
  int ksp_norm = FISHGPU_NORM_PRECONDITIONED;  // norm of the CG loop the graphs are built for
  double *f_own = nullptr, *g_own = nullptr, *u_own = nullptr;  // FISHGPU_USER, host-array form
  // fishgpu_solver_solve_host_many: device staging of the next f and the last u, and their copy streams
  double *f_stage = nullptr, *u_stage = nullptr;
  cudaStream_t cs_in = nullptr, cs_out = nullptr;
  // batch groups: 2D instances of one size stacked as k-planes
  int batch = 0, nplanes = 1;
  unsigned int *ndone = nullptr;
  double *scl = nullptr, *iscl = nullptr;    // per-plane refinement scales (device)
  std::vector<void *> allocs;
  long long bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int *fault = nullptr;  // set by a kernel whose bounded wait on a copy gave up
  // persistent solve: grid barrier, partial sums, blocks (one per SM at most)
  unsigned *pbar = nullptr;
  double *ppart = nullptr;
  int pblocks = 0;
  // the mixed solve in one launch (k_mixed_persist): its report, device and pinned host
  fg::MixedOut *mout = nullptr, *mout_h = nullptr;
  // another solver's persistent kernel on this hierarchy (solver_persist32): its level table
  fg::TailLevel<float> *hplev = nullptr;
};

namespace fg {

template <typename T>
static int dalloc(fishgpu_solver *S, T **p, size_t n) {
  void *q = nullptr;
  const size_t bytes = (sizeof(T) * (n ? n : 1) + 255) / 256 * 256;
  if (cudaMalloc(&q, bytes) != cudaSuccess) {
    cudaGetLastError();
    return FISHGPU_ERR_NOMEM;
  }
  S->allocs.push_back(q);
  S->bytes += (long long)bytes;
  if (cudaMemsetAsync(q, 0, bytes, S->stream) != cudaSuccess) return FISHGPU_ERR_CUDA;
  *p = (T *)q;
  return FISHGPU_OK;
}

// Rows per thread of the batch stencils (2D instances stacked as planes): the
// planes give the parallelism, so a thread can march a strip of rows with the
// y-neighbours in registers.  A function of the instance size only, so an
// instance is decomposed alike alone and in any batch.  Swept at 820
// instances per size: 16 rows beat 8 and 32 at 257^2-513^2, 8 is best at
// 65^2-129^2 and 4 at 33^2.
static int batch_rows(const Geom &g) {
  if (g.dim != 2) return 0;
  return g.mx >= 257 ? 16 : g.mx >= 65 ? 8 : g.mx >= 33 ? 4 : 0;  // measured per size: 4096-instance batch
}

// Levels up to tail_max_points nodes (per instance) below the finest run as
// the one-block V-cycle tail.  One SM then does the level's work, so the
// level must be small enough that a phase costs less than a launch (about
// one point per thread): up to 33^2 / 9^3 nodes.  Swept (limits 300, 1200,
// 5000, 17000 nodes) on 2D 257^2 and 3D 129^3 / 513^3 solves: 1200 is best
// or level with the best in both precisions; 17000 (129^2) took the 2D
// FP64 solve from 2.4 to 4.0 ms (FP64 on one SM is slow on this part).
static long long tail_max_points(const fishgpu_opts &o, size_t) {
  return o.vtail_points > 0 ? o.vtail_points : 1200;
}

static long long level_points(const Geom &g) { return (long long)g.mx * g.my * (g.dim >= 3 ? g.mz : 1); }

// A level's arrays and enq_smooth's Chebyshev coefficients (the same
// expressions) for the block-level V-cycle code.
template <typename T>
static TailLevel<T> tail_level(const Level<T> &lv, bool smoothed) {
  TailLevel<T> t;
  memset(&t, 0, sizeof(t));
  t.g = lv.g;
  t.b = lv.b;
  t.r = lv.r;
  for (int q = 0; q < 3; q++) t.X[q] = lv.X[q];
  if (!smoothed) return t;
  const double dinv = 1.0 / lv.g.scdiag;
  const double scale = 2.0 / (lv.emax + lv.emin);
  const double alpha = 1.0 - scale * lv.emin;
  const double mu = 1.0 / alpha, omegaprod = 2.0 / alpha;
  const double c1 = scale * dinv;
  {
    const double ckp1 = 2.0 * mu * mu - 1.0, omega = omegaprod * mu / ckp1;
    t.a0 = (T)(2.0 * omega * c1);
    t.a1 = (T)(omega * c1 * c1);
  }
  t.c1 = (T)c1;
  {
    const double ckm1 = 1.0, ck = mu;
    const double ckp1 = 2.0 * mu * ck - ckm1;
    const double omega = omegaprod * ck / ckp1;
    t.ckm1 = (T)(1.0 - omega);
    t.ck = (T)omega;
    t.crd = (T)(omega * c1);
  }
  return t;
}

// ------------------------------------------------------------------ V-cycle tail
// The coarse end of a V-cycle in ONE block per grid (per instance of a
// batch): vtail_body's phases, a block barrier between them instead of a
// launch each; bit-identical to the launch-per-phase form.
template <int DIM, typename T>
__global__ void __launch_bounds__(1024) k_vtail(const TailLevel<T> *__restrict__ tl, int top, KspState *st, int batch,
                                                const T *__restrict__ S0, const T *__restrict__ S1,
                                                const T *__restrict__ S2, const T *__restrict__ ilam, T *work, int n0,
                                                int n1, int n2, int smem, T dinv, int copy_off) {
  extern __shared__ __align__(16) unsigned char fg_tail_sm[];
  __shared__ TailLevel<T> sv[MAX_LEVELS];
  const int plane = (DIM < 3 && batch) ? (int)blockIdx.x : 0;  // instance of a batch
  if (batch && st) st += plane;
  if (ksp_done(st)) return;
  if (copy_off >= 0) {
    vtail_prepare<DIM, T>(tl, top, fg_tail_sm, copy_off, sv);
    __syncthreads();
  }
  vtail_run<DIM, T>(tl, top, plane, S0, S1, S2, ilam, work, n0, n1, n2, smem, dinv, fg_tail_sm, copy_off, sv);
}

// Dynamic shared memory of a block-level V-cycle over levels 0..top with
// pts[l] nodes per grid: the coarse solve's scratch (when it fits 48 KB) and
// the copy of the tail's arrays (when the whole fits kTailSmemMax).
constexpr size_t kTailSmemMax = 160 * 1024;
static void tail_smem_plan(int dim, const int *n, size_t es, int top, const long long *pts, size_t *coarse,
                           int *copy_off, size_t *total) {
  const size_t smb = es * (size_t)(3 * (size_t)n[0] * n[1] * n[2] + (size_t)n[0] * n[0] +
                                   (dim >= 2 ? (size_t)n[1] * n[1] : 0) + (dim >= 3 ? (size_t)n[2] * n[2] : 0));
  *coarse = ((long long)n[0] * n[1] * n[2] > 0 && smb <= 48 * 1024) ? smb : 0;
  const size_t off = (*coarse + 15) / 16 * 16;
  size_t copy = 0;
  for (int l = 0; l <= top; l++) copy += (size_t)tail_copy_elems(l, pts[l]) * es;
  if (off + copy <= kTailSmemMax) {
    *copy_off = (int)off;
    *total = off + copy;
  } else {
    *copy_off = -1;
    *total = *coarse;
  }
}

// Lets `fn` take `bytes` of dynamic shared memory; false if the device refuses.
static bool allow_smem(const void *fn, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) return true;
  cudaGetLastError();
  return false;
}

// The V-cycle tail of a hierarchy (k_vtail): the largest level below the
// finest with at most TAIL_MAX_POINTS nodes per instance and everything
// under it, for V-cycles of two Chebyshev/Jacobi steps (the default
// smoother; other smoothers keep a launch per phase).
template <typename T>
static int build_tail(fishgpu_solver *S, Hier<T> &H) {
  const fishgpu_opts &o = S->o;
  H.tail_top = 0;
  if (!o.vtail || o.pc_type != FISHGPU_PC_MG || o.smooth_type != FISHGPU_SMOOTH_CHEBYSHEV || o.smooth_its != 2 ||
      o.mg_cycles != 1 || S->fine.dim < 2 || H.nlev < 3)
    return FISHGPU_OK;
  int top = 0;
  for (int l = 1; l <= H.nlev - 2; l++)
    if (level_points(H.lev[l].g) <= tail_max_points(o, sizeof(T))) top = l;
  if (top < 1) return FISHGPU_OK;
  std::vector<TailLevel<T>> tl(top + 1);
  for (int l = 0; l <= top; l++) tl[l] = tail_level<T>(H.lev[l], l > 0);
  // the level's b of the top level is the restriction target of the level
  // above it (allocated); levels below the finest all have r
  int rc;
  if ((rc = dalloc(S, &H.tail, (size_t)(top + 1)))) return rc;
  if (cudaMemcpyAsync(H.tail, tl.data(), sizeof(TailLevel<T>) * (top + 1), cudaMemcpyHostToDevice, S->stream) !=
      cudaSuccess)
    return FISHGPU_ERR_CUDA;
  const long long per = level_points(H.lev[top].g);
  H.tail_threads = (int)std::min<long long>(1024, std::max<long long>(64, (per + 31) / 32 * 32));
  std::vector<long long> pts(top + 1);
  for (int l = 0; l <= top; l++) pts[l] = level_points(H.lev[l].g);
  tail_smem_plan(S->fine.dim, H.lev[0].n, sizeof(T), top, pts.data(), &H.tail_coarse, &H.tail_copy, &H.tail_smem);
  const void *fn = S->fine.dim == 2 ? (const void *)k_vtail<2, T> : (const void *)k_vtail<3, T>;
  if (!allow_smem(fn, H.tail_smem)) {
    H.tail_copy = -1;
    H.tail_smem = H.tail_coarse;
  }
  H.tail_top = top;
  return FISHGPU_OK;
}

// Whether a solve's CG loop runs as one persistent launch (k_ksp_persist):
// CG + MG with two Chebyshev/Jacobi steps, V-cycles, a 2D or 3D single grid,
// the device loop, and (default) a finest grid of at most persist_points
// nodes (by default 2.5e6 in FP64, 5e5 in FP32).  The levels of at most
// persist_tail nodes run in block 0 between two grid barriers (*btop: the
// largest of them, >= 1): one SM's FP64 rate is 1/152 of the GPU's, so in
// FP64 only the smallest levels stay there.  pts: nodes per level
// (0 .. nlev-1); cn: the coarsest level's interior sizes.  Returns the
// blocks of the launch (one of 512 threads per SM at most, fewer for fewer
// fine points), 0 for no persistent solve; *nsm: the device's SMs (the
// partial sums' capacity); *coarse, *copy_off, *psmem: the dynamic shared
// memory plan (tail_smem_plan) for block 0's tail.
template <typename T>
static int persist_shape(const fishgpu_opts &o, int dim, bool batch, int nlev, const long long *pts, const int *cn,
                         int *btop, int *nsm, size_t *coarse, int *copy_off, size_t *psmem) {
  if (!o.persist || !o.device_loop || batch || o.pc_type != FISHGPU_PC_MG ||
      o.smooth_type != FISHGPU_SMOOTH_CHEBYSHEV || o.smooth_its != 2 || o.mg_cycles != 1 || dim < 2 || nlev < 3 ||
      nlev > kMaxPersistLevels)
    return 0;
  const long long fine_pts = pts[nlev - 1];
  // measured against the launch-per-phase solve (2D 257^2 .. 2049^2, 3D 33^3 .. 129^3): the FP64 form
  // gains at every size up to 2.1e6 nodes (its kernels are FP64-bound there, the launch overhead is not
  // hidden); the mixed form, its refinement loop in the same launch, up to 2.7e5 nodes and loses from
  // 1.05e6 (2D 1025^2: 2.78 against 2.64 ms)
  const long long lim = o.persist_points > 0 ? o.persist_points : sizeof(T) == 8 ? 2500000 : 500000;
  if (o.persist < 0 && fine_pts > lim) return 0;
  const long long tmax = o.persist_tail > 0 ? o.persist_tail : sizeof(T) == 8 ? 300 : 1200;
  *btop = 0;
  for (int l = 1; l <= nlev - 2; l++)
    if (pts[l] <= tmax) *btop = l;
  if (*btop < 1) return 0;
  int dev = 0, coop = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop || *nsm < 1) {
    cudaGetLastError();
    return 0;
  }
  tail_smem_plan(dim, cn, sizeof(T), *btop, pts, coarse, copy_off, psmem);
  // every kernel that may run the plan: the CG solve, and in FP32 its accurate
  // form and the whole mixed solve in both forms
  std::vector<const void *> fns{dim == 2 ? (const void *)k_ksp_persist<2, T, false>
                                         : (const void *)k_ksp_persist<3, T, false>};
  if constexpr (sizeof(T) == 4) {
    fns.push_back(dim == 2 ? (const void *)k_ksp_persist<2, T, true> : (const void *)k_ksp_persist<3, T, true>);
    fns.push_back(dim == 2 ? (const void *)k_mixed_persist<2, true> : (const void *)k_mixed_persist<3, true>);
    fns.push_back(dim == 2 ? (const void *)k_mixed_persist<2, false> : (const void *)k_mixed_persist<3, false>);
  }
  bool ok = true;
  for (const void *fn : fns) ok = ok && allow_smem(fn, *psmem);
  if (!ok) {
    *copy_off = -1;
    *psmem = *coarse;
  }
  for (const void *fn : fns)
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 512, *psmem) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      return 0;
    }
  int blocks = (int)std::max<long long>(1, std::min<long long>(*nsm, (fine_pts + 511) / 512));
  return blocks;
}

template <typename T>
static int build_persist(fishgpu_solver *S, Hier<T> &H) {
  H.plev = nullptr;
  std::vector<long long> pts(H.nlev);
  for (int l = 0; l < H.nlev; l++) pts[l] = level_points(H.lev[l].g);
  int btop = 0, nsm = 0, copy_off = -1;
  size_t coarse = 0, psmem = 0;
  const int blocks = persist_shape<T>(S->o, S->fine.dim, S->batch != 0, H.nlev, pts.data(), H.lev[0].n, &btop, &nsm,
                                      &coarse, &copy_off, &psmem);
  if (!blocks) return FISHGPU_OK;
  std::vector<TailLevel<T>> tl(H.nlev);
  for (int l = 0; l < H.nlev; l++) tl[l] = tail_level<T>(H.lev[l], l > 0);
  tl[H.nlev - 1].b = sizeof(T) == 8 ? (T *)(void *)S->r64 : (T *)(void *)S->r32;  // the KSP residual
  int rc;
  if ((rc = dalloc(S, &H.plev, (size_t)H.nlev))) return rc;
  if (cudaMemcpyAsync(H.plev, tl.data(), sizeof(TailLevel<T>) * H.nlev, cudaMemcpyHostToDevice, S->stream) !=
      cudaSuccess)
    return FISHGPU_ERR_CUDA;
  if (!S->pbar && ((rc = dalloc(S, &S->pbar, 2)) || (rc = dalloc(S, &S->ppart, (size_t)4 * nsm)))) return rc;
  if (sizeof(T) == 4 && S->o.precision == FISHGPU_MIXED && !S->mout) {  // the whole mixed solve in one launch
    if ((rc = dalloc(S, &S->mout, 1))) return rc;
    if (cudaMallocHost((void **)&S->mout_h, sizeof(MixedOut)) != cudaSuccess) return FISHGPU_ERR_NOMEM;
  }
  H.pbtop = btop;
  H.psmem = psmem;
  H.pcoarse = coarse;
  H.pcopy = copy_off;
  S->pblocks = blocks;
  return FISHGPU_OK;
}

// The cooperative V-cycle tail of a launch-per-phase solve of a single grid:
// levels up to coop_tail nodes below the finest (the largest of them and
// everything under it) as one launch of k_vtail_coop, for V-cycles of two
// Chebyshev/Jacobi steps.  Below it, levels of at most 1200 (FP32) / 300
// (FP64) nodes run in block 0, as in the persistent solve.  Only when it
// reaches above the one-block tail (k_vtail).
template <typename T>
static int build_ctail(fishgpu_solver *S, Hier<T> &H) {
  const fishgpu_opts &o = S->o;
  H.ctail_top = 0;
  const int dim = S->fine.dim;
  if (!o.coop_tail || S->batch || !S->fault || o.pc_type != FISHGPU_PC_MG || o.smooth_type != FISHGPU_SMOOTH_CHEBYSHEV ||
      o.smooth_its != 2 || o.mg_cycles != 1 || dim < 2 || H.nlev < 3 || H.nlev > kMaxPersistLevels)
    return FISHGPU_OK;
  const long long lim = o.coop_tail > 0 ? o.coop_tail : FISHGPU_COOP_TAIL_POINTS;
  std::vector<long long> pts(H.nlev);
  for (int l = 0; l < H.nlev; l++) pts[l] = level_points(H.lev[l].g);
  int top = 0;
  for (int l = 1; l <= H.nlev - 2; l++)
    if (pts[l] <= lim) top = l;
  if (top <= H.tail_top) return FISHGPU_OK;
  const long long tmax = sizeof(T) == 8 ? 300 : 1200;
  int btop = 0;
  for (int l = 1; l < top; l++)
    if (pts[l] <= tmax) btop = l;
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop || nsm < 1) {
    cudaGetLastError();
    return FISHGPU_OK;
  }
  size_t coarse = 0, psmem = 0;
  int copy_off = -1;
  tail_smem_plan(dim, H.lev[0].n, sizeof(T), btop, pts.data(), &coarse, &copy_off, &psmem);
  const void *fn = dim == 2 ? (const void *)k_vtail_coop<2, T> : (const void *)k_vtail_coop<3, T>;
  if (!allow_smem(fn, psmem)) {
    copy_off = -1;
    psmem = coarse;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 512, psmem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return FISHGPU_OK;
  }
  std::vector<TailLevel<T>> tl(top + 1);
  for (int l = 0; l <= top; l++) tl[l] = tail_level<T>(H.lev[l], l > 0);
  TailLevel<T> *dtl = nullptr;
  int rc;
  if ((rc = dalloc(S, &dtl, (size_t)(top + 1)))) return rc;
  if (cudaMemcpyAsync(dtl, tl.data(), sizeof(TailLevel<T>) * (top + 1), cudaMemcpyHostToDevice, S->stream) !=
      cudaSuccess)
    return FISHGPU_ERR_CUDA;
  if (!S->pbar && ((rc = dalloc(S, &S->pbar, 2)) || (rc = dalloc(S, &S->ppart, (size_t)4 * nsm)))) return rc;
  PersistArgs<T> &a = H.ctail;
  memset(&a, 0, sizeof(a));
  a.lv = dtl;
  a.top = top;
  a.btop = btop;
  a.part = S->ppart;
  a.bar = S->pbar;
  a.fault = S->fault;
  const Level<T> &c = H.lev[0];
  a.S0 = c.S[0];
  a.S1 = c.S[1];
  a.S2 = c.S[2];
  a.ilam = c.ilam;
  a.work = c.work;
  a.n0 = c.n[0];
  a.n1 = c.n[1];
  a.n2 = c.n[2];
  a.smem = coarse ? 1 : 0;
  a.dinv = (T)(1.0 / c.g.scdiag);
  a.copy_off = copy_off;
  H.ctail_blocks = (int)std::max<long long>(1, std::min<long long>(nsm, (pts[top] + 511) / 512));
  H.ctail_smem = psmem;
  H.ctail_top = top;
  return FISHGPU_OK;
}

template <typename T>
static int build_hier(fishgpu_solver *S, Hier<T> &H) {
  const fishgpu_opts &o = S->o;
  int rc;
  if (o.pc_type != FISHGPU_PC_MG) {  // Jacobi / none: z has its own buffer
    H.nlev = 1;
    H.lev[0].g = S->fine;
    H.lev[0].sl = S->sf;
    return dalloc(S, &H.zbuf, nelem(S->fine));
  }
  const int L = o.mg_levels;
  if (L < 1 || L > MAX_LEVELS) return FISHGPU_ERR_ARG;
  H.nlev = L;
  Geom g = S->fine;
  for (int l = L - 1; l >= 0; l--) {
    Level<T> &lv = H.lev[l];
    if (S->batch) g.mz = S->nplanes;  // a batch keeps its instances as planes on every level
    lv.g = g;
    lv.sl = make_slots(g, ZC, 2432, level_chunk(g, S->batch), S->batch);
    lv.st = S->batch ? make_slots(g, ZC, 2432, 256, 1, batch_rows(g)) : lv.sl;
    if (g.dim == 3) lv.pz = post2z_shape(g);
    double lmin, lmax;
    spectrum(g, &lmin, &lmax);
    lv.emin = o.esteig[0] * lmin + o.esteig[1] * lmax;
    lv.emax = o.esteig[2] * lmin + o.esteig[3] * lmax;
    const size_t N = nelem(g);
    if (l < L - 1 && (rc = dalloc(S, &lv.b, N))) return rc;
    for (int q = 0; q < 3; q++)
      if ((rc = dalloc(S, &lv.X[q], N))) return rc;
    if (l > 0 && (rc = dalloc(S, &lv.r, N))) return rc;
    if (l > 0) {
      const int m[3] = {g.mx, g.my, g.mz};
      for (int d = 0; d < g.dim; d++)
        if (m[d] < 3 || (m[d] - 1) % 2 != 0) return FISHGPU_ERR_ARG;  // cannot coarsen
      g = coarsen(g, o.ctx);
    }
  }
  // coarsest level: sine-transform data for the exact solve
  Level<T> &c = H.lev[0];
  const int m[3] = {c.g.mx, c.g.my, c.g.mz};
  long long ni = 1;
  for (int d = 0; d < 3; d++) {
    c.n[d] = d < c.g.dim ? m[d] - 2 : 1;
    ni *= c.n[d] > 0 ? c.n[d] : 0;
  }
  if (ni > 300000) return FISHGPU_ERR_UNSUPPORTED;  // single-block exact solve only for small grids
  if (ni > 0) {
    std::vector<T> hS, hl((size_t)ni);
    for (int d = 0; d < c.g.dim; d++) {
      const int n = c.n[d];
      hS.assign((size_t)n * n, T(0));
      const double a = sqrt(2.0 / (n + 1));
      for (int i = 1; i <= n; i++)
        for (int k = 1; k <= n; k++) hS[(size_t)(i - 1) * n + (k - 1)] = (T)(a * sin(M_PI * (double)i * k / (n + 1)));
      if ((rc = dalloc(S, &c.S[d], (size_t)n * n))) return rc;
      // on the solver's stream: ordered after dalloc's memset of the same buffer
      // (a legacy-stream copy is not ordered with a non-blocking stream); the
      // pageable source is staged before the call returns
      if (cudaMemcpyAsync(c.S[d], hS.data(), sizeof(T) * n * n, cudaMemcpyHostToDevice, S->stream) != cudaSuccess)
        return FISHGPU_ERR_CUDA;
    }
    for (int k = 0; k < c.n[2]; k++)
      for (int j = 0; j < c.n[1]; j++)
        for (int i = 0; i < c.n[0]; i++) {
          const int q[3] = {i, j, k};
          double lam = 0.0;
          for (int d = 0; d < c.g.dim; d++) lam += c.g.sc[d] * (2.0 - 2.0 * cos(M_PI * (q[d] + 1) / (c.n[d] + 1)));
          hl[((size_t)k * c.n[1] + j) * c.n[0] + i] = (T)(1.0 / lam);
        }
    const size_t nwork = 2 * (size_t)ni * (c.g.dim < 3 ? (size_t)c.g.mz : 1);  // one work area per block
    if ((rc = dalloc(S, &c.ilam, (size_t)ni)) || (rc = dalloc(S, &c.work, nwork))) return rc;
    if (cudaMemcpyAsync(c.ilam, hl.data(), sizeof(T) * ni, cudaMemcpyHostToDevice, S->stream) != cudaSuccess)
      return FISHGPU_ERR_CUDA;
    for (int d = c.g.dim; d < 3; d++) c.S[d] = c.S[0];  // unused
  }
  if ((rc = build_tail<T>(S, H))) return rc;
  if ((rc = build_ctail<T>(S, H))) return rc;
  return build_persist<T>(S, H);
}

// ------------------------------------------------------------------ enqueue
static inline int third(int a, int b) { return 3 - a - b; }

// The accurate CG direction update + apply of a 3D FP32 grid from a TMA ring
// (v_cgp_apply_tma): false when the grid is too narrow for its tiles (less
// than one 43-slot tile per row), the reduction scratch too small for its
// blocks, or the driver refuses the tensor maps; the caller then launches
// v_cgp_apply.
static bool launch_cgp_tma(fishgpu_solver *S, const Geom &g, KspState *st, const float *z, const float *pold,
                           float *pnew, float *w, double *y, int slot) {
  if (g.dim != 3 || g.pitch / 4 < 43) return false;
  const CgTile q = cg_tile_shape(g);
  if ((int)q.blocks() > S->red.cap) return false;
  CUtensorMap zm, pm, ym;
  const long long rb = (long long)g.pitch * 4, pb = g.plane * 4LL;
  if (!tma_map_3d(&zm, z, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, g.pitch, g.my, g.mz, rb, pb, CgRing::ZW, CgRing::ZR, 1) ||
      !tma_map_3d(&pm, pold, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, g.pitch, g.my, g.mz, rb, pb, CgRing::ZW, CgRing::ZR,
                  1) ||
      !tma_map_3d(&ym, y, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, g.pitch, g.my, g.mz, rb * 2, pb * 2, CgRing::YW,
                  CgRing::YR, 1))
    return false;
  v_cgp_apply_tma<<<q.blocks(), CgRing::THREADS, CgRing::SMEM, S->stream>>>(zm, pm, ym, g, q, st, pnew, w, y, S->red,
                                                                            slot, S->fault);
  return true;
}

// b_c = P^T (b - A x) of a 3D level in one kernel (v_resid_restrict): tensor
// maps of x and b for the kernel's ring; false if the driver refuses them.
template <typename T>
static bool launch_resid_restrict(fishgpu_solver *S, const Geom &gf, const Geom &gc, const T *b, const T *x, T *bc,
                                  KspState *st) {
  using R = RRRing<T>;
  const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  CUtensorMap xm, bm;
  const long long rb = (long long)gf.pitch * sizeof(T), pb = gf.plane * (long long)sizeof(T);
  if (!tma_map_3d(&xm, x, dt, gf.pitch, gf.my, gf.mz, rb, pb, R::XW, R::XR, 1) ||
      !tma_map_3d(&bm, b, dt, gf.pitch, gf.my, gf.mz, rb, pb, R::BW, R::BR, 1))
    return false;
  const RRShape q = rr_shape(gf, gc);
  v_resid_restrict<T><<<q.blocks(), 320, R::SMEM, S->stream>>>(xm, bm, gf, gc, q, st, bc, S->fault);
  return true;
}

// Level smoother, PETSc KSPCHEBYSHEV / KSPRICHARDSON with PCJACOBI, `its`
// iterations, nonzero initial guess; from_zero: the iterate is known to be 0
// (the arithmetic is identical).  Rotates the level's three buffers.
// dots: when >= 0, the last step also reduces z.z and z.b and runs Fin(dots)
// (the CG scalar update), so the separate dot kernel is not needed.
// Smoothing step that also reduces z.z and z.b: per-plane reductions for a
// batch (2D only), one reduction over the grid otherwise.
template <int DIM, typename T, bool HAS_KM1>
static void launch_cheb_dots(fishgpu_solver *S, Level<T> &lv, const T *xkm1, const T *xk, T *out, T ckm1, T ck,
                             T crd, Fin fin) {
  const unsigned gb = slot_blocks(lv.st);
  if constexpr (DIM == 2) {
    if (S->batch) {
      v_cheb<DIM, T, HAS_KM1, true, true><<<gb, lv.st.chunk, 0, S->stream>>>(lv.g, lv.st, S->st, lv.b, xkm1, xk, out,
                                                                         ckm1, ck, crd, S->red, 0, fin);
      return;
    }
  }
  v_cheb<DIM, T, HAS_KM1, true, false><<<gb, lv.st.chunk, 0, S->stream>>>(lv.g, lv.st, S->st, lv.b, xkm1, xk, out, ckm1,
                                                                       ck, crd, S->red, 0, fin);
}

// The CG residual update of an iteration, r_new = r - alpha w, carried into
// the first smoothing pass of its V-cycle (v_cheb2_zero's RUPD form): the
// finest level's b is r_new, formed from r and w and stored there.
template <typename T>
struct RUpd {
  const T *r, *w;
  bool rr;  // unpreconditioned norm: r_new.r_new and FIN_RR
};

template <int DIM, typename T>
static void enq_smooth(fishgpu_solver *S, Level<T> &lv, bool from_zero, int dots = -1,
                       const RUpd<T> *ru = nullptr) {
  const fishgpu_opts &o = S->o;
  const Fin fin = (Fin)(dots < 0 ? 0 : dots);
  const double dinv = 1.0 / lv.g.scdiag;
  cudaStream_t s = S->stream;
  KspState *st = S->st;
  const unsigned gb = slot_blocks(lv.sl), gbs = slot_blocks(lv.st);
  const unsigned gf = flat_grid(lv.sl.tot4);
  if (o.smooth_type == FISHGPU_SMOOTH_RICHARDSON) {
    const T crd = (T)(o.richardson_scale * dinv);
    int cur = lv.cur;
    for (int it = 0; it < o.smooth_its; it++) {
      const int nxt = (cur + 1) % 3;
      const bool last = it == o.smooth_its - 1 && dots >= 0;
      if (from_zero && it == 0)
        v_scale<T><<<gb, lv.sl.chunk, 0, s>>>(lv.g, lv.sl, st, lv.b, crd, lv.X[nxt]);
      else if (last)
        launch_cheb_dots<DIM, T, false>(S, lv, nullptr, lv.X[cur], lv.X[nxt], T(0), T(1), crd, fin);
      else
        v_cheb<DIM, T, false><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, nullptr, lv.X[cur], lv.X[nxt], T(0), T(1), crd);
      cur = nxt;
    }
    lv.cur = cur;
    return;
  }
  // Chebyshev (first kind) on [emin, emax]
  const double scale = 2.0 / (lv.emax + lv.emin);
  const double alpha = 1.0 - scale * lv.emin;
  const double mu = 1.0 / alpha, omegaprod = 2.0 / alpha;
  const double c1 = scale * dinv;
  if (from_zero && o.smooth_its == 2) {
    // x1 = c1 b; x2 = omega x1 + omega c1 (b - A x1) = 2 omega c1 b - omega c1^2 (A b)
    const double ckp1 = 2.0 * mu * mu - 1.0, omega = omegaprod * mu / ckp1;
    const int nxt = (lv.cur + 1) % 3;
    if (ru && ru->rr)
      v_cheb2_zero<DIM, T, true, true><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, ru->r, lv.X[nxt],
                                                                   (T)(2.0 * omega * c1), (T)(omega * c1 * c1),
                                                                   ru->w, lv.b, S->red, 0);
    else if (ru)
      v_cheb2_zero<DIM, T, true, false><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, ru->r, lv.X[nxt],
                                                                    (T)(2.0 * omega * c1), (T)(omega * c1 * c1),
                                                                    ru->w, lv.b, S->red, 0);
    else
      v_cheb2_zero<DIM, T><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, lv.X[nxt], (T)(2.0 * omega * c1),
                                              (T)(omega * c1 * c1));
    lv.cur = nxt;
    return;
  }
  if constexpr (DIM == 3 && sizeof(T) == 4) {
    if (!from_zero && o.smooth_its == 2 && o.fuse_smooth && !S->batch && lv.pz.ok()) {
      // both steps in one temporally blocked kernel (bit-identical to the two below)
      const double ckp1 = 2.0 * mu * mu - 1.0, omega = omegaprod * mu / ckp1;
      const int km = lv.cur, out = third(km, (km + 1) % 3);
      if (dots >= 0)
        v_cheb_post2z<true><<<lv.pz.blocks(), lv.pz.threads, lv.pz.smem, s>>>(
            lv.g, lv.pz, st, (const float *)lv.b, (const float *)lv.X[km], (float *)lv.X[out], (float)c1,
            (float)(1.0 - omega), (float)omega, (float)(omega * c1), S->red, 0, fin);
      else
        v_cheb_post2z<false><<<lv.pz.blocks(), lv.pz.threads, lv.pz.smem, s>>>(
            lv.g, lv.pz, st, (const float *)lv.b, (const float *)lv.X[km], (float *)lv.X[out], (float)c1,
            (float)(1.0 - omega), (float)omega, (float)(omega * c1));
      lv.cur = out;
      return;
    }
  }
  int km1 = -1, kk;  // -1: the zero iterate
  if (from_zero) {
    kk = (lv.cur + 1) % 3;
    v_scale<T><<<gb, lv.sl.chunk, 0, s>>>(lv.g, lv.sl, st, lv.b, (T)c1, lv.X[kk]);
  } else {
    km1 = lv.cur;
    kk = (lv.cur + 1) % 3;
    if (o.smooth_its == 1 && dots >= 0)
      launch_cheb_dots<DIM, T, false>(S, lv, nullptr, lv.X[km1], lv.X[kk], T(0), T(1), (T)c1, fin);
    else
      v_cheb<DIM, T, false><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, nullptr, lv.X[km1], lv.X[kk], T(0), T(1), (T)c1);
  }
  double ckm1 = 1.0, ck = mu;
  for (int it = 1; it < o.smooth_its; it++) {
    const double ckp1 = 2.0 * mu * ck - ckm1;
    const double omega = omegaprod * ck / ckp1;
    // x_{k+1} = (1-omega) x_{k-1} + omega x_k + omega scale D^{-1}(b - A x_k)
    const int out = km1 < 0 ? (kk + 1) % 3 : third(km1, kk);
    const bool last = it == o.smooth_its - 1 && dots >= 0;
    if (km1 < 0)
      v_cheb<DIM, T, false><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, nullptr, lv.X[kk], lv.X[out], T(0), (T)omega,
                                               (T)(omega * c1));
    else if (last)
      launch_cheb_dots<DIM, T, true>(S, lv, lv.X[km1], lv.X[kk], lv.X[out], (T)(1.0 - omega), (T)omega,
                                     (T)(omega * c1), fin);
    else
      v_cheb<DIM, T, true><<<gbs, lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, lv.X[km1], lv.X[kk], lv.X[out],
                                              (T)(1.0 - omega), (T)omega, (T)(omega * c1));
    km1 = kk;
    kk = out;
    ckm1 = ck;
    ck = ckp1;
  }
  lv.cur = kk;
}

template <int DIM, typename T>
static void enq_vcycle(fishgpu_solver *S, Hier<T> &H, int l, bool from_zero, int dots = -1,
                       const RUpd<T> *ru = nullptr) {
  Level<T> &lv = H.lev[l];
  cudaStream_t s = S->stream;
  KspState *st = S->st;
  if constexpr (DIM >= 2) {
    if (l > 0 && l == H.ctail_top && from_zero && dots < 0 && !ru) {  // levels l .. 0 in one cooperative launch
      cudaMemsetAsync(H.ctail.bar, 0, 2 * sizeof(unsigned), s);
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.gridDim = dim3(H.ctail_blocks);
      cfg.blockDim = dim3(512);
      cfg.dynamicSmemBytes = H.ctail_smem;
      cfg.stream = s;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_vtail_coop<DIM, T>, H.ctail, (const KspState *)st);
      for (int q = 0; q <= l; q++) H.lev[q].cur = 0;  // every level ends with its iterate in X[0]
      return;
    }
    if (l > 0 && l == H.tail_top && from_zero && dots < 0) {  // levels l .. 0 in one block per instance
      const Level<T> &c = H.lev[0];
      k_vtail<DIM, T><<<DIM < 3 && S->batch ? (unsigned)S->nplanes : 1u, H.tail_threads, H.tail_smem, s>>>(
          H.tail, l, st, DIM < 3 ? S->batch : 0, c.S[0], c.S[1], c.S[2], c.ilam, c.work, c.n[0], c.n[1], c.n[2],
          H.tail_coarse ? 1 : 0, (T)(1.0 / c.g.scdiag), H.tail_copy);
      for (int q = 0; q <= l; q++) H.lev[q].cur = 0;  // every tail level ends with its iterate in X[0]
      return;
    }
  }
  if (l == 0) {
    lv.cur = 0;
    // a block of just enough threads (tiny coarsest grids start and synchronise
    // faster), the transforms staged in shared memory when they fit 48 KB
    const int per = lv.g.mx * lv.g.my * (DIM < 3 ? 1 : lv.g.mz), ni = lv.n[0] * lv.n[1] * lv.n[2];
    const int nt = std::min(1024, std::max(32, (std::max(per, ni) + 31) / 32 * 32));
    const size_t smb = coarse_smem_bytes<T>(DIM, lv.n[0], lv.n[1], lv.n[2]);
    const bool sm = ni > 0 && smb <= 48 * 1024;
    k_coarse<DIM, T><<<DIM < 3 ? lv.g.mz : 1, nt, sm ? smb : 0, s>>>(lv.g, st, lv.sl.batch, lv.b, lv.X[0], lv.S[0],
                                                                    lv.S[1], lv.S[2], lv.ilam, lv.work, lv.n[0],
                                                                    lv.n[1], lv.n[2], sm ? 1 : 0,
                                                                    (T)(1.0 / lv.g.scdiag));
    return;
  }
  Level<T> &lc = H.lev[l - 1];
  enq_smooth<DIM, T>(S, lv, from_zero, -1, ru);
  if (DIM == 3 && !S->batch && S->o.fuse_restrict &&
      launch_resid_restrict<T>(S, lv.g, lc.g, lv.b, lv.X[lv.cur], lc.b, st)) {  // b_c = P^T (b - A x) in one pass
  } else {
    v_resid<DIM, T><<<slot_blocks(lv.st), lv.st.chunk, 0, s>>>(lv.g, lv.st, st, lv.b, lv.X[lv.cur], lv.r);
    v_restrict<DIM, T><<<slot_blocks(lc.sl), lc.sl.chunk, 0, s>>>(lv.g, lc.g, lc.sl, st, lv.r, lc.b);
  }
  for (int c = 0; c < S->o.mg_cycles; c++) enq_vcycle<DIM, T>(S, H, l - 1, c == 0);
  v_prolong<DIM, T><<<slot_blocks(lc.sl), lc.sl.chunk, 0, s>>>(lv.g, lc.g, lc.sl, st, lc.X[lc.cur], lv.X[lv.cur]);
  enq_smooth<DIM, T>(S, lv, false, dots);
}

// z = B r; H.z is where z lands (the same buffer at every application).
// Returns true when z.z and z.r were reduced (and Fin(dots) run) by the last
// smoothing step, false when the caller still has to reduce them.
template <int DIM, typename T>
static bool enq_pc(fishgpu_solver *S, Hier<T> &H, const T *r, int dots, const RUpd<T> *ru = nullptr) {
  const fishgpu_opts &o = S->o;
  if (o.pc_type == FISHGPU_PC_NONE) {
    v_scale<T><<<slot_blocks(S->sf), S->sf.chunk, 0, S->stream>>>(S->fine, S->sf, S->st, r, T(1), H.zbuf);
    H.z = H.zbuf;
    return false;
  }
  if (o.pc_type == FISHGPU_PC_JACOBI) {  // z = D^{-1} r
    v_scale<T><<<slot_blocks(S->sf), S->sf.chunk, 0, S->stream>>>(S->fine, S->sf, S->st, r, (T)(1.0 / S->fine.scdiag), H.zbuf);
    H.z = H.zbuf;
    return false;
  }
  for (int l = 0; l < H.nlev; l++) H.lev[l].cur = 0;
  Level<T> &top = H.lev[H.nlev - 1];
  top.b = const_cast<T *>(r);
  const bool fused = H.nlev > 1;  // a single level ends with the coarse solve, no smoother
  enq_vcycle<DIM, T>(S, H, H.nlev - 1, true, fused ? dots : -1, ru);
  H.z = top.X[top.cur];
  return fused;
}

template <typename T>
struct KspVecs {
  T *r, *p[2], *w, *y;  // p: two buffers, the direction update reads one and writes the other
  double *y64 = nullptr;  // FP32 solves with FP64 accumulation: the outer solution the updates go to
  T *r2 = nullptr;        // a second residual buffer: the residual update goes into the V-cycle's first
                          // pass (RUpd), which reads r and writes r_new; iteration i reads r from
                          // {r, r2}[i & 1] and writes the other
};

// Whether CG iterations carry their residual update into the V-cycle's first
// smoothing pass (v_cheb2_zero's RUPD form): the mixed form's FP32 inner
// solves of a single grid, MG with two Chebyshev/Jacobi steps from zero on
// the finest level.  Not the FP64 form: forming r - alpha w at every stencil
// point adds FP64 FMAs to an FP64-bound pass (513^3: 231 -> 241 ms; the mixed
// form 46.9 -> 46.3 ms).
static bool fuse_cgr_ok(const fishgpu_opts &o, int batch, int nlev) {
  return o.fuse_cgr && o.precision == FISHGPU_MIXED && !batch && o.pc_type == FISHGPU_PC_MG && nlev > 1 &&
         o.smooth_type == FISHGPU_SMOOTH_CHEBYSHEV && o.smooth_its == 2;
}

// src64 (FP32 solves of the mixed form, unpreconditioned norm): the FP64
// residual the right-hand side is demoted from, its r.r in dval[0]
template <int DIM, typename T>
static void enq_cg_init(fishgpu_solver *S, Hier<T> &H, KspVecs<T> v, const double *src64 = nullptr) {
  cudaStream_t s = S->stream;
  if constexpr (sizeof(T) == 4) {
    if (src64) {
      k_inv_norm<<<1, 1, 0, s>>>(S->dval, S->dval + 6);
      v_demote_init<<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, S->st, src64, S->dval + 6, v.r, S->red,
                                                               0);
      if (!enq_pc<DIM, T>(S, H, v.r, FIN_INIT_ZZZR))
        v_dots<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, S->st, H.z, v.r, S->red, 0, FIN_INIT_ZZZR,
                                                             nullptr);
      return;
    }
  }
  if (S->ksp_norm == FISHGPU_NORM_UNPRECONDITIONED)
    v_dots<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, S->st, v.r, v.r, S->red, 0, FIN_INIT_RR, nullptr);
  if (!enq_pc<DIM, T>(S, H, v.r, FIN_INIT_ZZZR))
    v_dots<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, S->st, H.z, v.r, S->red, 0, FIN_INIT_ZZZR, nullptr);
}

// One CG iteration; `par` selects which p buffer holds the previous direction.
template <int DIM, typename T>
static void enq_cg_iter(fishgpu_solver *S, Hier<T> &H, KspVecs<T> v, int par) {
  cudaStream_t s = S->stream;
  KspState *st = S->st;
  T *pold = v.p[par], *pnew = v.p[1 - par];
  // p = z + beta/betaold p (z of the previous application), w = A p, p.w
  bool planes = false;
  if constexpr (DIM == 2) {
    if (S->batch) {
      if constexpr (sizeof(T) == 4) {
        if (v.y64)
          v_cgp_apply<DIM, T, true, true><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(
              S->fine, S->sfst, st, H.z, pold, pnew, v.w, v.y64, S->red, 0);
        else
          v_cgp_apply<DIM, T, true><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(S->fine, S->sfst, st, H.z, pold, pnew,
                                                                           v.w, v.y, S->red, 0);
      } else {
        v_cgp_apply<DIM, T, true><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(S->fine, S->sfst, st, H.z, pold, pnew, v.w,
                                                                         v.y, S->red, 0);
      }
      planes = true;
    }
  }
  if constexpr (sizeof(T) == 4) {
    if (!planes && v.y64) {  // accurate inner form: difference-form apply, FP64 accumulation
      if (!(DIM == 3 && S->o.tma_apply && launch_cgp_tma(S, S->fine, st, H.z, pold, pnew, v.w, v.y64, 0))) {
        if (S->o.pair_y) {  // y64 updated in pairs (a captured iteration's parity is its own)
          if (par == 0)
            v_cgp_apply<DIM, T, false, true, 1><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(
                S->fine, S->sfst, st, H.z, pold, pnew, v.w, v.y64, S->red, 0);
          else
            v_cgp_apply<DIM, T, false, true, 2><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(
                S->fine, S->sfst, st, H.z, pold, pnew, v.w, v.y64, S->red, 0);
        } else {
          v_cgp_apply<DIM, T, false, true><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(
              S->fine, S->sfst, st, H.z, pold, pnew, v.w, v.y64, S->red, 0);
        }
      }
      planes = true;
    }
  }
  if (!planes)
    v_cgp_apply<DIM, T, false><<<slot_blocks(S->sfst), S->sfst.chunk, 0, s>>>(S->fine, S->sfst, st, H.z, pold, pnew, v.w,
                                                                      v.y, S->red, 0);
  const bool unprec = S->ksp_norm == FISHGPU_NORM_UNPRECONDITIONED;
  if (v.r2 && fuse_cgr_ok(S->o, S->batch, H.nlev)) {  // r -= alpha w inside the V-cycle's first pass
    T *rcur = par ? v.r2 : v.r, *rnext = par ? v.r : v.r2;
    const RUpd<T> ru{rcur, v.w, unprec};
    if (!enq_pc<DIM, T>(S, H, rnext, FIN_ZZZR, &ru))
      v_dots<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, st, H.z, rnext, S->red, 0, FIN_ZZZR,
                                                           nullptr);
    return;
  }
  if (unprec)
    v_cg_r<T, true><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, st, v.w, v.r, S->red, 0);
  else
    v_cg_r<T, false><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, st, v.w, v.r, S->red, 0);
  if (!enq_pc<DIM, T>(S, H, v.r, FIN_ZZZR))
    v_dots<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, st, H.z, v.r, S->red, 0, FIN_ZZZR, nullptr);
}

static long long kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  long long k = 0;
  for (size_t q = 0; q < n; q++) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[q], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

// Capture what `enq` enqueues on the solver's stream into an executable graph.
template <typename F>
static int capture(fishgpu_solver *S, F enq, cudaGraphExec_t *exec, long long *nkern) {
  cudaGraph_t graph;
  FG_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
  enq();
  cudaError_t e = cudaStreamEndCapture(S->stream, &graph);
  if (e != cudaSuccess) return FISHGPU_ERR_CUDA;
  *nkern = kernel_nodes(graph);
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    *exec = nullptr;
    return FISHGPU_ERR_CUDA;
  }
  return FISHGPU_OK;
}

static void reset_state(fishgpu_solver *S, double rtol, double atol, double dtol, int max_it, int norm,
                        double yscale = 0.0, bool yfresh = false) {
  KspState *h = S->st_h;
  memset(h, 0, sizeof(*h));
  h->rtol = rtol;
  h->atol = atol;
  h->dtol = dtol;
  h->max_it = max_it;
  h->norm_type = norm;
  h->betaold = 1.0;
  h->yscale = yscale;
  h->yfresh = yfresh ? 1 : 0;
}

// CG solve of J y = r from y = 0 (r is overwritten), on the solver's stream.
// from64 >= 0 (FP32 solves of the mixed form): r is set up from the FP64
// residual in b64 (0) or r64 (1), scaled by 1/||.|| from dval[0], and the
// last deferred y += alpha p is left to the caller (v_pend_promote).
// yscale, yfresh: the FP64 accumulation of the accurate inner form (v.y64).
// The caller reads S->st_h for its, reason and the history.
// run_ksp as one cooperative launch of k_ksp_persist (build_persist chose it)
template <int DIM, typename T>
static int run_ksp_persist(fishgpu_solver *S, Hier<T> &H, KspVecs<T> v, double rtol, int max_it, int from64,
                           double yscale, bool yfresh, bool read_back = true) {
  cudaStream_t s = S->stream;
  reset_state(S, rtol, S->o.atol, S->o.dtol, max_it, S->ksp_norm, yscale, yfresh);
  FG_CUDA(cudaMemcpyAsync(S->st, S->st_h, sizeof(KspState), cudaMemcpyHostToDevice, s));
  FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
  PersistArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.lv = H.plev;
  a.top = H.nlev - 1;
  a.btop = H.pbtop;
  a.r = v.r;
  a.p[0] = v.p[0];
  a.p[1] = v.p[1];
  a.w = v.w;
  a.y = v.y;
  a.y64 = v.y64;
  a.src64 = from64 < 0 ? nullptr : from64 ? S->r64 : S->b64;
  a.rr64 = S->dval;
  a.unprec = S->ksp_norm == FISHGPU_NORM_UNPRECONDITIONED;
  a.do_pend = from64 < 0;
  // the device loop's cap: loop_cap bodies of giters iterations
  a.max_iters = S->o.loop_cap > 0 ? S->o.loop_cap * S->giters : max_it + 8;
  a.st = S->st;
  a.part = S->ppart;
  a.bar = S->pbar;
  a.fault = S->fault;
  const Level<T> &c = H.lev[0];
  a.S0 = c.S[0];
  a.S1 = c.S[1];
  a.S2 = c.S[2];
  a.ilam = c.ilam;
  a.work = c.work;
  a.n0 = c.n[0];
  a.n1 = c.n[1];
  a.n2 = c.n[2];
  a.smem = H.pcoarse ? 1 : 0;
  a.dinv = (T)(1.0 / c.g.scdiag);
  a.copy_off = H.pcopy;
  void *args[] = {&a};
  const void *fn;
  if constexpr (sizeof(T) == 4) {
    fn = v.y64 ? (const void *)k_ksp_persist<DIM, T, true> : (const void *)k_ksp_persist<DIM, T, false>;
  } else {
    fn = (const void *)k_ksp_persist<DIM, T, false>;
  }
  FG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(S->pblocks), dim3(512), args, H.psmem, s));
  S->launches += 1;
  if (!read_back) return FISHGPU_OK;  // the caller reads the state and the fault word
  FG_CUDA(cudaMemcpyAsync(S->st_h, S->st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(S->hval + 7, S->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  int fault = 0;
  memcpy(&fault, S->hval + 7, sizeof(int));
  if (fault || !S->st_h->done) {  // a barrier gave up, or the iteration cap ran out
    if (fault) {  // the next solve starts clean
      FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
      FG_CUDA(cudaStreamSynchronize(s));
    }
    return FISHGPU_ERR_TIMEOUT;
  }
  return FISHGPU_OK;
}

template <int DIM, typename T>
static int run_ksp(fishgpu_solver *S, Hier<T> &H, KspVecs<T> v, double rtol, int max_it, int from64 = -1,
                   double yscale = 0.0, bool yfresh = false) {
  if constexpr (DIM >= 2) {
    if (H.plev) return run_ksp_persist<DIM, T>(S, H, v, rtol, max_it, from64, yscale, yfresh);
  }
  cudaStream_t s = S->stream;
  const int norm = S->ksp_norm;  // the captured graphs compute this norm
  int rc;
  cudaGraphExec_t *gi = from64 < 0 ? &S->gexec_init : &S->gexec_init64[from64 & 1];
  const double *src64 = from64 < 0 ? nullptr : from64 ? S->r64 : S->b64;
  if (!*gi && (rc = capture(S, [&] { enq_cg_init<DIM, T>(S, H, v, src64); }, gi, &S->n_init))) return rc;
  const long long guard = S->o.loop_cap > 0 ? (long long)S->o.loop_cap - 1 : (long long)max_it / S->giters + 4;
  // The loop on the device: one launch runs bodies of giters iterations until
  // the state says stop (or guard bodies ran).  A driver that refuses the
  // conditional node gets the host loop: a graph of giters iterations per
  // launch and a read of the stop flag after each.
  if (!S->gloop && !S->loop_refused && S->o.device_loop)
    S->loop_refused = !build_loop_graph(
        s, [&] { for (int g = 0; g < S->giters; g++) enq_cg_iter<DIM, T>(S, H, v, g & 1); }, &S->st->done, nullptr,
        0u, &S->st->loops, (unsigned int)(guard + 1), &S->gloop, &S->n_loop);
  if (!S->gloop && !S->gexec &&
      (rc = capture(S, [&] { for (int g = 0; g < S->giters; g++) enq_cg_iter<DIM, T>(S, H, v, g & 1); },
                    &S->gexec, &S->n_iter)))
    return rc;
  reset_state(S, rtol, S->o.atol, S->o.dtol, max_it, norm, yscale, yfresh);
  FG_CUDA(cudaMemcpyAsync(S->st, S->st_h, sizeof(KspState), cudaMemcpyHostToDevice, s));
  FG_CUDA(cudaGraphLaunch(*gi, s));
  S->launches += S->n_init;
  if (S->gloop) {
    FG_CUDA(cudaGraphLaunch(S->gloop, s));
  } else {
    for (long long launch = 0;; launch++) {
      FG_CUDA(cudaMemcpyAsync(&S->st_h->done, &S->st->done, sizeof(int), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaStreamSynchronize(s));
      if (S->st_h->done) break;
      if (launch > guard) return FISHGPU_ERR_TIMEOUT;
      FG_CUDA(cudaGraphLaunch(S->gexec, s));
      S->launches += S->n_iter;
    }
  }
  if (from64 < 0) {  // the last iteration's deferred y += alpha p
    v_cg_pend<T><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(S->fine, S->sf, S->st, v.p[0], v.p[1], v.y);
    S->launches += 1;
  }
  FG_CUDA(cudaMemcpyAsync(S->st_h, S->st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  if (S->gloop) {
    S->launches += (long long)S->st_h->loops * S->n_loop;
    if (!S->st_h->done) return FISHGPU_ERR_TIMEOUT;
  }
  return FISHGPU_OK;
}

// ------------------------------------------------------------------ FP64 helpers
// F(u) = A u - beff with A the Jacobian (boundary rows scdiag, boundary
// columns eliminated): beff = scdiag*g on boundary rows; on interior rows
// vol*f plus sc_d*g at each neighbour on the boundary -- the reference's
// residual (poissonfunctions.c:10-19, :43-59, :86-106) rearranged.
// USERP: FISHGPU_USER data, read directly (the problem-generic accessors would
// carry the built-in problems' FP64 transcendentals into the loop)
template <int DIM, bool USERP>
__global__ void __launch_bounds__(256) k_beff64(Geom g, Tiles tm, Prob pb, double *__restrict__ be) {
  const Range R = full_range(g);
  auto fa = [&](int i, int j, int k) -> double {
    if constexpr (USERP) return pb.f[uidx(pb, i, j, k)];
    else return f_at(pb, g, i, j, k);
  };
  auto ga = [&](int i, int j, int k) -> double {
    if constexpr (USERP) return pb.g[uidx(pb, i, j, k)];
    else return g_at(pb, g, i, j, k);
  };
  FG_POINT_LOOP_BEGIN(R)
  if (on_bdry<DIM>(g, i, j, k)) {
    be[n] = g.scdiag * ga(i, j, k);
  } else {
    double v = g.vol * fa(i, j, k);
    if (i - 1 == 0) v = fma(g.sc[0], ga(i - 1, j, k), v);
    if (i + 1 == g.mx - 1) v = fma(g.sc[0], ga(i + 1, j, k), v);
    if (DIM >= 2) {
      if (j - 1 == 0) v = fma(g.sc[1], ga(i, j - 1, k), v);
      if (j + 1 == g.my - 1) v = fma(g.sc[1], ga(i, j + 1, k), v);
    }
    if (DIM >= 3) {
      if (k - 1 == 0) v = fma(g.sc[2], ga(i, j, k - 1), v);
      if (k + 1 == g.mz - 1) v = fma(g.sc[2], ga(i, j, k + 1), v);
    }
    be[n] = v;
  }
  FG_POINT_LOOP_END
}

// u0 into the padded u (InitialState, poissonfunctions.c:260-346); GIVEN packs
// the caller's dense array
template <int DIM>
__global__ void __launch_bounds__(256) k_initial64(Geom g, Geom gd, Tiles tm, Prob pb, int type, int gbdry,
                                                   unsigned long long seed, const double *__restrict__ given,
                                                   double *__restrict__ u) {
  const Range R = full_range(g);
  FG_POINT_LOOP_BEGIN(R)
  double v;
  if (type == FISHGPU_INITIAL_GIVEN) {
    v = given[gidx(gd, i, j, k)];
  } else if (type == FISHGPU_INITIAL_RANDOM) {
    unsigned long long x = (seed ^ (((unsigned long long)k * g.my + j) * g.mx + i)) + 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x ^= x >> 31;
    v = (double)(x >> 11) * 0x1.0p-53;
  } else {
    v = 0.0;
  }
  if (gbdry && on_bdry<DIM>(g, i, j, k)) v = g_at(pb, g, i, j, k);
  u[n] = v;
  FG_POINT_LOOP_END
}

// u = u0 + y into the caller's dense u (y NULL: y = +0, an update never made);
// keep: u0 is overwritten with u as well
template <int DIM>
__global__ void __launch_bounds__(256) k_unpack_add64(Geom g, Geom gd, Tiles tm, double *__restrict__ up,
                                                      const double *__restrict__ y, double *__restrict__ ud,
                                                      bool keep) {
  const Range R = full_range(g);
  FG_POINT_LOOP_BEGIN(R)
  const double v = up[n] + (y ? y[n] : 0.0);
  ud[gidx(gd, i, j, k)] = v;
  if (keep) up[n] = v;
  FG_POINT_LOOP_END
}

// The start of a mixed solve of user data (FISHGPU_USER f, g) from the zero
// initial state, in one vectorised pass: u0 (g on the boundary when asked,
// 0 elsewhere), the KSP right-hand side b = -F(u0) = beff - J u0 and its
// b.b.  The same values as k_initial64, k_beff64 and v_resid_zero0 in turn
// (every point the same expressions in the same order, the norm reduced as
// v_resid_zero0 reduces it), without the beff array.
template <int DIM>
__global__ void __launch_bounds__(256) v_user_start(Geom g, Slots s, Prob pb, int gbdry, double *__restrict__ u0,
                                                    double *__restrict__ b, Reducer red, int slot, double *out) {
  const double sd = g.scdiag;
  // the user arrays read directly: the problem-generic accessors would carry
  // the built-in problems' FP64 transcendentals into the loop
  const double *__restrict__ fu = pb.f, *__restrict__ gu = pb.g;
  auto uf = [&](int i, int j, int k) { return fu[uidx(pb, i, j, k)]; };
  auto ug = [&](int i, int j, int k) { return gu[uidx(pb, i, j, k)]; };
  double rr = 0.0;
  FG_PW_BEGIN
  V4<double> uo, bo;
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int i = p.i4 + e, j = p.j;
    double uv = 0.0, bv = 0.0;
    if (i < g.mx) {
      if (on_bdry<DIM>(g, i, j, k)) {
        const double gv = ug(i, j, k);
        uv = gbdry ? gv : 0.0;
        bv = fma(-sd, uv, g.scdiag * gv);
      } else {
        double v = g.vol * uf(i, j, k);
        if (i - 1 == 0) v = fma(g.sc[0], ug(i - 1, j, k), v);
        if (i + 1 == g.mx - 1) v = fma(g.sc[0], ug(i + 1, j, k), v);
        if (DIM >= 2) {
          if (j - 1 == 0) v = fma(g.sc[1], ug(i, j - 1, k), v);
          if (j + 1 == g.my - 1) v = fma(g.sc[1], ug(i, j + 1, k), v);
        }
        if (DIM >= 3) {
          if (k - 1 == 0) v = fma(g.sc[2], ug(i, j, k - 1), v);
          if (k + 1 == g.mz - 1) v = fma(g.sc[2], ug(i, j, k + 1), v);
        }
        bv = v + 0.0;
      }
    }
    set_el(uo, e, uv);
    set_el(bo, e, bv);
  }
  st4(u0 + n, uo);
  st4(b + n, bo);
  rr = fma(bo.x, bo.x, fma(bo.y, bo.y, fma(bo.z, bo.z, fma(bo.w, bo.w, rr))));
  FG_PW_END
  double v1[1] = {rr};
  reduce_slots<1>(v1, red, slot, nullptr, FIN_STORE, out, s);
}

static int read_vals(fishgpu_solver *S, int n) {
  FG_CUDA(cudaMemcpyAsync(S->hval, S->dval, sizeof(double) * n, cudaMemcpyDeviceToHost, S->stream));
  FG_CUDA(cudaStreamSynchronize(S->stream));
  return FISHGPU_OK;
}

static void fill_from_state(const KspState *h, fishgpu_report *rep) {
  rep->its = h->its;
  rep->reason = h->reason;
  rep->nhist = h->nhist;
  const int n = h->nhist < FISHGPU_MAX_HIST ? h->nhist : FISHGPU_MAX_HIST;
  for (int q = 0; q < n; q++) rep->hist[q] = h->hist[q];
}

// The mixed form's refinement loop as one launch (k_mixed_persist): the
// right-hand side b64 and its b.b (dval[0]) are on the device already; the
// report comes back in one read at the end.
// The FP64 form's solve as one persistent launch followed by the unpacking
// and F(u), with ONE read of the results at the end (the initial norm, the
// KSP state, F(u)'s norm and the fault word), instead of a host round trip
// before and after the KSP.
template <int DIM>
static int solve_fp64_persist(fishgpu_solver *S, double *u, fishgpu_report *rep) {
  const fishgpu_opts &o = S->o;
  cudaStream_t s = S->stream;
  const Geom &g = S->fine;
  const Launch &L = S->Lf;
  KspVecs<double> v{S->r64, {S->p64, S->q64}, S->w64, S->y64};
  int rc = run_ksp_persist<DIM, double>(S, S->h64, v, o.rtol, o.max_it, -1, 0.0, false, false);
  if (rc) return rc;
  k_unpack_add64<DIM><<<L.grid, L.block, 0, s>>>(g, S->dense, L.tm, S->u64, S->y64, u, true);
  // F(u) for the final SNES norm (r64 is free now)
  v_resid<DIM, double, true><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, nullptr, S->beff, S->u64, S->r64,
                                                                       S->red, 1, S->dval + 1);
  S->launches += 2;
  FG_CUDA(cudaEventRecord(S->ev1, s));
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaMemcpyAsync(S->st_h, S->st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(S->hval, S->dval, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(S->hval + 7, S->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  int fault = 0;
  memcpy(&fault, S->hval + 7, sizeof(int));
  if (fault || !S->st_h->done) {  // a barrier gave up, or the iteration cap ran out
    if (fault) {
      FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
      FG_CUDA(cudaStreamSynchronize(s));
    }
    return FISHGPU_ERR_TIMEOUT;
  }
  const double bn = sqrt(S->hval[0]);
  rep->fnorm0 = bn;
  fill_from_state(S->st_h, rep);
  rep->outer_its = 0;
  rep->fnorm1 = sqrt(S->hval[1]);
  rep->true_rel_resid = bn > 0.0 ? rep->fnorm1 / bn : 0.0;
  float ms = 0.f;
  FG_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
  rep->solve_ms = ms;
  return FISHGPU_OK;
}

template <int DIM>
static int solve_mixed_persist(fishgpu_solver *S, double *u, fishgpu_report *rep) {
  const fishgpu_opts &o = S->o;
  cudaStream_t s = S->stream;
  const Geom &g = S->fine;
  const Launch &L = S->Lf;
  Hier<float> &H = S->h32;
  double lmin, lmax;
  spectrum(g, &lmin, &lmax);
  const double kappa = lmax / fmax(lmin, 1e-300);
  const bool accurate = inner_accurate_for(o.inner_accurate, o.rtol, o.inner_rtol, kappa);
  int mmax = g.mx;
  if (g.dim >= 2) mmax = std::max(mmax, g.my);
  if (g.dim >= 3) mmax = std::max(mmax, g.mz);
  // the first step's floor, as in solve_dim
  const double first_floor = accurate ? fmin(0.5, o.first_floor_scale * kappa * (M_PI / (mmax - 1)) * 0x1.0p-24)
                                      : fmin(0.5, 0.3 * kappa * 0x1.0p-24);
  PersistArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.lv = H.plev;
  a.top = H.nlev - 1;
  a.btop = H.pbtop;
  a.r = S->r32;
  a.p[0] = S->p32;
  a.p[1] = S->q32;
  a.w = S->w32;
  a.y = S->y32;
  a.y64 = accurate ? S->y64 : nullptr;
  a.unprec = 1;
  a.do_pend = 0;
  a.max_iters = o.loop_cap > 0 ? o.loop_cap * S->giters : o.inner_max_it + 8;
  a.st = S->st;
  a.part = S->ppart;
  a.bar = S->pbar;
  a.fault = S->fault;
  const Level<float> &c = H.lev[0];
  a.S0 = c.S[0];
  a.S1 = c.S[1];
  a.S2 = c.S[2];
  a.ilam = c.ilam;
  a.work = c.work;
  a.n0 = c.n[0];
  a.n1 = c.n[1];
  a.n2 = c.n[2];
  a.smem = H.pcoarse ? 1 : 0;
  a.dinv = (float)(1.0 / c.g.scdiag);
  a.copy_off = H.pcopy;
  MixedArgs m;
  m.b64 = S->b64;
  m.y64 = S->y64;
  m.r64 = S->r64;
  m.y32 = S->y32;
  m.bb = S->dval;
  m.rtol = o.rtol;
  m.atol = o.atol;
  m.inner_rtol = o.inner_rtol;
  m.first_floor = first_floor;
  m.outer_max_it = o.outer_max_it;
  m.max_it = o.max_it;
  m.inner_max_it = o.inner_max_it;
  m.dtol = o.dtol;
  m.out = S->mout;
  FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
  void *args[] = {&a, &m};
  const void *fn = accurate ? (const void *)k_mixed_persist<DIM, true> : (const void *)k_mixed_persist<DIM, false>;
  FG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(S->pblocks), dim3(512), args, H.psmem, s));
  // u = u0 + y (the kernel leaves y64 = 0 when no refinement step ran)
  k_unpack_add64<DIM><<<L.grid, L.block, 0, s>>>(g, S->dense, L.tm, S->u64, S->y64, u, false);
  S->launches += 2;
  FG_CUDA(cudaEventRecord(S->ev1, s));
  FG_CUDA(cudaMemcpyAsync(S->mout_h, S->mout, sizeof(MixedOut), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(S->hval + 7, S->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  int fault = 0;
  memcpy(&fault, S->hval + 7, sizeof(int));
  const MixedOut &mo = *S->mout_h;
  if (fault || mo.status) {
    if (fault) {
      FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
      FG_CUDA(cudaStreamSynchronize(s));
    }
    return FISHGPU_ERR_TIMEOUT;
  }
  rep->fnorm0 = mo.bn;
  rep->its = mo.its;
  rep->reason = mo.reason;
  rep->outer_its = mo.outer;
  rep->nhist = mo.nhist;
  for (int q = 0; q < std::min(mo.nhist, FISHGPU_MAX_HIST); q++) rep->hist[q] = mo.hist[q];
  for (int q = 0; q < std::min(mo.outer, FISHGPU_MAX_OUTER); q++) rep->inner_its[q] = mo.inner_its[q];
  rep->fnorm1 = mo.nhist > 0 ? mo.hist[std::min(mo.nhist, FISHGPU_MAX_HIST) - 1] : mo.bn;
  rep->true_rel_resid = mo.bn > 0.0 ? rep->fnorm1 / mo.bn : 0.0;
  float ms = 0.f;
  FG_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
  rep->solve_ms = ms;
  return FISHGPU_OK;
}

template <int DIM>
static int solve_dim(fishgpu_solver *S, double *u, fishgpu_report *rep) {
  const fishgpu_opts &o = S->o;
  cudaStream_t s = S->stream;
  const Launch &L = S->Lf;
  const Geom &g = S->fine;
  FG_CUDA(cudaEventRecord(S->ev0, s));
  // a solve that ended early on an error may have left the fault word set
  if (S->fault) FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
  // the KSP right-hand side is -F(u0) = beff - A u0 and its norm; it solves
  // for -y and u = u0 + (-y)
  double *F = o.precision == FISHGPU_MIXED ? S->b64 : S->r64;
  if (o.precision == FISHGPU_MIXED && o.ctx.problem == FISHGPU_USER && o.initial_type == FISHGPU_INITIAL_ZEROS) {
    // user data change between solves: u0, b and ||b|| in one pass (beff is
    // not needed by the mixed form)
    v_user_start<DIM><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, S->prob, o.initial_gonboundary, S->u64,
                                                                  F, S->red, 1, S->dval);
    S->launches = 1;
  } else {
    S->launches = 2;  // initial state, -F(u0) with its norm
    k_initial64<DIM><<<L.grid, L.block, 0, s>>>(g, S->dense, L.tm, S->prob, o.initial_type, o.initial_gonboundary,
                                                 o.seed, u, S->u64);
    if (!S->beff_ready) {
      if (S->prob.problem == FISHGPU_USER)
        k_beff64<DIM, true><<<L.grid, L.block, 0, s>>>(g, L.tm, S->prob, S->beff);
      else
        k_beff64<DIM, false><<<L.grid, L.block, 0, s>>>(g, L.tm, S->prob, S->beff);
      S->launches += 1;
      S->beff_ready = S->o.ctx.problem != FISHGPU_USER;  // user data may change between solves
    }
    if (o.initial_type == FISHGPU_INITIAL_ZEROS)
      v_resid_zero0<DIM><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, S->beff, S->u64, F, S->red, 1,
                                                                     S->dval);
    else
      v_resid<DIM, double, true><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, nullptr, S->beff, S->u64, F,
                                                                           S->red, 1, S->dval);
  }
  FG_CUDA(cudaGetLastError());
  if constexpr (DIM >= 2) {
    if (o.precision == FISHGPU_MIXED && S->h32.plev && S->mout) return solve_mixed_persist<DIM>(S, u, rep);
    if (o.precision == FISHGPU_FP64 && S->h64.plev) return solve_fp64_persist<DIM>(S, u, rep);
  }
  int rc = read_vals(S, 1);
  if (rc) return rc;
  const double bn = sqrt(S->hval[0]);
  rep->fnorm0 = bn;
  if (o.precision == FISHGPU_FP64) {
    KspVecs<double> v{S->r64, {S->p64, S->q64}, S->w64, S->y64};
    if ((rc = run_ksp<DIM, double>(S, S->h64, v, o.rtol, o.max_it))) return rc;
    fill_from_state(S->st_h, rep);
    rep->outer_its = 0;
  } else {
    // FP64 iterative refinement around an FP32 CG + FP32 V-cycle
    const double ttol = fmax(o.rtol * bn, o.atol);
    double rn = bn;
    int reason = 0, its = 0, outer = 0, nh = 0;
    rep->hist[nh++] = rn;
    double lmin, lmax;
    spectrum(g, &lmin, &lmax);
    const double kappa = lmax / fmax(lmin, 1e-300);
    const bool accurate = inner_accurate_for(o.inner_accurate, o.rtol, o.inner_rtol, kappa);
    KspVecs<float> v{S->r32, {S->p32, S->q32}, S->w32, S->y32, accurate ? S->y64 : nullptr, S->r32b};
    // The first correction is smooth and carries the FP32 rounding of its
    // storage and of the FP32 apply's diagonal term, which J amplifies by up
    // to its condition number: the true residual cannot drop below ~kappa *
    // 2^-24 of ||b|| in that step, so the first inner solve stops there.  The
    // accurate form (difference-form apply, FP64 accumulation) leaves the
    // rounding of the differences, ~kappa * pi h * 2^-24 (h: the finest grid
    // spacing in units of the longest side).  kappa is the exact ratio of the
    // extreme eigenvalues of D^{-1}J on the fine grid.
    int mmax = g.mx;
    if (g.dim >= 2) mmax = std::max(mmax, g.my);
    if (g.dim >= 3) mmax = std::max(mmax, g.mz);
    const double first_floor = accurate ? fmin(0.5, o.first_floor_scale * kappa * (M_PI / (mmax - 1)) * 0x1.0p-24)
                                        : fmin(0.5, 0.3 * kappa * 0x1.0p-24);
    while (true) {
      if (isnan(rn) || isinf(rn)) { reason = R_DIVERGED_NANORINF; break; }
      if (rn <= ttol) { reason = rn < o.atol ? R_CONVERGED_ATOL : R_CONVERGED_RTOL; break; }
      if (outer >= o.outer_max_it || its >= o.max_it) { reason = R_DIVERGED_ITS; break; }
      S->launches += 2;  // promote-add, FP64 residual with its norm
      // inner tolerance: what is still needed, never below the FP32 floor
      double irtol = fmax(o.inner_rtol, 0.5 * ttol / rn);
      if (outer == 0) irtol = fmax(irtol, first_floor);
      if (irtol > 0.5) irtol = 0.5;
      // r32 = r / ||r|| (r: b64 in the first step, r64 after) inside the KSP set-up
      if ((rc = run_ksp<DIM, float>(S, S->h32, v, irtol, o.inner_max_it, outer == 0 ? 0 : 1, rn, outer == 0)))
        return rc;
      const KspState *h = S->st_h;
      its += h->its;
      if (outer < FISHGPU_MAX_OUTER) rep->inner_its[outer] = h->its;
      if (h->reason == R_DIVERGED_NANORINF || h->reason == R_DIVERGED_INDEFINITE_MAT ||
          h->reason == R_DIVERGED_INDEFINITE_PC) {
        reason = h->reason;
        break;
      }
      if (accurate) {  // the last deferred y64 += rn alpha p (the others went to y64 in the loop)
        v_pend_acc<<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, S->st, S->p32, S->q32, S->y64);
      } else {
        // y32 += alpha p (deferred), y64 += rn y32; y64 = 0 before the first
        // step: that step writes it without reading
        v_pend_promote<<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, S->st, S->p32, S->q32, S->y32, rn, S->y64,
                                                                  outer == 0);
      }
      // FP64 true residual r = b - J y and its norm
      v_resid<DIM, double, true><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, nullptr, S->b64, S->y64,
                                                                           S->r64, S->red, 1, S->dval);
      FG_CUDA(cudaGetLastError());
      if ((rc = read_vals(S, 1))) return rc;
      rn = sqrt(S->hval[0]);
      outer++;
      if (nh < FISHGPU_MAX_HIST) rep->hist[nh] = rn;
      nh++;
    }
    rep->its = its;
    rep->reason = reason;
    rep->outer_its = outer;
    rep->nhist = nh;
  }
  // u = u0 + (-y) into the caller's dense u (the FP64 form keeps it for F(u);
  // a mixed solve that stopped before its first step has y = 0)
  const bool fp64 = o.precision != FISHGPU_MIXED;
  const double *yv = fp64 || rep->outer_its > 0 ? S->y64 : nullptr;
  k_unpack_add64<DIM><<<L.grid, L.block, 0, s>>>(g, S->dense, L.tm, S->u64, yv, u, fp64);
  S->launches += 1;
  if (o.precision == FISHGPU_MIXED) {
    // the last refinement step computed the FP64 residual beff - A(u0 + y) = -F(u)
    FG_CUDA(cudaEventRecord(S->ev1, s));
    rep->fnorm1 = rep->nhist > 0 ? rep->hist[(rep->nhist < FISHGPU_MAX_HIST ? rep->nhist : FISHGPU_MAX_HIST) - 1] : bn;
  } else {
    // F(u) for the final SNES norm (r64 is free now)
    v_resid<DIM, double, true><<<slot_blocks(S->sf), S->sf.chunk, 0, s>>>(g, S->sf, nullptr, S->beff, S->u64,
                                                                         S->r64, S->red, 1, S->dval + 1);
    S->launches += 1;
    FG_CUDA(cudaEventRecord(S->ev1, s));
    FG_CUDA(cudaGetLastError());
    if ((rc = read_vals(S, 2))) return rc;
    rep->fnorm1 = sqrt(S->hval[1]);
  }
  rep->true_rel_resid = bn > 0.0 ? rep->fnorm1 / bn : 0.0;
  float ms = 0.f;
  FG_CUDA(cudaEventSynchronize(S->ev1));
  FG_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
  rep->solve_ms = ms;
  if (S->fault) {  // a kernel's bounded wait on a copy gave up: its results are not to be trusted
    FG_CUDA(cudaMemcpyAsync(S->hval + 7, S->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    int f = 0;
    memcpy(&f, S->hval + 7, sizeof(int));
    if (f) {
      FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
      return FISHGPU_ERR_TIMEOUT;
    }
  }
  return FISHGPU_OK;
}

// Largest grid of a reduction kernel on the fine level.
static int reduction_blocks(const fishgpu_solver *S) { return (int)slot_blocks(S->sf); }

template <int DIM>
static int time_kernel_dim(fishgpu_solver *S, const char *name, int reps, double *ms, double *bytes) {
  const bool mixed = S->o.precision == FISHGPU_MIXED;
  const double N = (double)S->fine.mx * S->fine.my * S->fine.mz;
  cudaStream_t s = S->stream;
  const Geom &g = S->fine;
  const Slots &sl = S->sf;
  const unsigned gb = slot_blocks(sl);
  if (S->o.pc_type != FISHGPU_PC_MG) return FISHGPU_ERR_UNSUPPORTED;
  Level<float> &lf = S->h32.lev[S->h32.nlev > 0 ? S->h32.nlev - 1 : 0];
  Level<double> &ld = S->h64.lev[S->h64.nlev > 0 ? S->h64.nlev - 1 : 0];
  Level<float> &cf = S->h32.lev[S->h32.nlev > 1 ? S->h32.nlev - 2 : 0];
  Level<double> &cd = S->h64.lev[S->h64.nlev > 1 ? S->h64.nlev - 2 : 0];
  const double sz = mixed ? 4.0 : 8.0;
  float t = 0.f;
  // cgp_apply and cg_update read a CG state: one past its first iteration
  // (beta/betaold = 1, a small alpha); p.w > 0 keeps it running, and a stop
  // (non-finite data) is reported
  KspState *tst = nullptr;
  if (!strncmp(name, "cgp_apply", 9) || !strcmp(name, "cg_update") || !strcmp(name, "demote")) {
    KspState h;
    memset(&h, 0, sizeof(h));
    h.i = 2;  // a direction update that also reads y (the first one, i = 1, starts y from 0)
    h.beta = h.betaold = h.dpi = h.bratio = 1.0;
    h.alpha = 1e-3;
    h.pend = 1;  // cgp_apply also applies a deferred y update
    h.norm_type = FISHGPU_NORM_UNPRECONDITIONED;
    if (cudaMalloc((void **)&tst, sizeof(KspState)) != cudaSuccess) return FISHGPU_ERR_NOMEM;
    if (cudaMemcpyAsync(tst, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      cudaFree(tst);
      return FISHGPU_ERR_CUDA;
    }
  }
  struct Free {
    KspState *p;
    ~Free() { if (p) cudaFree(p); }
  } free_tst{tst};
  if (!strcmp(name, "grid_sync")) {  // one barrier of the persistent solve (launches of 100)
    if (!S->pbar || S->pblocks < 1) return FISHGPU_ERR_UNSUPPORTED;
    int nb = 100, absent = -1;
    void *args[] = {&S->pbar, &S->fault, &nb, &absent};
    FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
    FG_CUDA(cudaLaunchCooperativeKernel((const void *)k_grid_sync_probe, dim3(S->pblocks), dim3(512), args, 0, s));
    FG_CUDA(cudaEventRecord(S->ev0, s));
    for (int q = 0; q < reps; q++) {
      FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
      FG_CUDA(cudaLaunchCooperativeKernel((const void *)k_grid_sync_probe, dim3(S->pblocks), dim3(512), args, 0, s));
    }
    FG_CUDA(cudaEventRecord(S->ev1, s));
    FG_CUDA(cudaEventSynchronize(S->ev1));
    FG_CUDA(cudaEventElapsedTime(&t, S->ev0, S->ev1));
    *ms = (double)t / (reps * (double)nb);
    *bytes = 0.0;
    return FISHGPU_OK;
  }
  FG_CUDA(cudaEventRecord(S->ev0, s));
  for (int q = 0; q < reps; q++) {
    if (!strcmp(name, "smooth")) {  // one Chebyshev step with x_{k-1}: reads b, x_{k-1}, x_k, writes x_{k+1}
      if (mixed)
        v_cheb<DIM, float, true><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r32, lf.X[0], lf.X[1], lf.X[2], 0.5f, 0.5f, 0.1f);
      else
        v_cheb<DIM, double, true><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, ld.X[0], ld.X[1], ld.X[2], 0.5, 0.5, 0.1);
      *bytes = 4.0 * sz * N;
    } else if (!strcmp(name, "smooth_first")) {  // a Chebyshev step without x_{k-1}: reads b, x_k, writes x_{k+1}
      if (mixed)
        v_cheb<DIM, float, false><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r32, nullptr, lf.X[1], lf.X[2], 0.f, 0.5f, 0.1f);
      else
        v_cheb<DIM, double, false><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, nullptr, ld.X[1], ld.X[2], 0.0, 0.5, 0.1);
      *bytes = 3.0 * sz * N;
    } else if (!strcmp(name, "smooth_dots")) {  // the same step with z.z and z.b reduced (last post-smoothing step)
      if (mixed)
        v_cheb<DIM, float, true, true><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r32, lf.X[0], lf.X[1], lf.X[2], 0.5f,
                                                               0.5f, 0.1f, S->red, 1, FIN_STORE);
      else
        v_cheb<DIM, double, true, true><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, ld.X[0], ld.X[1], ld.X[2], 0.5,
                                                                0.5, 0.1, S->red, 1, FIN_STORE);
      *bytes = 4.0 * sz * N;
    } else if (!strcmp(name, "cgp_apply")) {  // p = z + beta p_old, w = A p, p.w, y += alpha p_old: reads z, p_old, y, writes p, w, y
      if (mixed)
        v_cgp_apply<DIM, float><<<gb, sl.chunk, 0, s>>>(g, sl, tst, lf.X[0], S->p32, S->q32, S->w32, S->y32, S->red, 1);
      else
        v_cgp_apply<DIM, double><<<gb, sl.chunk, 0, s>>>(g, sl, tst, ld.X[0], S->p64, S->q64, S->w64, S->y64, S->red, 1);
      *bytes = 6.0 * sz * N;
    } else if (!strcmp(name, "cgp_apply_acc")) {  // the same with the difference-form apply and y in FP64
      if (!mixed) return FISHGPU_ERR_UNSUPPORTED;
      v_cgp_apply<DIM, float, false, true><<<gb, sl.chunk, 0, s>>>(g, sl, tst, lf.X[0], S->p32, S->q32, S->w32, S->y64,
                                                                 S->red, 1);
      *bytes = (4.0 + 4.0 + 8.0 + 4.0 + 4.0 + 8.0) * N;
    } else if (!strcmp(name, "cgp_apply_acc_pair")) {  // the solve's pair of iterations: y left alone, then
      // both owed updates (reads z, p_old, p_older, y64; writes p, w, y64); one rep is the two launches
      if (!mixed) return FISHGPU_ERR_UNSUPPORTED;
      v_cgp_apply<DIM, float, false, true, 1><<<gb, sl.chunk, 0, s>>>(g, sl, tst, lf.X[0], S->p32, S->q32, S->w32,
                                                                    S->y64, S->red, 1);
      v_cgp_apply<DIM, float, false, true, 2><<<gb, sl.chunk, 0, s>>>(g, sl, tst, lf.X[0], S->q32, S->p32, S->w32,
                                                                    S->y64, S->red, 1);
      *bytes = (4.0 + 4.0 + 4.0 + 4.0) * N + (4.0 + 4.0 + 4.0 + 8.0 + 4.0 + 4.0 + 8.0) * N;
    } else if (!strcmp(name, "cgp_apply_tma")) {  // the accurate form from the TMA ring (3D)
      if (!mixed || !launch_cgp_tma(S, g, tst, lf.X[0], S->p32, S->q32, S->w32, S->y64, 1))
        return FISHGPU_ERR_UNSUPPORTED;
      *bytes = (4.0 + 4.0 + 8.0 + 4.0 + 4.0 + 8.0) * N;
    } else if (!strcmp(name, "post2")) {  // both post-smoothing steps fused: reads b, x0, writes x2
      if constexpr (DIM == 3) {
        if (!mixed) return FISHGPU_ERR_UNSUPPORTED;
        if (!lf.pz.ok()) return FISHGPU_ERR_UNSUPPORTED;
        v_cheb_post2z<false><<<lf.pz.blocks(), lf.pz.threads, lf.pz.smem, s>>>(g, lf.pz, nullptr, S->r32, lf.X[0],
                                                                               lf.X[2], 0.5f, 0.5f, 0.5f, 0.1f);
        *bytes = 3.0 * sz * N;
      } else {
        return FISHGPU_ERR_UNSUPPORTED;
      }
    } else if (!strcmp(name, "smooth_zero")) {  // two steps from zero: reads b, writes x
      if (mixed)
        v_cheb2_zero<DIM, float><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r32, lf.X[0], 0.5f, 0.1f);
      else
        v_cheb2_zero<DIM, double><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, ld.X[0], 0.5, 0.1);
      *bytes = 2.0 * sz * N;
    } else if (!strcmp(name, "resid")) {
      if (mixed)
        v_resid<DIM, float><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r32, lf.X[0], lf.X[1]);
      else
        v_resid<DIM, double><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, ld.X[0], ld.X[1]);
      *bytes = 3.0 * sz * N;
    } else if (!strcmp(name, "apply")) {
      if (mixed)
        v_apply_dot<DIM, float><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->p32, S->w32, S->red, 1, FIN_STORE, S->dval + 2);
      else
        v_apply_dot<DIM, double><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->p64, S->w64, S->red, 1, FIN_STORE, S->dval + 2);
      *bytes = 2.0 * sz * N;
    } else if (!strcmp(name, "cg_update")) {
      if (mixed)
        v_cg_r<float, false><<<gb, sl.chunk, 0, s>>>(g, sl, tst, S->w32, S->r32, S->red, 1);
      else
        v_cg_r<double, false><<<gb, sl.chunk, 0, s>>>(g, sl, tst, S->w64, S->r64, S->red, 1);
      *bytes = 3.0 * sz * N;
    } else if (!strcmp(name, "demote")) {  // an inner solve's set-up: r32 = r64 / ||r64||, r32.r32
      if (!mixed) return FISHGPU_ERR_UNSUPPORTED;
      if (q == 0) k_inv_norm<<<1, 1, 0, s>>>(S->dval, S->dval + 6);
      v_demote_init<<<gb, sl.chunk, 0, s>>>(g, sl, tst, S->r64, S->dval + 6, S->r32, S->red, 1);
      *bytes = (8.0 + 4.0) * N;
    } else if (!strcmp(name, "restrict")) {
      if (mixed)
        v_restrict<DIM, float><<<slot_blocks(cf.sl), cf.sl.chunk, 0, s>>>(g, cf.g, cf.sl, nullptr, lf.X[0], cf.b);
      else
        v_restrict<DIM, double><<<slot_blocks(cd.sl), cd.sl.chunk, 0, s>>>(g, cd.g, cd.sl, nullptr, ld.X[0], cd.b);
      *bytes = sz * N * (1.0 + 1.0 / (1 << DIM));
    } else if (!strcmp(name, "resid_restrict")) {  // fused: reads b, x; writes the coarse b
      if constexpr (DIM == 3) {
        const bool ok = mixed ? launch_resid_restrict<float>(S, g, cf.g, S->r32, lf.X[0], cf.b, nullptr)
                              : launch_resid_restrict<double>(S, g, cd.g, S->r64, ld.X[0], cd.b, nullptr);
        if (!ok) return FISHGPU_ERR_UNSUPPORTED;
        *bytes = sz * N * (2.0 + 1.0 / 8.0);
      } else {
        return FISHGPU_ERR_UNSUPPORTED;
      }
    } else if (!strcmp(name, "prolong")) {
      if (mixed)
        v_prolong<DIM, float><<<slot_blocks(cf.sl), cf.sl.chunk, 0, s>>>(g, cf.g, cf.sl, nullptr, cf.X[0], lf.X[0]);
      else
        v_prolong<DIM, double><<<slot_blocks(cd.sl), cd.sl.chunk, 0, s>>>(g, cd.g, cd.sl, nullptr, cd.X[0], ld.X[0]);
      *bytes = sz * N * (2.0 + 1.0 / (1 << DIM));
    } else if (!strcmp(name, "residual64")) {
      v_resid<DIM, double><<<gb, sl.chunk, 0, s>>>(g, sl, nullptr, S->r64, S->y64, S->u64);
      *bytes = 3.0 * 8.0 * N;
    } else {
      return FISHGPU_ERR_ARG;
    }
  }
  FG_CUDA(cudaEventRecord(S->ev1, s));
  FG_CUDA(cudaEventSynchronize(S->ev1));
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaEventElapsedTime(&t, S->ev0, S->ev1));
  *ms = (double)t / reps;
  if (tst) {
    int done = 0;
    FG_CUDA(cudaMemcpy(&done, &tst->done, sizeof(int), cudaMemcpyDeviceToHost));
    if (done) return FISHGPU_ERR_NONFINITE;  // the state stopped: launches exited early
  }
  return FISHGPU_OK;
}

// ------------------------------------------------------------------ hooks
// For other solvers of this library that precondition with the Poisson
// multigrid hierarchy of a 2D mixed-form solver (mg_hooks.cuh).
const Geom &solver_fine(const fishgpu_solver *S) { return S->fine; }
const Slots &solver_slots(const fishgpu_solver *S) { return S->sf; }
cudaStream_t solver_stream(const fishgpu_solver *S) { return S->stream; }

bool solver_coarse32(const fishgpu_solver *S, CoarseView *c) {
  if (S->o.ctx.dim != 2 || S->o.precision != FISHGPU_MIXED || S->o.pc_type != FISHGPU_PC_MG || S->h32.nlev != 1)
    return false;
  const Level<float> &lv = S->h32.lev[0];
  c->g = lv.g;
  c->S0 = lv.S[0];
  c->S1 = lv.S[1];
  c->ilam = lv.ilam;
  c->work = lv.work;
  c->x = lv.X[0];
  c->n0 = lv.n[0];
  c->n1 = lv.n[1];
  const size_t smb = coarse_smem_bytes<float>(2, lv.n[0], lv.n[1], 1);
  c->smem = (lv.n[0] * lv.n[1] > 0 && smb <= 48 * 1024) ? smb : 0;
  c->dinv = (float)(1.0 / lv.g.scdiag);
  return true;
}

bool solver_persist32(fishgpu_solver *S, const void *kernel, long long tail_pts, PersistArgs<float> *a,
                      int *blocks, size_t *smem) {
  const fishgpu_opts &o = S->o;
  Hier<float> &H = S->h32;
  if (o.ctx.dim != 2 || o.precision != FISHGPU_MIXED || o.pc_type != FISHGPU_PC_MG ||
      o.smooth_type != FISHGPU_SMOOTH_CHEBYSHEV || o.smooth_its != 2 || o.mg_cycles != 1 || H.nlev < 2 ||
      H.nlev > kMaxPersistLevels)
    return false;
  std::vector<long long> pts(H.nlev);
  for (int l = 0; l < H.nlev; l++) pts[l] = level_points(H.lev[l].g);
  int btop = 0;
  for (int l = 1; l <= H.nlev - 2; l++)
    if (pts[l] <= tail_pts) btop = l;
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop || nsm < 1) {
    cudaGetLastError();
    return false;
  }
  size_t coarse = 0, psmem = 0;
  int copy_off = -1;
  tail_smem_plan(2, H.lev[0].n, sizeof(float), btop, pts.data(), &coarse, &copy_off, &psmem);
  if (!allow_smem(kernel, psmem)) {
    copy_off = -1;
    psmem = coarse;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 512, psmem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return false;
  }
  if (!S->hplev) {  // the fine level's b is the caller's right-hand side (formed on the fly)
    std::vector<TailLevel<float>> tl(H.nlev);
    for (int l = 0; l < H.nlev; l++) tl[l] = tail_level<float>(H.lev[l], l > 0);
    if (dalloc(S, &S->hplev, (size_t)H.nlev) ||
        cudaMemcpyAsync(S->hplev, tl.data(), sizeof(TailLevel<float>) * H.nlev, cudaMemcpyHostToDevice, S->stream) !=
            cudaSuccess) {
      cudaGetLastError();
      S->hplev = nullptr;
      return false;
    }
  }
  if (!S->pbar && (dalloc(S, &S->pbar, 2) || dalloc(S, &S->ppart, (size_t)4 * nsm))) return false;
  memset(a, 0, sizeof(*a));
  a->lv = S->hplev;
  a->top = H.nlev - 1;
  a->btop = btop;
  a->part = S->ppart;
  a->bar = S->pbar;
  a->fault = S->fault;
  const Level<float> &c = H.lev[0];
  a->S0 = c.S[0];
  a->S1 = c.S[1];
  a->S2 = c.S[2];
  a->ilam = c.ilam;
  a->work = c.work;
  a->n0 = c.n[0];
  a->n1 = c.n[1];
  a->n2 = c.n[2];
  a->smem = coarse ? 1 : 0;
  a->dinv = (float)(1.0 / c.g.scdiag);
  a->copy_off = copy_off;
  *blocks = (int)std::max<long long>(1, std::min<long long>(nsm, (pts[H.nlev - 1] + 511) / 512));
  *smem = psmem;
  return true;
}

const float *solver_vcycle32(fishgpu_solver *S, const float *r, KspState *st) {
  if (S->o.ctx.dim != 2 || S->o.precision != FISHGPU_MIXED || S->o.pc_type != FISHGPU_PC_MG) return nullptr;
  KspState *saved = S->st;
  S->st = st;  // the V-cycle's kernels return at once when st->done is set
  enq_pc<2, float>(S, S->h32, r, -1);
  S->st = saved;
  return S->h32.z;
}

}  // namespace fg

// ------------------------------------------------------------------ C ABI
extern "C" int fishgpu_solver_destroy(fishgpu_solver *S) {
  if (!S) return FISHGPU_OK;
  if (S->stream) cudaStreamSynchronize(S->stream);
  if (S->gexec) cudaGraphExecDestroy(S->gexec);
  if (S->gloop) cudaGraphExecDestroy(S->gloop);
  if (S->gexec_init) cudaGraphExecDestroy(S->gexec_init);
  for (cudaGraphExec_t &e : S->gexec_init64)
    if (e) cudaGraphExecDestroy(e);
  for (void *p : S->allocs) cudaFree(p);
  if (S->st_h) cudaFreeHost(S->st_h);
  if (S->hval) cudaFreeHost(S->hval);
  if (S->mout_h) cudaFreeHost(S->mout_h);
  if (S->ev0) cudaEventDestroy(S->ev0);
  if (S->ev1) cudaEventDestroy(S->ev1);
  if (S->cs_in) cudaStreamDestroy(S->cs_in);
  if (S->cs_out) cudaStreamDestroy(S->cs_out);
  if (S->own_stream && S->stream) cudaStreamDestroy(S->stream);
  delete S;
  return FISHGPU_OK;
}

static int validate_opts(const fishgpu_opts *o) {
  if (!o) return FISHGPU_ERR_ARG;
  const int dim = o->ctx.dim;
  if (dim < 1 || dim > 3) return FISHGPU_ERR_ARG;
  if (o->mx < 3 || (dim >= 2 && o->my < 3) || (dim >= 3 && o->mz < 3)) return FISHGPU_ERR_ARG;
  if (!(o->ctx.cx > 0) || !(o->ctx.cy > 0) || !(o->ctx.cz > 0)) return FISHGPU_ERR_ARG;
  if (!(o->ctx.Lx > 0) || !(o->ctx.Ly > 0) || !(o->ctx.Lz > 0)) return FISHGPU_ERR_ARG;
  if (o->ctx.problem < 0 || o->ctx.problem > FISHGPU_USER) return FISHGPU_ERR_ARG;
  if (o->ctx.problem == FISHGPU_USER && (!o->ctx.f) != (!o->ctx.g)) return FISHGPU_ERR_ARG;
  if (o->pc_type < 0 || o->pc_type > FISHGPU_PC_MG) return FISHGPU_ERR_UNSUPPORTED;
  if (o->smooth_its < 1 || o->max_it < 0 || o->mg_cycles < 1 || o->mg_cycles > 2) return FISHGPU_ERR_ARG;
  if (o->precision != FISHGPU_FP64 && o->precision != FISHGPU_MIXED) return FISHGPU_ERR_ARG;
  if (o->loop_cap < 0 || !(o->first_floor_scale > 0) || o->inner_accurate < -1 || o->inner_accurate > 1 ||
      o->vtail_points < 0)
    return FISHGPU_ERR_ARG;
  if (o->precision == FISHGPU_MIXED && o->pc_type != FISHGPU_PC_MG) return FISHGPU_ERR_UNSUPPORTED;
  if (o->initial_type < 0 || o->initial_type > FISHGPU_INITIAL_GIVEN) return FISHGPU_ERR_ARG;
  if (!(o->rtol >= 0) || !(o->atol >= 0) || !(o->dtol > 0)) return FISHGPU_ERR_ARG;
  const long long N = (long long)o->mx * (dim >= 2 ? o->my : 1) * (dim >= 3 ? o->mz : 1);
  if (N > (1LL << 40)) return FISHGPU_ERR_ARG;
  return FISHGPU_OK;
}

extern "C" int fishgpu_solver_create(const fishgpu_opts *o, void *stream, fishgpu_solver **out) {
  if (!out) return FISHGPU_ERR_ARG;
  *out = nullptr;
  int rc = validate_opts(o);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FISHGPU_ERR_NODEVICE;
  }
  fishgpu_solver *S = new fishgpu_solver();
  S->o = *o;
  const int dim = o->ctx.dim;
  if (stream) {
    S->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete S;
      return FISHGPU_ERR_CUDA;
    }
    S->own_stream = true;
  }
  S->dense = make_geom(dim, o->mx, dim >= 2 ? o->my : 1, dim >= 3 ? o->mz : 1, o->ctx.Lx, o->ctx.Ly, o->ctx.Lz,
                       o->ctx.cx, o->ctx.cy, o->ctx.cz);
  S->fine = padded(S->dense);
  S->sf = make_slots(S->fine, ZC, 2432, level_chunk(S->fine, 0));
  S->sfst = S->sf;
  S->Lf = launch_for(S->fine);
  S->gfl = flat_grid(S->sf.tot4);
  S->prob = Prob{o->ctx.problem, dim, o->ctx.cx, o->ctx.cy, o->ctx.cz, o->ctx.f, o->ctx.g, S->dense.pitch,
                 S->dense.plane};
  const size_t N = nelem(S->fine);
  const long long dofs = (long long)S->dense.plane * S->dense.mz;
  // iterations per graph launch: even, since consecutive iterations alternate the two p buffers
  // iterations per graph body: with the device-side loop a body costs no host
  // round trip, so short bodies waste fewer early-exit launches after the stop
  S->giters = o->graph_iters > 0 ? o->graph_iters : (o->device_loop || dofs >= (1LL << 20) ? 2 : 4);
  S->giters += S->giters & 1;
  // FP64 form: the user's norm; mixed form: the inner CG stops on its own
  // (unpreconditioned) residual, which the refinement loop relates to the true one
  S->ksp_norm = o->precision == FISHGPU_MIXED ? FISHGPU_NORM_UNPRECONDITIONED : o->norm_type;
#define CK(x)                            \
  do {                                   \
    if ((rc = (x)) != FISHGPU_OK) {      \
      fishgpu_solver_destroy(S);         \
      return rc;                         \
    }                                    \
  } while (0)
  if (cudaMallocHost((void **)&S->st_h, sizeof(KspState)) != cudaSuccess ||
      cudaMallocHost((void **)&S->hval, sizeof(double) * 8) != cudaSuccess ||
      cudaEventCreate(&S->ev0) != cudaSuccess || cudaEventCreate(&S->ev1) != cudaSuccess) {
    fishgpu_solver_destroy(S);
    return FISHGPU_ERR_CUDA;
  }
  int cap = reduction_blocks(S);
  if (dim == 3 && o->precision == FISHGPU_MIXED) {
    const Post2Z pz = post2z_shape(S->fine);
    if (pz.ok()) cap = std::max(cap, (int)pz.blocks());  // the fused post-smoother reduces too
    const int smax = 96 * 1024;  // the largest ring of any level (3 x (R+2) x P4 float4 <= 3 x 1056 x 16 B)
    if (cudaFuncSetAttribute(v_cheb_post2z<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax) != cudaSuccess ||
        cudaFuncSetAttribute(v_cheb_post2z<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax) !=
            cudaSuccess) {
      fishgpu_solver_destroy(S);
      return FISHGPU_ERR_CUDA;
    }
  }
  CK(dalloc(S, &S->st, 1));
  CK(dalloc(S, &S->fault, 1));
  CK(dalloc(S, &S->dval, 8));
  if (dim == 3 &&
      (cudaFuncSetAttribute(v_cgp_apply_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CgRing::SMEM) !=
           cudaSuccess ||
       cudaFuncSetAttribute(v_resid_restrict<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)RRRing<float>::SMEM) != cudaSuccess ||
       cudaFuncSetAttribute(v_resid_restrict<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)RRRing<double>::SMEM) != cudaSuccess)) {
    fishgpu_solver_destroy(S);
    return FISHGPU_ERR_CUDA;
  }
  CK(dalloc(S, &S->red.partials, (size_t)2 * 2 * cap));  // two slots of up to two values
  CK(dalloc(S, &S->red.tickets, 4));
  S->red.cap = cap;
  S->red.tcap = 1;
  CK(dalloc(S, &S->u64, N));
  CK(dalloc(S, &S->beff, N));
  CK(dalloc(S, &S->y64, N));
  CK(dalloc(S, &S->r64, N));
  if (o->ctx.problem == FISHGPU_USER && !o->ctx.f) {  // the solver owns f and g (dense)
    const size_t Nd = (size_t)dofs;
    CK(dalloc(S, &S->f_own, Nd));
    CK(dalloc(S, &S->g_own, Nd));
    S->prob.f = S->f_own;
    S->prob.g = S->g_own;
    S->o.ctx.f = S->f_own;
    S->o.ctx.g = S->g_own;
  }
  const bool fuse_r = fuse_cgr_ok(*o, 0, o->pc_type == FISHGPU_PC_MG ? o->mg_levels : 1);
  if (o->precision == FISHGPU_FP64) {
    CK(dalloc(S, &S->p64, N));
    CK(dalloc(S, &S->q64, N));
    CK(dalloc(S, &S->w64, N));
    CK(build_hier<double>(S, S->h64));
  } else {
    CK(dalloc(S, &S->b64, N));
    CK(dalloc(S, &S->r32, N));
    CK(dalloc(S, &S->p32, N));
    CK(dalloc(S, &S->q32, N));
    CK(dalloc(S, &S->w32, N));
    CK(dalloc(S, &S->y32, N));
    if (fuse_r) CK(dalloc(S, &S->r32b, N));
    CK(build_hier<float>(S, S->h32));
  }
#undef CK
  if (cudaStreamSynchronize(S->stream) != cudaSuccess) {
    fishgpu_solver_destroy(S);
    return FISHGPU_ERR_CUDA;
  }
  *out = S;
  return FISHGPU_OK;
}

extern "C" long long fishgpu_solver_bytes(const fishgpu_solver *S) { return S ? S->bytes : 0; }

// Device bytes fishgpu_solver_create would allocate for these options (plus
// the host-array buffers of fishgpu_solver_solve_host), without allocating.
extern "C" long long fishgpu_solver_estimate_bytes(const fishgpu_opts *o) {
  if (validate_opts(o)) return -1;
  const int dim = o->ctx.dim;
  auto rnd = [](long long b) { return (b + 255) / 256 * 256; };
  Geom d = make_geom(dim, o->mx, dim >= 2 ? o->my : 1, dim >= 3 ? o->mz : 1, 1, 1, 1, 1, 1, 1);
  Geom g = padded(d);
  const long long N = (long long)nelem(g), Nd = (long long)d.plane * d.mz;
  long long b = rnd(sizeof(KspState)) + rnd(4) + rnd(64);  // state, fault word, scalars
  const long long cap = slot_blocks(make_slots(g, ZC, 2432, level_chunk(g, 0)));
  b += rnd(8LL * 4 * cap) + rnd(16);
  b += 4 * rnd(8LL * N);                                          // u, beff, y, r
  if (o->ctx.problem == FISHGPU_USER && !o->ctx.f) b += 3 * rnd(8LL * Nd);  // f, g, u (host-array form)
  const int es = o->precision == FISHGPU_MIXED ? 4 : 8;
  if (o->precision == FISHGPU_MIXED) b += rnd(8LL * N) + 5 * rnd(4LL * N);  // b64; r p q w y (FP32)
  else b += 3 * rnd(8LL * N);                                              // p q w
  if (fuse_cgr_ok(*o, 0, o->pc_type == FISHGPU_PC_MG ? o->mg_levels : 1)) b += rnd((long long)es * N);  // r2
  if (o->pc_type != FISHGPU_PC_MG) return b + rnd((long long)es * N);
  Geom lv = g;
  std::vector<long long> pts(o->mg_levels, 0);  // nodes per level (build_tail's choice below)
  for (int l = o->mg_levels - 1; l >= 0; l--) {
    pts[l] = level_points(lv);
    const long long Nl = (long long)nelem(lv);
    b += 3 * rnd((long long)es * Nl) + (l > 0 ? rnd((long long)es * Nl) : 0) + (l < o->mg_levels - 1 ? rnd((long long)es * Nl) : 0);
    if (l > 0) {
      const int m[3] = {lv.mx, lv.my, lv.mz};
      for (int q = 0; q < dim; q++)
        if (m[q] < 3 || (m[q] - 1) % 2) return -1;
      lv = padded(make_geom(dim, (lv.mx - 1) / 2 + 1, dim >= 2 ? (lv.my - 1) / 2 + 1 : 1,
                            dim >= 3 ? (lv.mz - 1) / 2 + 1 : 1, 1, 1, 1, 1, 1, 1));
    } else {
      const int m[3] = {lv.mx, lv.my, lv.mz};
      long long ni = 1;
      for (int q = 0; q < dim; q++) ni *= m[q] - 2;
      for (int q = 0; q < dim && ni > 0; q++) b += rnd((long long)es * (m[q] - 2) * (m[q] - 2));
      if (ni > 0) b += rnd((long long)es * ni) + rnd((long long)es * 2 * ni);  // 1/lambda, work area
    }
  }
  if (o->vtail && o->smooth_type == FISHGPU_SMOOTH_CHEBYSHEV && o->smooth_its == 2 && o->mg_cycles == 1 &&
      dim >= 2 && o->mg_levels >= 3) {  // the V-cycle tail's level table
    int top = 0;
    for (int l = 1; l <= o->mg_levels - 2; l++)
      if (pts[l] <= tail_max_points(*o, es)) top = l;
    if (top > 0)
      b += rnd((long long)(es == 4 ? sizeof(TailLevel<float>) : sizeof(TailLevel<double>)) * (top + 1));
  }
  {  // the persistent solve's level table, grid barrier and partial sums
    int n[3] = {1, 1, 1}, btop = 0, nsm = 0, copy_off = -1;
    size_t coarse = 0, psmem = 0;
    for (int q = 0; q < dim; q++) n[q] = (q == 0 ? lv.mx : q == 1 ? lv.my : lv.mz) - 2;
    const int L = o->mg_levels;
    const int blocks =
        es == 4 ? persist_shape<float>(*o, dim, false, L, pts.data(), n, &btop, &nsm, &coarse, &copy_off, &psmem)
                : persist_shape<double>(*o, dim, false, L, pts.data(), n, &btop, &nsm, &coarse, &copy_off, &psmem);
    if (blocks)
      b += rnd((long long)(es == 4 ? sizeof(TailLevel<float>) : sizeof(TailLevel<double>)) * L) + rnd(8) +
           rnd(8LL * 4 * nsm) + (es == 4 ? rnd((long long)sizeof(MixedOut)) : 0);
  }
  return b;
}

extern "C" int fishgpu_solver_solve(fishgpu_solver *S, double *u_dev, fishgpu_report *rep) {
  if (!S || !u_dev || !rep) return FISHGPU_ERR_ARG;
  memset(rep, 0, sizeof(*rep));
  rep->dofs = (long long)S->dense.plane * S->dense.mz;
  int rc;
  switch (S->o.ctx.dim) {
  case 1: rc = solve_dim<1>(S, u_dev, rep); break;
  case 2: rc = solve_dim<2>(S, u_dev, rep); break;
  default: rc = solve_dim<3>(S, u_dev, rep); break;
  }
  if (rc) return rc;
  // error report against the exact solution (fish.c:250-276)
  if (S->o.ctx.problem != FISHGPU_USER) {
    fishgpu_info info;
    memset(&info, 0, sizeof(info));
    info.dim = S->o.ctx.dim;
    info.mx = S->dense.mx; info.my = S->dense.my; info.mz = S->dense.mz;
    info.xm = info.mx; info.ym = info.my; info.zm = info.mz;
    info.xmax[0] = S->o.ctx.Lx; info.xmax[1] = S->o.ctx.Ly; info.xmax[2] = S->o.ctx.Lz;
    fishgpu_ctx c = S->o.ctx;
    rc = ErrorNorms_gpu(&info, u_dev, &c, &rep->errinf, &rep->err2h, (void *)S->stream);
    if (rc) return rc;
    S->launches += 1;
  }
  rep->launches = S->launches;
  if (rep->reason == R_DIVERGED_NANORINF) return FISHGPU_ERR_NONFINITE;
  if (rep->reason < 0) return FISHGPU_ERR_NOT_CONVERGED;
  return FISHGPU_OK;
}

extern "C" int fishgpu_solve(const fishgpu_opts *o, double *u_dev, fishgpu_report *rep) {
  fishgpu_solver *S = nullptr;
  int rc = fishgpu_solver_create(o, nullptr, &S);
  if (rc) return rc;
  rc = fishgpu_solver_solve(S, u_dev, rep);
  fishgpu_solver_destroy(S);
  return rc;
}

namespace fg {
// Boundary nodes of a dense mx x my x mz array, enumerated face by face
// (3D: k faces, then j faces of the inner planes, then i faces of the inner
// rows; 2D: j rows, then i ends of the inner rows; 1D: both ends).
__host__ __device__ inline long long bdry_count(int dim, int mx, int my, int mz) {
  if (dim == 1) return mx > 1 ? 2 : 1;
  if (dim == 2) return 2LL * mx + 2LL * (my - 2);
  return 2LL * mx * my + 2LL * mx * (mz - 2) + 2LL * (my - 2) * (mz - 2);
}

// dst[n] = src[n] on the boundary nodes only: the solver reads the boundary
// data g nowhere else, so a host g in pinned memory is gathered through the
// device's mapping of it instead of being copied whole (6 faces instead of
// the volume in 3D).
template <int DIM>
__global__ void __launch_bounds__(256) k_gather_bdry(int mx, int my, int mz, const double *__restrict__ src,
                                                     double *__restrict__ dst) {
  const long long tot = bdry_count(DIM, mx, my, mz);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    int i, j = 0, k = 0;
    if (DIM == 1) {
      i = t == 0 ? 0 : mx - 1;
    } else if (DIM == 2) {
      if (t < 2LL * mx) {
        i = (int)(t % mx);
        j = t < mx ? 0 : my - 1;
      } else {
        const long long r = t - 2LL * mx;
        j = 1 + (int)(r / 2);
        i = (r & 1) ? mx - 1 : 0;
      }
    } else {
      const long long fz = 2LL * mx * my, fy = 2LL * mx * (mz - 2);
      if (t < fz) {
        k = t < (long long)mx * my ? 0 : mz - 1;
        const long long r = t % ((long long)mx * my);
        j = (int)(r / mx);
        i = (int)(r % mx);
      } else if (t < fz + fy) {
        const long long r = t - fz;
        k = 1 + (int)(r / (2LL * mx));
        const long long q = r % (2LL * mx);
        j = q < mx ? 0 : my - 1;
        i = (int)(q % mx);
      } else {
        const long long r = t - fz - fy;
        k = 1 + (int)(r / (2LL * (my - 2)));
        const long long q = r % (2LL * (my - 2));
        j = 1 + (int)(q / 2);
        i = (q & 1) ? mx - 1 : 0;
      }
    }
    const long long n = ((long long)k * my + j) * mx + i;
    dst[n] = src[n];
  }
}

// dst = src, n doubles, both 16-byte aligned, one side pinned host memory
// through its device mapping: the pipelined host-array solves move f and u
// with this kernel instead of the copy engines, on whose queues the solve's
// own small state copies would otherwise wait behind the 1 GB transfers.
// Blocks of 128 threads with few registers fit beside a stencil kernel's
// blocks; four 16-byte loads in flight per thread.
static __global__ void __launch_bounds__(128) k_copy_mapped(const double2 *__restrict__ src, double2 *__restrict__ dst,
                                                          long long n) {
  const long long n2 = n / 2, stride = (long long)gridDim.x * blockDim.x;
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)  // the odd last element
    reinterpret_cast<double *>(dst)[n - 1] = reinterpret_cast<const double *>(src)[n - 1];
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n2; i += 4 * stride) {
    const double2 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n2; i += stride) dst[i] = src[i];
}
}  // namespace fg

// A device-usable address of pinned (page-locked, mapped) host memory, or
// null for any other pointer.
static const double *pinned_device_view(const double *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? (const double *)a.devicePointer : nullptr;
}

extern "C" long long fishgpu_solver_host_bytes_in(const fishgpu_solver *S, const double *g_host) {
  // bytes fishgpu_solver_solve_host moves to the device for f and g (FISHGPU_USER)
  if (!S || S->o.ctx.problem != FISHGPU_USER) return 0;
  const long long N = (long long)S->dense.plane * S->dense.mz;
  long long b = 8LL * N;  // f
  if (g_host) b += pinned_device_view(g_host) ? 8LL * fg::bdry_count(S->dense.dim, S->dense.mx, S->dense.my, S->dense.mz)
                                              : 8LL * N;
  return b;
}

// g into the solver's g buffer on its stream: boundary values only, read in
// place from pinned host memory; all of it from pageable memory; zeros for
// NULL (the solver reads g nowhere but on the boundary)
static int stage_g(fishgpu_solver *S, const double *g_host) {
  cudaStream_t s = S->stream;
  const size_t N = (size_t)S->dense.plane * S->dense.mz;
  const double *gdev = g_host ? pinned_device_view(g_host) : nullptr;
  if (gdev) {
    const Geom &d = S->dense;
    const long long nb = fg::bdry_count(d.dim, d.mx, d.my, d.mz);
    const unsigned blocks = (unsigned)std::min<long long>((nb + 255) / 256, 4LL * sm_count());
    if (d.dim == 1) fg::k_gather_bdry<1><<<blocks, 256, 0, s>>>(d.mx, d.my, d.mz, gdev, S->g_own);
    else if (d.dim == 2) fg::k_gather_bdry<2><<<blocks, 256, 0, s>>>(d.mx, d.my, d.mz, gdev, S->g_own);
    else fg::k_gather_bdry<3><<<blocks, 256, 0, s>>>(d.mx, d.my, d.mz, gdev, S->g_own);
    return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  }
  return (g_host ? cudaMemcpyAsync(S->g_own, g_host, sizeof(double) * N, cudaMemcpyHostToDevice, s)
                 : cudaMemsetAsync(S->g_own, 0, sizeof(double) * N, s)) == cudaSuccess
             ? FISHGPU_OK
             : FISHGPU_ERR_CUDA;
}

extern "C" int fishgpu_solver_solve_host(fishgpu_solver *S, const double *f_host, const double *g_host,
                                         double *u_host, fishgpu_report *rep) {
  if (!S || !u_host || !rep) return FISHGPU_ERR_ARG;
  const bool user = S->o.ctx.problem == FISHGPU_USER;
  if (user && (!S->f_own || !f_host)) return FISHGPU_ERR_ARG;  // g_host NULL: zero boundary data
  const size_t N = (size_t)S->dense.plane * S->dense.mz;
  cudaStream_t s = S->stream;
  if (!S->u_own) {
    int rc = dalloc(S, &S->u_own, N);
    if (rc) return rc;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return FISHGPU_ERR_CUDA;
  int rc = FISHGPU_OK;
  cudaEventRecord(e0, s);
  if (user && cudaMemcpyAsync(S->f_own, f_host, sizeof(double) * N, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = FISHGPU_ERR_CUDA;
  if (user && !rc) rc = stage_g(S, g_host);
  if (!rc && S->o.initial_type == FISHGPU_INITIAL_GIVEN &&
      cudaMemcpyAsync(S->u_own, u_host, sizeof(double) * N, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = FISHGPU_ERR_CUDA;
  const int src = rc ? rc : fishgpu_solver_solve(S, S->u_own, rep);
  if (!rc && src != FISHGPU_OK && src != FISHGPU_ERR_NOT_CONVERGED) rc = src;
  if (!rc && cudaMemcpyAsync(u_host, S->u_own, sizeof(double) * N, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = FISHGPU_ERR_CUDA;
  cudaEventRecord(e1, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = FISHGPU_ERR_CUDA;
  float ms = 0.f;
  if (!rc && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) rep->solve_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc ? rc : src;
}

// n host-array solves in order, pipelined: while problem k is solved, f of
// problem k+1 comes in (copy stream cs_in) and u of problem k-1 goes out
// (cs_out), each into or out of the second of two device buffers.  Each
// problem's results are those of fishgpu_solver_solve_host.
// dst = src (n doubles) on stream st: by k_copy_mapped when the host side is
// pinned memory (host is dst for d2h) and both ends are 16-byte aligned, else
// by the copy engine
static int copy_host(double *dst, const double *src, size_t n, bool d2h, cudaStream_t st) {
  const double *hv = pinned_device_view(d2h ? dst : src);
  const double *s = d2h ? src : hv;
  double *d = d2h ? const_cast<double *>(hv) : dst;
  if (hv && ((uintptr_t)s & 15) == 0 && ((uintptr_t)d & 15) == 0) {
    fg::k_copy_mapped<<<64, 128, 0, st>>>(reinterpret_cast<const double2 *>(s), reinterpret_cast<double2 *>(d),
                                          (long long)n);
    return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
  }
  return cudaMemcpyAsync(dst, src, sizeof(double) * n, d2h ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, st) ==
                 cudaSuccess
             ? FISHGPU_OK
             : FISHGPU_ERR_CUDA;
}

extern "C" int fishgpu_solver_solve_host_many(fishgpu_solver *S, int n, const double *const *f_host,
                                              const double *const *g_host, double *const *u_host,
                                              fishgpu_report *reps) {
  if (!S || n < 0 || (n && (!f_host || !u_host || !reps))) return FISHGPU_ERR_ARG;
  if (S->o.ctx.problem != FISHGPU_USER || !S->f_own) return FISHGPU_ERR_ARG;
  for (int k = 0; k < n; k++)
    if (!f_host[k] || !u_host[k]) return FISHGPU_ERR_ARG;
  if (!n) return FISHGPU_OK;
  const size_t N = (size_t)S->dense.plane * S->dense.mz, bytes = sizeof(double) * N;
  cudaStream_t s = S->stream;
  int rc = FISHGPU_OK;
  if (!S->u_own && (rc = dalloc(S, &S->u_own, N))) return rc;
  if (!S->f_stage && ((rc = dalloc(S, &S->f_stage, N)) || (rc = dalloc(S, &S->u_stage, N)))) return rc;
  if (!S->cs_in && (cudaStreamCreateWithFlags(&S->cs_in, cudaStreamNonBlocking) != cudaSuccess ||
                    cudaStreamCreateWithFlags(&S->cs_out, cudaStreamNonBlocking) != cudaSuccess))
    return FISHGPU_ERR_CUDA;
  // Two f and two u buffers alternate (the solver's own and the staging ones): problem k reads
  // fb[k & 1] (the solve takes f by value at its start, in S->prob, never from a captured graph) and
  // writes ub[k & 1] (a launch parameter); f of problem k+1 comes into the other f buffer while
  // problem k is solved, and u of problem k-1 leaves the other u buffer.
  double *fb[2] = {S->f_own, S->f_stage}, *ub[2] = {S->u_own, S->u_stage};
  cudaEvent_t e_in = nullptr, e_z = nullptr, e_us = nullptr, e_out[2] = {nullptr, nullptr};
  if (cudaEventCreateWithFlags(&e_in, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e_z, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e_us, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e_out[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e_out[1], cudaEventDisableTiming) != cudaSuccess) {
    rc = FISHGPU_ERR_CUDA;
  }
  int src = FISHGPU_OK;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = FISHGPU_ERR_CUDA;
    return !rc;
  };
  // the staging buffers were zeroed on the solver's stream: the copy streams start after that
  if (!rc && ok(cudaEventRecord(e_z, s)) && ok(cudaStreamWaitEvent(S->cs_in, e_z, 0)) &&
      ok(cudaStreamWaitEvent(S->cs_out, e_z, 0)) && !(rc = copy_host(fb[0], f_host[0], N, false, S->cs_in)))
    ok(cudaEventRecord(e_in, S->cs_in));
  for (int k = 0; k < n && !rc; k++) {
    double *fk = fb[k & 1], *uk = ub[k & 1];
    // f of problem k has arrived; problem k+1's goes into the other buffer, which problem k-1 (done:
    // fishgpu_solver_solve returns after its solve) was the last to read
    if (!ok(cudaStreamWaitEvent(s, e_in, 0))) break;
    if (k + 1 < n &&
        ((rc = copy_host(fb[(k + 1) & 1], f_host[k + 1], N, false, S->cs_in)) || !ok(cudaEventRecord(e_in, S->cs_in))))
      break;
    if ((rc = stage_g(S, g_host ? g_host[k] : nullptr))) break;
    // uk is free once u of problem k-2 has left it
    if (k >= 2 && !ok(cudaStreamWaitEvent(s, e_out[k & 1], 0))) break;
    if (S->o.initial_type == FISHGPU_INITIAL_GIVEN &&
        !ok(cudaMemcpyAsync(uk, u_host[k], bytes, cudaMemcpyHostToDevice, s)))
      break;
    S->prob.f = fk;
    src = fishgpu_solver_solve(S, uk, &reps[k]);
    S->prob.f = S->f_own;
    if (src != FISHGPU_OK && src != FISHGPU_ERR_NOT_CONVERGED) {
      rc = src;
      break;
    }
    if (!ok(cudaEventRecord(e_us, s)) || !ok(cudaStreamWaitEvent(S->cs_out, e_us, 0)) ||
        (rc = copy_host(u_host[k], uk, N, true, S->cs_out)) || !ok(cudaEventRecord(e_out[k & 1], S->cs_out)))
      break;
  }
  S->prob.f = S->f_own;
  if (S->cs_in && cudaStreamSynchronize(S->cs_in) != cudaSuccess && !rc) rc = FISHGPU_ERR_CUDA;
  if (S->cs_out && cudaStreamSynchronize(S->cs_out) != cudaSuccess && !rc) rc = FISHGPU_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = FISHGPU_ERR_CUDA;
  for (cudaEvent_t e : {e_in, e_z, e_us, e_out[0], e_out[1]})
    if (e) cudaEventDestroy(e);
  return rc ? rc : src;
}

extern "C" int fishgpu_solve_host(const fishgpu_opts *o, const double *f_host, const double *g_host,
                                  double *u_host, fishgpu_report *rep) {
  if (!o || !u_host || !rep) return FISHGPU_ERR_ARG;
  fishgpu_opts oo = *o;
  oo.ctx.f = nullptr;
  oo.ctx.g = nullptr;
  fishgpu_solver *S = nullptr;
  int rc = fishgpu_solver_create(&oo, nullptr, &S);
  if (rc) return rc;
  rc = fishgpu_solver_solve_host(S, f_host, g_host, u_host, rep);
  fishgpu_solver_destroy(S);
  return rc;
}

extern "C" int fishgpu_solver_time_kernel(fishgpu_solver *S, const char *name, int reps,
                                          double *ms_per_launch, double *bytes_per_launch) {
  if (!S || !name || reps < 1 || !ms_per_launch || !bytes_per_launch) return FISHGPU_ERR_ARG;
  switch (S->o.ctx.dim) {
  case 1: return time_kernel_dim<1>(S, name, reps, ms_per_launch, bytes_per_launch);
  case 2: return time_kernel_dim<2>(S, name, reps, ms_per_launch, bytes_per_launch);
  default: return time_kernel_dim<3>(S, name, reps, ms_per_launch, bytes_per_launch);
  }
}

// Eight independent FMA chains per thread; the multiplier and addend are
// kernel arguments, so nothing folds, and one store per thread keeps the work.
static __global__ void __launch_bounds__(256) k_dfma_rate(double *__restrict__ out, double m, double c, int iters) {
  double a[8];
#pragma unroll
  for (int q = 0; q < 8; q++) a[q] = threadIdx.x * 1e-3 + q;
  for (int t = 0; t < iters; t++) {
#pragma unroll
    for (int q = 0; q < 8; q++) a[q] = fma(a[q], m, c);
  }
  double sum = 0.0;
#pragma unroll
  for (int q = 0; q < 8; q++) sum += a[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

extern "C" int fishgpu_fp64_fma_rate(int reps, double *tflops) {
  if (reps < 1 || !tflops) return FISHGPU_ERR_ARG;
  int dev = 0, sms = 0;
  FG_CUDA(cudaGetDevice(&dev));
  FG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double *out = nullptr;
  if (cudaMalloc((void **)&out, sizeof(double) * blocks * threads) != cudaSuccess) return FISHGPU_ERR_NOMEM;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FISHGPU_OK;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    rc = FISHGPU_ERR_CUDA;
  float best = 0.f;
  for (int q = 0; q <= reps && rc == FISHGPU_OK; q++) {
    float ms = 0.f;
    k_dfma_rate<<<blocks, threads, 0, s>>>(out, 0.999999, 1e-6, iters);  // launch 0 warms up
    if (q == 0) continue;
    if (cudaEventRecord(e0, s) != cudaSuccess) rc = FISHGPU_ERR_CUDA;
    k_dfma_rate<<<blocks, threads, 0, s>>>(out, 0.999999, 1e-6, iters);
    if (rc == FISHGPU_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                             cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      rc = FISHGPU_ERR_CUDA;
    if (rc == FISHGPU_OK && (best == 0.f || ms < best)) best = ms;
  }
  if (rc == FISHGPU_OK && cudaGetLastError() != cudaSuccess) rc = FISHGPU_ERR_CUDA;
  if (rc == FISHGPU_OK) *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(out);
  return rc;
}

// ====================================================================== batches
// Thousands of independent 2D problems -Laplace(u) = f on the unit square with
// u = 0 on the boundary (fish's operator with cx = cy = 1), of uneven sizes
// n = 2^k + 1.  Instances of one size form a group: a 2D grid whose k-planes
// are the instances, solved by one set of launches per multigrid phase (every
// kernel works per plane: own CG state, own reductions, own refinement
// scale), with the mixed form (FP64 refinement around FP32 CG + V-cycle).
// Groups run concurrently, each on its own stream and host thread.
namespace fg {

// f of instance q (dense n x n) -> b = h^2 f on interior nodes, 0 on the boundary
__global__ void __launch_bounds__(256) k_pack_rhs(Geom g, const double *const *f, double *__restrict__ b) {
  const long long per = (long long)g.mx * g.my;
  const int q = blockIdx.y;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < per; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.mx), j = (int)(t / g.mx);
    const bool bd = i == 0 || j == 0 || i == g.mx - 1 || j == g.my - 1;
    b[(long long)q * g.plane + (long long)j * g.pitch + i] = bd ? 0.0 : g.vol * f[q][t];
  }
}

// u of instance q (dense) from plane q of y
__global__ void __launch_bounds__(256) k_unpack_planes(Geom g, const double *__restrict__ y, double *const *u) {
  const long long per = (long long)g.mx * g.my;
  const int q = blockIdx.y;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < per; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.mx), j = (int)(t / g.mx);
    u[q][t] = y[(long long)q * g.plane + (long long)j * g.pitch + i];
  }
}

// ---------------------------------------------------------------- autotuner
// Tiles: the block size (slots per block) and the strip of rows a stencil
// thread marches (ry: 0 = one slot per thread, or 4 .. 32 rows) of each level
// of a group, by timing one Chebyshev step with each candidate pair; cached
// per (n, planes).  Sweeps: the smoothing steps per level (V(1,1), V(2,2),
// V(3,3)) of a group, by timing whole batched solves of up to 32 instances of
// its size with each count (tune_sweeps); cached per n.
struct TileChoice {
  int chunk, ry;
};
static std::mutex g_tune_mu;
static std::map<std::pair<int, int>, TileChoice> g_tune_cache;
static std::map<std::pair<int, int>, int> g_sweep_cache;

static TileChoice tune_tiles(fishgpu_solver *S, Level<float> &lv) {
  const std::pair<int, int> key(lv.g.mx, lv.g.mz);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) return it->second;
  }
  static const int cand[3] = {64, 128, 256};
  static const int rows[5] = {0, 4, 8, 16, 32};
  TileChoice best{256, batch_rows(lv.g)};
  float best_ms = 1e30f;
  cudaStream_t s = S->stream;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 5; r++) {
      if (rows[r] > lv.g.my) continue;
      const Slots sl = make_slots(lv.g, ZC, 2432, cand[c], 1, rows[r]);
      const unsigned gb = slot_blocks(sl);
      // b = the level's residual buffer, x_{k-1}, x_k, out: its three iterate buffers
      for (int w = 0; w < 2; w++)
        v_cheb<2, float, true><<<gb, sl.chunk, 0, s>>>(lv.g, sl, nullptr, lv.r, lv.X[0], lv.X[1], lv.X[2], 0.5f,
                                                        0.5f, 0.1f);
      cudaEventRecord(S->ev0, s);
      for (int q = 0; q < 5; q++)
        v_cheb<2, float, true><<<gb, sl.chunk, 0, s>>>(lv.g, sl, nullptr, lv.r, lv.X[0], lv.X[1], lv.X[2], 0.5f,
                                                        0.5f, 0.1f);
      cudaEventRecord(S->ev1, s);
      if (cudaEventSynchronize(S->ev1) != cudaSuccess) return best;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, S->ev0, S->ev1);
      if (ms < best_ms) {
        best_ms = ms;
        best = TileChoice{cand[c], rows[r]};
      }
    }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return best;
}

}  // namespace fg

struct fishgpu_batch_s {
  fishgpu_batch_opts o;
  int ninst = 0;
  std::vector<int> n;                     // nodes per side, per instance
  std::vector<fishgpu_solver *> groups;   // one per distinct size
  std::vector<std::vector<int>> members;  // instances of each group, plane order
  std::vector<int> inner_its, outer_its;
  std::vector<double> rel_resid;
  std::vector<int> reason;
  cudaStream_t user_stream = nullptr;
};

namespace fg {

static int group_create(const fishgpu_batch_opts &bo, int n, int count, fishgpu_solver **out) {
  fishgpu_opts o;
  fishgpu_opts_default(&o);
  o.ctx.dim = 2;
  o.ctx.problem = FISHGPU_ZERO;
  o.mx = o.my = n;
  o.mz = 1;
  int levels = 1;
  for (int m = n; m > 3 && (m - 1) % 2 == 0; m = (m - 1) / 2 + 1) levels++;
  o.mg_levels = levels;
  o.pc_type = FISHGPU_PC_MG;
  o.precision = FISHGPU_MIXED;
  o.rtol = bo.rtol;
  o.atol = bo.atol;
  o.max_it = bo.inner_max_it;
  o.inner_max_it = bo.inner_max_it;
  o.outer_max_it = bo.outer_max_it;
  o.inner_rtol = bo.inner_rtol;
  o.smooth_its = bo.smooth_its;
  o.mg_cycles = bo.mg_cycles;
  for (int q = 0; q < 4; q++) o.esteig[q] = bo.esteig[q];
  o.graph_iters = 2;
  o.inner_accurate = bo.inner_accurate;
  o.norm_type = FISHGPU_NORM_UNPRECONDITIONED;
  fishgpu_solver *S = new fishgpu_solver();
  S->o = o;
  S->ksp_norm = FISHGPU_NORM_UNPRECONDITIONED;
  S->batch = 1;
  S->nplanes = count;
  int rc = FISHGPU_OK;
  if (cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete S;
    return FISHGPU_ERR_CUDA;
  }
  S->own_stream = true;
  S->dense = make_geom(2, n, n, 1, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0);
  S->fine = padded(S->dense);
  S->fine.mz = count;
  S->sf = make_slots(S->fine, 1, 0, 256, 1);
  S->Lf = launch_for(S->fine);
  S->prob = Prob{FISHGPU_ZERO, 2, 1.0, 1.0, 1.0, nullptr, nullptr, S->dense.pitch, S->dense.plane};
  S->giters = 2;
  const size_t N = nelem(S->fine);
#define CK(x)                         \
  do {                                \
    if ((rc = (x)) != FISHGPU_OK) {   \
      fishgpu_solver_destroy(S);      \
      return rc;                      \
    }                                 \
  } while (0)
  if (cudaMallocHost((void **)&S->st_h, sizeof(KspState) * count) != cudaSuccess ||
      cudaMallocHost((void **)&S->hval, sizeof(double) * 2 * count) != cudaSuccess ||
      cudaEventCreate(&S->ev0) != cudaSuccess || cudaEventCreate(&S->ev1) != cudaSuccess) {
    fishgpu_solver_destroy(S);
    return FISHGPU_ERR_CUDA;
  }
  CK(dalloc(S, &S->st, (size_t)count));
  CK(dalloc(S, &S->dval, 2 * (size_t)count));
  CK(dalloc(S, &S->ndone, 1));
  CK(dalloc(S, &S->scl, (size_t)count));
  CK(dalloc(S, &S->iscl, (size_t)count));
  CK(dalloc(S, &S->b64, N));
  CK(dalloc(S, &S->y64, N));
  CK(dalloc(S, &S->r64, N));
  CK(dalloc(S, &S->r32, N));
  CK(dalloc(S, &S->p32, N));
  CK(dalloc(S, &S->q32, N));
  CK(dalloc(S, &S->w32, N));
  CK(dalloc(S, &S->y32, N));
  CK(build_hier<float>(S, S->h32));
  // tune block sizes per level before anything is captured
  if (bo.tune) {
    if (cudaStreamSynchronize(S->stream) != cudaSuccess) {
      fishgpu_solver_destroy(S);
      return FISHGPU_ERR_CUDA;
    }
    for (int l = S->h32.nlev - 1; l >= 1; l--) {
      Level<float> &lv = S->h32.lev[l];
      const TileChoice c = tune_tiles(S, lv);
      lv.sl = make_slots(lv.g, ZC, 2432, c.chunk, 1);
      lv.st = make_slots(lv.g, ZC, 2432, c.chunk, 1, c.ry);
    }
    S->sf = S->h32.lev[S->h32.nlev - 1].sl;
  }
  S->sfst = S->h32.lev[S->h32.nlev - 1].st;
  // reductions are over the fine level's blocks, tickets per plane
  const int cap = (int)slot_blocks(S->sf);
  CK(dalloc(S, &S->red.partials, (size_t)2 * 2 * cap));
  CK(dalloc(S, &S->red.tickets, (size_t)2 * count));
  S->red.cap = cap;
  S->red.tcap = count;
#undef CK
  if (cudaStreamSynchronize(S->stream) != cudaSuccess) {
    fishgpu_solver_destroy(S);
    return FISHGPU_ERR_CUDA;
  }
  *out = S;
  return FISHGPU_OK;
}

// per-plane FP64 norms^2 of a into hval[0..count)
static int plane_norms(fishgpu_solver *S, const double *a) {
  v_dots<double><<<slot_blocks(S->sf), S->sf.chunk, 0, S->stream>>>(S->fine, S->sf, nullptr, a, a, S->red, 1,
                                                                    FIN_STORE, S->dval);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaMemcpyAsync(S->hval, S->dval, sizeof(double) * 2 * S->nplanes, cudaMemcpyDeviceToHost, S->stream));
  FG_CUDA(cudaStreamSynchronize(S->stream));
  return FISHGPU_OK;
}

// Batched refinement solve of one group; f, u: device arrays of `count`
// device pointers.  Results per plane into its/outer/relres/reason.
static int group_solve(fishgpu_solver *S, const double *const *f, double *const *u, int *its_out, int *outer_out,
                       double *relres_out, int *reason_out) {
  const fishgpu_opts &o = S->o;
  const int count = S->nplanes;
  cudaStream_t s = S->stream;
  const Geom &g = S->fine;
  const unsigned gb = slot_blocks(S->sf);
  S->launches = 0;
  {
    dim3 grid((unsigned)std::min<long long>(((long long)g.mx * g.my + 255) / 256, 64), (unsigned)count);
    k_pack_rhs<<<grid, 256, 0, s>>>(g, f, S->b64);
  }
  v_zero<double><<<gb, S->sf.chunk, 0, s>>>(g, S->sf, S->y64);
  int rc = plane_norms(S, S->b64);
  if (rc) return rc;
  std::vector<double> bn(count), rn(count), ttol(count);
  std::vector<int> active(count), its(count, 0), outer(count, 0), reason(count, 0);
  for (int q = 0; q < count; q++) {
    bn[q] = rn[q] = sqrt(S->hval[2 * q]);
    ttol[q] = fmax(o.rtol * bn[q], o.atol);
  }
  // the first step's FP32 floor, as in solve_dim (y64 is zero-filled above,
  // so the accurate form's updates always read it: yfresh = 0)
  double lmin, lmax;
  spectrum(g, &lmin, &lmax);
  const double kappa = lmax / fmax(lmin, 1e-300);
  const bool accurate = inner_accurate_for(o.inner_accurate, o.rtol, o.inner_rtol, kappa);
  const double first_floor = accurate ? fmin(0.5, o.first_floor_scale * kappa * (M_PI / (g.mx - 1)) * 0x1.0p-24)
                                      : fmin(0.5, 0.3 * kappa * 0x1.0p-24);
  std::vector<double> hs(count), his(count);
  KspVecs<float> v{S->r32, {S->p32, S->q32}, S->w32, S->y32, accurate ? S->y64 : nullptr};
  for (int step = 0;; step++) {
    int nact = 0;
    for (int q = 0; q < count; q++) {
      active[q] = 0;
      if (reason[q]) continue;
      if (isnan(rn[q]) || isinf(rn[q])) reason[q] = R_DIVERGED_NANORINF;
      else if (rn[q] <= ttol[q]) reason[q] = rn[q] < o.atol ? R_CONVERGED_ATOL : R_CONVERGED_RTOL;
      else if (step >= o.outer_max_it) reason[q] = R_DIVERGED_ITS;
      else active[q] = 1;
      nact += active[q];
    }
    if (!nact) break;
    // per-plane scales and fresh inner KSP states (inactive planes: done)
    unsigned int ninact = 0;
    for (int q = 0; q < count; q++) {
      KspState *h = &S->st_h[q];
      memset(h, 0, sizeof(*h));
      h->betaold = 1.0;
      h->atol = o.atol;
      h->dtol = o.dtol;
      h->max_it = o.inner_max_it;
      h->norm_type = FISHGPU_NORM_UNPRECONDITIONED;
      h->ndone = S->ndone;
      if (active[q]) {
        double irtol = fmax(o.inner_rtol, 0.5 * ttol[q] / rn[q]);
        if (step == 0) irtol = fmax(irtol, first_floor);
        h->rtol = fmin(irtol, 0.5);
        h->yscale = rn[q];
        hs[q] = rn[q];
        his[q] = 1.0 / rn[q];
      } else {
        h->done = 1;
        ninact++;
        hs[q] = 0.0;
        his[q] = 0.0;
      }
    }
    FG_CUDA(cudaMemcpyAsync(S->scl, hs.data(), sizeof(double) * count, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(S->iscl, his.data(), sizeof(double) * count, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(S->st, S->st_h, sizeof(KspState) * count, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(S->ndone, &ninact, sizeof(unsigned int), cudaMemcpyHostToDevice, s));
    v_demote<<<gb, S->sf.chunk, 0, s>>>(g, S->sf, step == 0 ? S->b64 : S->r64, S->iscl, 0.0, S->r32);
    if (!S->gexec_init &&
        (rc = capture(S, [&] { enq_cg_init<2, float>(S, S->h32, v); }, &S->gexec_init, &S->n_init)))
      return rc;
    const long long guard = (long long)o.inner_max_it / S->giters + 4;
    // the CG loop on the device until every plane has stopped (plane 0's state
    // counts the bodies); the host loop is kept for a driver that refuses it
    if (!S->gloop && !S->loop_refused && S->o.device_loop)
      S->loop_refused = !build_loop_graph(
          s, [&] { for (int q = 0; q < S->giters; q++) enq_cg_iter<2, float>(S, S->h32, v, q & 1); }, nullptr,
          S->ndone, (unsigned int)count, &S->st[0].loops, (unsigned int)(guard + 1), &S->gloop, &S->n_loop);
    if (!S->gloop && !S->gexec &&
        (rc = capture(S, [&] { for (int q = 0; q < S->giters; q++) enq_cg_iter<2, float>(S, S->h32, v, q & 1); },
                      &S->gexec, &S->n_iter)))
      return rc;
    FG_CUDA(cudaGraphLaunch(S->gexec_init, s));
    S->launches += S->n_init + 2;
    if (S->gloop) {
      FG_CUDA(cudaGraphLaunch(S->gloop, s));
    } else {
      unsigned int *hdone = (unsigned int *)S->hval;  // reuse pinned scratch for the counter
      for (long long l = 0;; l++) {
        FG_CUDA(cudaMemcpyAsync(hdone, S->ndone, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
        if (*hdone >= (unsigned)count) break;
        if (l > guard) return FISHGPU_ERR_TIMEOUT;
        FG_CUDA(cudaGraphLaunch(S->gexec, s));
        S->launches += S->n_iter;
      }
    }
    if (accurate) {  // the last deferred y64 += scale alpha p (the others went to y64 in the loop)
      v_pend_acc<<<gb, S->sf.chunk, 0, s>>>(g, S->sf, S->st, v.p[0], v.p[1], S->y64);
      FG_CUDA(cudaMemcpyAsync(S->st_h, S->st, sizeof(KspState) * count, cudaMemcpyDeviceToHost, s));
    } else {
      v_cg_pend<float><<<gb, S->sf.chunk, 0, s>>>(g, S->sf, S->st, v.p[0], v.p[1], v.y);
      FG_CUDA(cudaMemcpyAsync(S->st_h, S->st, sizeof(KspState) * count, cudaMemcpyDeviceToHost, s));
      v_promote_add<<<gb, S->sf.chunk, 0, s>>>(g, S->sf, S->y32, S->scl, 0.0, S->y64);
      S->launches += 1;
    }
    v_resid<2, double><<<gb, S->sf.chunk, 0, s>>>(g, S->sf, nullptr, S->b64, S->y64, S->r64);
    S->launches += 2;
    if ((rc = plane_norms(S, S->r64))) return rc;  // synchronises: st_h holds the planes' states
    if (S->gloop) {
      S->launches += (long long)S->st_h[0].loops * S->n_loop;
      for (int q = 0; q < count; q++)
        if (active[q] && !S->st_h[q].done) return FISHGPU_ERR_TIMEOUT;
    }
    for (int q = 0; q < count; q++) {
      if (!active[q]) continue;
      const KspState *h = &S->st_h[q];
      its[q] += h->its;
      outer[q]++;
      rn[q] = sqrt(S->hval[2 * q]);
      if (h->reason == R_DIVERGED_NANORINF || h->reason == R_DIVERGED_INDEFINITE_MAT ||
          h->reason == R_DIVERGED_INDEFINITE_PC)
        reason[q] = h->reason;
    }
  }
  {
    dim3 grid((unsigned)std::min<long long>(((long long)g.mx * g.my + 255) / 256, 64), (unsigned)count);
    k_unpack_planes<<<grid, 256, 0, s>>>(g, S->y64, u);
    S->launches += 1;
  }
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(s));
  for (int q = 0; q < count; q++) {
    its_out[q] = its[q];
    outer_out[q] = outer[q];
    relres_out[q] = bn[q] > 0 ? rn[q] / bn[q] : 0.0;
    reason_out[q] = reason[q];
  }
  return FISHGPU_OK;
}

}  // namespace fg

namespace fg {

// a deterministic right-hand side for the sweep tuner: uniform in [-1, 1)
static __global__ void k_fill_rhs(double *__restrict__ f, long long n, unsigned long long seed) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    unsigned long long x = (seed ^ (unsigned long long)t) + 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x ^= x >> 31;
    f[t] = (double)(x >> 11) * 0x1.0p-52 - 1.0;
  }
}

// Smoothing steps per level for a group of n x n instances: the count among
// 1, 2, 3 whose batched solve of min(count, 32) instances (a fixed random
// right-hand side, the batch's tolerances) takes least time, every instance
// converged; the batch's own count when no candidate does better.
static int tune_sweeps(const fishgpu_batch_opts &bo, int n, int count) {
  const int q = std::min(count, 32);
  const std::pair<int, int> key(n, q);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_sweep_cache.find(key);
    if (it != g_sweep_cache.end()) return it->second;
  }
  const long long per = (long long)n * n;
  double *f = nullptr, *u = nullptr;
  double **fp = nullptr, **up = nullptr;
  int best = bo.smooth_its;
  if (cudaMalloc((void **)&f, sizeof(double) * per * q) != cudaSuccess ||
      cudaMalloc((void **)&u, sizeof(double) * per * q) != cudaSuccess ||
      cudaMalloc((void **)&fp, sizeof(double *) * q) != cudaSuccess ||
      cudaMalloc((void **)&up, sizeof(double *) * q) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(f); cudaFree(u); cudaFree(fp); cudaFree(up);
    return best;
  }
  std::vector<double *> hf(q), hu(q);
  for (int p = 0; p < q; p++) {
    hf[p] = f + per * p;
    hu[p] = u + per * p;
  }
  cudaMemcpy(fp, hf.data(), sizeof(double *) * q, cudaMemcpyHostToDevice);
  cudaMemcpy(up, hu.data(), sizeof(double *) * q, cudaMemcpyHostToDevice);
  k_fill_rhs<<<256, 256>>>(f, per * q, 12345ULL);
  cudaDeviceSynchronize();
  std::vector<int> its(q), outer(q), reason(q);
  std::vector<double> rel(q);
  double best_s = 1e30;
  for (int sw = 1; sw <= 3; sw++) {
    fishgpu_batch_opts b2 = bo;
    b2.smooth_its = sw;
    b2.tune_sweeps = 0;
    fishgpu_solver *S = nullptr;
    if (group_create(b2, n, q, &S) != FISHGPU_OK) continue;
    double dt = 1e30;
    bool ok = true;
    for (int rep = 0; rep < 2 && ok; rep++) {  // the first builds the graphs
      const auto t0 = std::chrono::steady_clock::now();
      ok = group_solve(S, fp, up, its.data(), outer.data(), rel.data(), reason.data()) == FISHGPU_OK;
      dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      for (int p = 0; p < q && ok; p++) ok = reason[p] > 0;
    }
    fishgpu_solver_destroy(S);
    if (ok && dt < best_s) {
      best_s = dt;
      best = sw;
    }
  }
  cudaFree(f); cudaFree(u); cudaFree(fp); cudaFree(up);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_sweep_cache[key] = best;
  return best;
}

}  // namespace fg

extern "C" int fishgpu_batch_opts_default(fishgpu_batch_opts *o) {
  if (!o) return FISHGPU_ERR_ARG;
  memset(o, 0, sizeof(*o));
  o->rtol = 1e-8;
  o->atol = 1e-50;
  o->inner_rtol = 1e-6;
  o->inner_max_it = 100;
  o->outer_max_it = 30;
  o->smooth_its = 2;
  o->mg_cycles = 1;
  o->esteig[0] = 0.0;
  o->esteig[1] = 0.1;
  o->esteig[2] = 0.0;
  o->esteig[3] = 1.1;
  o->tune = 1;
  o->inner_accurate = -1;
  o->tune_sweeps = 1;
  return FISHGPU_OK;
}

extern "C" int fishgpu_batch_destroy(fishgpu_batch *B) {
  if (!B) return FISHGPU_OK;
  for (fishgpu_solver *S : B->groups) fishgpu_solver_destroy(S);
  delete B;
  return FISHGPU_OK;
}

extern "C" int fishgpu_batch_create(const fishgpu_batch_opts *o, int ninst, const int *n, fishgpu_batch **out) {
  if (!o || ninst < 1 || !n || !out) return FISHGPU_ERR_ARG;
  *out = nullptr;
  if (!(o->rtol >= 0) || o->inner_max_it < 1 || o->smooth_its < 1 || o->mg_cycles < 1 || o->mg_cycles > 2 ||
      o->inner_accurate < -1 || o->inner_accurate > 1)
    return FISHGPU_ERR_ARG;
  std::map<int, std::vector<int>> bysize;
  for (int q = 0; q < ninst; q++) {
    const int m = n[q];
    // 2^k + 1 nodes, k >= 1: coarsens down to 3 x 3
    if (m < 3 || m > (1 << 15) + 1 || ((m - 1) & (m - 2)) != 0) return FISHGPU_ERR_ARG;
    bysize[m].push_back(q);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FISHGPU_ERR_NODEVICE;
  }
  fishgpu_batch *B = new fishgpu_batch();
  B->o = *o;
  B->ninst = ninst;
  B->n.assign(n, n + ninst);
  for (auto it = bysize.rbegin(); it != bysize.rend(); ++it) {  // largest first
    fishgpu_solver *S = nullptr;
    fishgpu_batch_opts go = *o;
    if (o->tune && o->tune_sweeps) go.smooth_its = tune_sweeps(*o, it->first, (int)it->second.size());
    int rc = group_create(go, it->first, (int)it->second.size(), &S);
    if (rc) {
      fishgpu_batch_destroy(B);
      return rc;
    }
    B->groups.push_back(S);
    B->members.push_back(it->second);
  }
  B->inner_its.assign(ninst, 0);
  B->outer_its.assign(ninst, 0);
  B->rel_resid.assign(ninst, 0.0);
  B->reason.assign(ninst, 0);
  *out = B;
  return FISHGPU_OK;
}

extern "C" int fishgpu_batch_solve(fishgpu_batch *B, const double *const *f, double *const *u,
                                   fishgpu_batch_report *rep) {
  if (!B || !f || !u || !rep) return FISHGPU_ERR_ARG;
  memset(rep, 0, sizeof(*rep));
  const int G = (int)B->groups.size();
  // per group: device arrays of the members' f and u pointers
  std::vector<const double **> fdev(G, nullptr);
  std::vector<double **> udev(G, nullptr);
  std::vector<int> grc(G, FISHGPU_OK);
  std::vector<std::vector<int>> its(G), outer(G), reason(G);
  std::vector<std::vector<double>> rel(G);
  cudaEvent_t e0, e1;
  cudaStream_t s0;
  if (cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking) != cudaSuccess) return FISHGPU_ERR_CUDA;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = FISHGPU_OK;
  for (int gi = 0; gi < G && !rc; gi++) {
    const std::vector<int> &mem = B->members[gi];
    std::vector<const double *> hf(mem.size());
    std::vector<double *> hu(mem.size());
    for (size_t q = 0; q < mem.size(); q++) {
      hf[q] = f[mem[q]];
      hu[q] = u[mem[q]];
      if (!hf[q] || !hu[q]) rc = FISHGPU_ERR_ARG;
    }
    if (rc) break;
    if (cudaMalloc((void **)&fdev[gi], sizeof(double *) * mem.size()) != cudaSuccess ||
        cudaMalloc((void **)&udev[gi], sizeof(double *) * mem.size()) != cudaSuccess) {
      rc = FISHGPU_ERR_NOMEM;
      break;
    }
    cudaMemcpy(fdev[gi], hf.data(), sizeof(double *) * mem.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(udev[gi], hu.data(), sizeof(double *) * mem.size(), cudaMemcpyHostToDevice);
    its[gi].resize(mem.size());
    outer[gi].resize(mem.size());
    reason[gi].resize(mem.size());
    rel[gi].resize(mem.size());
  }
  if (!rc) {
    cudaDeviceSynchronize();
    cudaEventRecord(e0, s0);
    std::vector<std::thread> th;
    int dev = 0;
    cudaGetDevice(&dev);
    for (int gi = 0; gi < G; gi++)
      th.emplace_back([&, gi, dev] {
        cudaSetDevice(dev);
        grc[gi] = group_solve(B->groups[gi], fdev[gi], udev[gi], its[gi].data(), outer[gi].data(), rel[gi].data(),
                              reason[gi].data());
      });
    for (auto &t : th) t.join();
    cudaDeviceSynchronize();
    cudaEventRecord(e1, s0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    rep->solve_ms = ms;
    for (int gi = 0; gi < G; gi++)
      if (grc[gi] && !rc) rc = grc[gi];
  }
  for (int gi = 0; gi < G; gi++) {
    if (fdev[gi]) cudaFree(fdev[gi]);
    if (udev[gi]) cudaFree(udev[gi]);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s0);
  if (rc) return rc;
  rep->ninst = B->ninst;
  rep->groups = G;
  for (int gi = 0; gi < G; gi++) {
    const std::vector<int> &mem = B->members[gi];
    rep->launches += B->groups[gi]->launches;
    for (size_t q = 0; q < mem.size(); q++) {
      const int id = mem[q];
      B->inner_its[id] = its[gi][q];
      B->outer_its[id] = outer[gi][q];
      B->rel_resid[id] = rel[gi][q];
      B->reason[id] = reason[gi][q];
      rep->total_inner_its += its[gi][q];
      if (reason[gi][q] > 0) rep->converged++;
      if (outer[gi][q] > rep->max_outer) rep->max_outer = outer[gi][q];
      if (its[gi][q] > rep->max_inner) rep->max_inner = its[gi][q];
      rep->dofs += (long long)B->n[id] * B->n[id];
    }
  }
  return rep->converged == B->ninst ? FISHGPU_OK : FISHGPU_ERR_NOT_CONVERGED;
}

extern "C" int fishgpu_batch_groups(const fishgpu_batch *B, int *n, int *count, int *sweeps) {
  if (!B) return FISHGPU_ERR_ARG;
  for (size_t g = 0; g < B->groups.size(); g++) {
    const fishgpu_solver *S = B->groups[g];
    if (n) n[g] = S->fine.mx;
    if (count) count[g] = S->nplanes;
    if (sweeps) sweeps[g] = S->o.smooth_its;
  }
  return (int)B->groups.size();
}

extern "C" int fishgpu_batch_results(const fishgpu_batch *B, int *inner_its, int *outer_its, double *rel_resid,
                                     int *reason) {
  if (!B) return FISHGPU_ERR_ARG;
  for (int q = 0; q < B->ninst; q++) {
    if (inner_its) inner_its[q] = B->inner_its[q];
    if (outer_its) outer_its[q] = B->outer_its[q];
    if (rel_resid) rel_resid[q] = B->rel_resid[q];
    if (reason) reason[q] = B->reason[q];
  }
  return FISHGPU_OK;
}

// ------------------------------------------------------------------ same-size groups
struct fishgpu_group_s {
  fishgpu_solver *S = nullptr;
  int n = 0, count = 0;
  double *fbuf = nullptr, *ubuf = nullptr;  // count dense n x n arrays each
  const double **fptr = nullptr;            // device: fbuf + q n^2
  double **uptr = nullptr;
  long long bytes = 0;
};

extern "C" int fishgpu_group_destroy(fishgpu_group *G) {
  if (!G) return FISHGPU_OK;
  if (G->S) fishgpu_solver_destroy(G->S);
  cudaFree(G->fbuf);
  cudaFree(G->ubuf);
  cudaFree(G->fptr);
  cudaFree(G->uptr);
  delete G;
  return FISHGPU_OK;
}

extern "C" int fishgpu_group_create(const fishgpu_batch_opts *o, int n, int count, fishgpu_group **out) {
  if (!o || !out || n < 3 || ((n - 1) & (n - 2)) != 0 || count < 1 || count > 65535) return FISHGPU_ERR_ARG;
  *out = nullptr;
  fishgpu_group *G = new fishgpu_group();
  G->n = n;
  G->count = count;
  int rc = fg::group_create(*o, n, count, &G->S);
  const size_t nn = (size_t)n * n;
  if (!rc) {
    if (cudaMalloc((void **)&G->fbuf, sizeof(double) * nn * count) != cudaSuccess ||
        cudaMalloc((void **)&G->ubuf, sizeof(double) * nn * count) != cudaSuccess ||
        cudaMalloc((void **)&G->fptr, sizeof(double *) * count) != cudaSuccess ||
        cudaMalloc((void **)&G->uptr, sizeof(double *) * count) != cudaSuccess) {
      cudaGetLastError();
      rc = FISHGPU_ERR_NOMEM;
    }
  }
  if (!rc) {
    std::vector<const double *> hf(count);
    std::vector<double *> hu(count);
    for (int q = 0; q < count; q++) {
      hf[q] = G->fbuf + nn * q;
      hu[q] = G->ubuf + nn * q;
    }
    if (cudaMemcpy(G->fptr, hf.data(), sizeof(double *) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(G->uptr, hu.data(), sizeof(double *) * count, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = FISHGPU_ERR_CUDA;
  }
  if (rc) {
    fishgpu_group_destroy(G);
    return rc;
  }
  G->bytes = G->S->bytes + (long long)(2 * nn * count * sizeof(double) + 2 * count * sizeof(double *));
  *out = G;
  return FISHGPU_OK;
}

extern "C" long long fishgpu_group_bytes(const fishgpu_group *G) { return G ? G->bytes : 0; }

extern "C" int fishgpu_group_solve_host(fishgpu_group *G, int k, const double *const *f_host, double *const *u_host,
                                        int *its, int *outer_its, double *rel_resid) {
  if (!G || k < 1 || k > G->count || !f_host || !u_host) return FISHGPU_ERR_ARG;
  for (int q = 0; q < k; q++)
    if (!f_host[q] || !u_host[q]) return FISHGPU_ERR_ARG;
  fishgpu_solver *S = G->S;
  cudaStream_t s = S->stream;
  const size_t nn = (size_t)G->n * G->n;
  for (int q = 0; q < k; q++)
    FG_CUDA(cudaMemcpyAsync(G->fbuf + nn * q, f_host[q], sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  if (k < G->count) FG_CUDA(cudaMemsetAsync(G->fbuf + nn * k, 0, sizeof(double) * nn * (G->count - k), s));
  std::vector<int> vi(G->count), vo(G->count), vr(G->count);
  std::vector<double> vrel(G->count);
  int rc = fg::group_solve(S, G->fptr, G->uptr, vi.data(), vo.data(), vrel.data(), vr.data());
  if (rc) return rc;
  for (int q = 0; q < k; q++)
    FG_CUDA(cudaMemcpyAsync(u_host[q], G->ubuf + nn * q, sizeof(double) * nn, cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  for (int q = 0; q < k; q++) {
    if (its) its[q] = vi[q];
    if (outer_its) outer_its[q] = vo[q];
    if (rel_resid) rel_resid[q] = vrel[q];
  }
  return FISHGPU_OK;
}

// The grid barrier's time limit, exercised: one barrier over the persistent
// solve's blocks with block 0 absent (missing = 1) must end with the fault
// word set (FISHGPU_ERR_TIMEOUT, after ~0.2 s), with every block present
// (missing = 0) without it.  The fault word and the barrier are cleared
// afterwards.
extern "C" int fishgpu_solver_barrier_selftest(fishgpu_solver *S, int missing) {
  if (!S) return FISHGPU_ERR_ARG;
  if (!S->pbar || S->pblocks < 1 || (missing && S->pblocks < 2)) return FISHGPU_ERR_UNSUPPORTED;
  cudaStream_t s = S->stream;
  int nb = 1, absent = missing ? 0 : -1;
  void *args[] = {&S->pbar, &S->fault, &nb, &absent};
  FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
  FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
  FG_CUDA(cudaLaunchCooperativeKernel((const void *)fg::k_grid_sync_probe, dim3(S->pblocks), dim3(512), args, 0, s));
  FG_CUDA(cudaMemcpyAsync(S->hval + 7, S->fault, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  int fault = 0;
  memcpy(&fault, S->hval + 7, sizeof(int));
  FG_CUDA(cudaMemsetAsync(S->fault, 0, sizeof(int), s));
  FG_CUDA(cudaMemsetAsync(S->pbar, 0, 2 * sizeof(unsigned), s));
  FG_CUDA(cudaStreamSynchronize(s));
  return fault ? FISHGPU_ERR_TIMEOUT : FISHGPU_OK;
}
