// vblock.cuh -- the V-cycle and the CG iteration written point by point for
// block-level execution, where a level is too small for a launch per phase:
//
//   * vtail_body: the coarse end of a V-cycle in ONE block (k_vtail, and
//     block 0 of the persistent solve);
//   * k_ksp_persist: a whole CG + multigrid solve of a small grid in ONE
//     cooperative launch, every phase (CG update and apply, residual update,
//     each level's smoothing steps, residual, restriction, prolongation)
//     separated by a grid-wide barrier, the dot products reduced by every
//     block from the same partial sums (so that every block runs the KSP
//     scalar recurrences on identical values, without a second barrier).
//
// Every point is computed with the operations of the vectorised kernels in
// the same order (resid_at restates resid_el, apply_diff_at apply_diff_el,
// and so on), so the V-cycle tail is bit-identical to the launch-per-phase
// form; the persistent solve differs from it only in the order in which the
// dot products are summed (its blocks partition the points differently).
#pragma once

#include "kernels.cuh"
#include "tma.cuh"
#include "vkernels.cuh"

namespace fg {

// One level of a block-level V-cycle: the level's arrays and the Chebyshev
// coefficients of its smoothing steps (the same values enq_smooth passes to
// v_cheb2_zero and v_cheb).  Every level ends its V-cycle with its iterate
// in X[0] (pre-smoothing writes X[1], the two post-smoothing steps X[2] and
// X[0]), as the rotation of enq_smooth leaves it.
template <typename T>
struct TailLevel {
  Geom g;
  T *b, *r, *X[3];
  T a0, a1;            // two steps from zero: x = a0 b - a1 (A b)
  T c1;                // post-smoothing step 1: x1 = x0 + c1 (b - A x0)
  T ckm1, ck, crd;     // step 2: x2 = ckm1 x0 + ck x1 + crd (b - A x1)
};

// ------------------------------------------------------------------ point functions
// Values of an array, or of an array formed on the fly (the CG direction).
template <typename T>
struct PtArr {
  const T *x;
  __device__ __forceinline__ T operator()(long long n) const { return x[n]; }
};

// b - A x at one point (resid_el's operations on one point)
template <int DIM, typename T, class X>
__device__ __forceinline__ T resid_at(const Geom &g, const Wv<T> &w, const X &x, long long n, int i, int j, int k,
                                      T bv) {
  const T xc = x(n);
  const bool bd = jk_bdry(g, DIM, j, k) || i == 0 || i == g.mx - 1;
  if (bd) return fma(-w.sd, xc, bv);
  const T a = (i - 1 > 0 ? x(n - 1) : T(0)) + (i + 1 < g.mx - 1 ? x(n + 1) : T(0));
  T s = fma(w.sx, a, bv);
  if (DIM >= 2) s = fma(w.sy, (j - 1 > 0 ? x(n - g.pitch) : T(0)) + (j + 1 < g.my - 1 ? x(n + g.pitch) : T(0)), s);
  if (DIM >= 3) s = fma(w.sz, (k - 1 > 0 ? x(n - g.plane) : T(0)) + (k + 1 < g.mz - 1 ? x(n + g.plane) : T(0)), s);
  return fma(-w.sd, xc, s);
}

template <int DIM, typename T>
__device__ __forceinline__ T resid_pt(const Geom &g, const Wv<T> &w, const T *x, long long n, int i, int j, int k,
                                      T bv) {
  return resid_at<DIM, T>(g, w, PtArr<T>{x}, n, i, j, k, bv);
}

// A x at one point in difference form (apply_diff_el's operations)
template <int DIM, typename T, class X>
__device__ __forceinline__ T apply_diff_at(const Geom &g, const Wv<T> &w, const X &x, long long n, int i, int j,
                                           int k) {
  const T xc = x(n);
  if (jk_bdry(g, DIM, j, k) || i == 0 || i == g.mx - 1) return w.sd * xc;
  const T a = (xc - (i - 1 > 0 ? x(n - 1) : T(0))) + (xc - (i + 1 < g.mx - 1 ? x(n + 1) : T(0)));
  T s = w.sx * a;
  if (DIM >= 2)
    s = fma(w.sy, (xc - (j - 1 > 0 ? x(n - g.pitch) : T(0))) + (xc - (j + 1 < g.my - 1 ? x(n + g.pitch) : T(0))), s);
  if (DIM >= 3)
    s = fma(w.sz, (xc - (k - 1 > 0 ? x(n - g.plane) : T(0))) + (xc - (k + 1 < g.mz - 1 ? x(n + g.plane) : T(0))), s);
  return s;
}

// x-interpolated coarse value at fine x-index fi of coarse row (jc, kc) (v_prolong's lo/hi)
template <typename T>
__device__ __forceinline__ T prolong_x(const Geom &gc, const T *xc, int fi, int jc, int kc) {
  const long long m = (long long)kc * gc.plane + (long long)jc * gc.pitch;
  const int I = fi >> 1;
  if ((fi & 1) == 0) return xc[m + I];
  return T(0.5) * (xc[m + I] + (I + 1 < gc.mx ? xc[m + I + 1] : T(0)));
}

// x_f + (P x_c) at fine point (i, j, k) (v_prolong); k is the instance plane in 2D
template <int DIM, typename T>
__device__ __forceinline__ T prolong_add(const Geom &gc, const T *xc, int i, int j, int k, T xf) {
  const T h = T(0.5);
  const int J = j >> 1, K = DIM >= 3 ? k >> 1 : k;
  const T a0 = prolong_x<T>(gc, xc, i, J, K);
  T v;
  T wgt = T(1);
  if (DIM >= 3 && (k & 1)) {
    const T b0 = prolong_x<T>(gc, xc, i, J, K + 1);
    if (j & 1) {
      const T a1 = prolong_x<T>(gc, xc, i, J + 1, K), b1 = prolong_x<T>(gc, xc, i, J + 1, K + 1);
      v = (a0 + a1) + (b0 + b1);
      wgt = T(0.25);
    } else {
      v = a0 + b0;
      wgt = h;
    }
  } else if (DIM >= 2 && (j & 1)) {
    v = a0 + prolong_x<T>(gc, xc, i, J + 1, K);
    wgt = h;
  } else {
    v = a0;
  }
  return fma(wgt, v, xf);
}

// restricted row value at coarse x-index I of fine row (fj, fk) (restrict_row)
template <typename T>
__device__ __forceinline__ T restrict_x(const Geom &gf, const T *rf, int I, int fj, int fk) {
  const long long m = (long long)fk * gf.plane + (long long)fj * gf.pitch;
  const int fi = 2 * I;
  const T L = fi > 0 ? rf[m + fi - 1] : T(0);
  const T R = fi + 1 < gf.pitch ? rf[m + fi + 1] : T(0);
  return fma(T(0.5), L + R, rf[m + fi]);
}

// (P^T r_f) at coarse point (I, J, K) (v_restrict); K is the instance plane in 2D
template <int DIM, typename T>
__device__ __forceinline__ T restrict_pt(const Geom &g, const T *rf, int I, int J, int K) {
  const T h = T(0.5);
  auto rowsum = [&](int fk) -> T {
    const int fj = 2 * J;
    const T c = restrict_x<T>(g, rf, I, fj, fk);
    if (DIM < 2) return c;
    const T sr = fj - 1 >= 0 ? restrict_x<T>(g, rf, I, fj - 1, fk) : T(0);
    const T nr = fj + 1 < g.my ? restrict_x<T>(g, rf, I, fj + 1, fk) : T(0);
    return fma(h, sr + nr, c);
  };
  if (DIM >= 3) {
    const T below = K > 0 ? rowsum(2 * K - 1) : T(0);
    const T mid = rowsum(2 * K);
    const T above = 2 * K + 1 < g.mz ? rowsum(2 * K + 1) : T(0);
    return fma(h, below + above, mid);
  }
  return rowsum(K);
}

// points of a level (one plane of a 2D batch) and the (i, j, k) / offset of
// point q; k is the instance plane in 2D
template <int DIM>
__device__ __forceinline__ int level_npts(const Geom &g) {
  return g.mx * g.my * (DIM < 3 ? 1 : g.mz);
}
template <int DIM>
__device__ __forceinline__ long long level_pos(const Geom &g, int q, int plane, int &i, int &j, int &k) {
  i = q % g.mx;
  const int r = q / g.mx;
  j = DIM >= 2 ? r % g.my : 0;
  k = DIM >= 3 ? r / g.my : plane;
  return (long long)k * g.plane + (long long)j * g.pitch + i;
}

// level_pos without integer division, for q < 2^24 (exact in FP32): q * (1/m)
// rounded twice is within one of q / m, and one comparison each way corrects
// it.  rx = 1/mx, ry = 1/my in FP32.
__device__ __forceinline__ int div_small(int q, int m, float rm) {
  int r = __float2int_rz(__int2float_rn(q) * rm);
  if (r * m > q) r--;
  else if ((r + 1) * m <= q) r++;
  return r;
}
struct LevelDiv {
  float rx, ry;
  __device__ __forceinline__ explicit LevelDiv(const Geom &g) : rx(1.0f / g.mx), ry(1.0f / g.my) {}
};
template <int DIM>
__device__ __forceinline__ long long level_pos_f(const Geom &g, const LevelDiv &d, int q, int plane, int &i, int &j,
                                                 int &k) {
  const int r = DIM >= 2 ? div_small(q, g.mx, d.rx) : 0;
  i = q - r * g.mx;
  if (DIM >= 3) {
    k = div_small(r, g.my, d.ry);
    j = r - k * g.my;
  } else {
    j = r;
    k = plane;
  }
  return (long long)k * g.plane + (long long)j * g.pitch + i;
}

// ------------------------------------------------------------------ the one-block tail
// Levels top .. 1 pre-smooth, take their residual and restrict it, level 0
// is solved exactly, and on the way up every level adds the prolongated
// correction and post-smooths: the work of ~7 launches per level as phases
// of one block separated by block barriers.  `plane`: the instance of a 2D
// batch (0 otherwise).  Tail levels have far fewer than 2^24 nodes
// (level_pos_f).
template <int DIM, typename T>
__device__ void vtail_body(const TailLevel<T> *tl, int top, int plane, const T *S0, const T *S1, const T *S2,
                           const T *ilam, T *work, int n0, int n1, int n2, int smem, T dinv, unsigned char *sm_raw) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int l = top; l >= 1; l--) {
    const TailLevel<T> &L = tl[l];
    const TailLevel<T> &C = tl[l - 1];
    const Geom &g = L.g;
    const Wv<T> w(g);
    const LevelDiv dv(g), dvc(C.g);
    const int N = level_npts<DIM>(g);
    for (int q = tid; q < N; q += nt) {  // two Chebyshev steps from zero (v_cheb2_zero): X[1]
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, q, plane, i, j, k);
      const T mab = resid_pt<DIM, T>(g, w, L.b, n, i, j, k, T(0));
      L.X[1][n] = fma(L.a1, mab, L.a0 * L.b[n]);
    }
    __syncthreads();
    for (int q = tid; q < N; q += nt) {  // r = b - A x (v_resid)
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, q, plane, i, j, k);
      L.r[n] = resid_pt<DIM, T>(g, w, L.X[1], n, i, j, k, L.b[n]);
    }
    __syncthreads();
    const Geom &gc = C.g;
    const int Nc = level_npts<DIM>(gc);
    for (int q = tid; q < Nc; q += nt) {  // b_c = P^T r (v_restrict)
      int I, J, K;
      const long long m = level_pos_f<DIM>(gc, dvc, q, plane, I, J, K);
      C.b[m] = restrict_pt<DIM, T>(g, L.r, I, J, K);
    }
    __syncthreads();
  }
  {  // exact solve on level 0 into X[0]
    const TailLevel<T> &C = tl[0];
    const long long off = DIM < 3 ? (long long)plane * C.g.plane : 0;
    coarse_solve_block<DIM, T>(C.g, C.b + off, C.X[0] + off, S0, S1, S2, ilam, work, n0, n1, n2, smem, dinv, sm_raw);
    __syncthreads();
  }
  for (int l = 1; l <= top; l++) {
    const TailLevel<T> &L = tl[l];
    const TailLevel<T> &C = tl[l - 1];
    const Geom &g = L.g, &gc = C.g;
    const Wv<T> w(g);
    const LevelDiv dv(g);
    const int N = level_npts<DIM>(g);
    for (int q = tid; q < N; q += nt) {  // x += P x_c (v_prolong), x in X[1]
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, q, plane, i, j, k);
      L.X[1][n] = prolong_add<DIM, T>(gc, C.X[0], i, j, k, L.X[1][n]);
    }
    __syncthreads();
    for (int q = tid; q < N; q += nt) {  // x1 = x0 + c1 (b - A x0) (v_cheb without x_{k-1}): X[2]
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, q, plane, i, j, k);
      const T r = resid_pt<DIM, T>(g, w, L.X[1], n, i, j, k, L.b[n]);
      L.X[2][n] = fma(L.c1, r, T(1) * L.X[1][n]);
    }
    __syncthreads();
    for (int q = tid; q < N; q += nt) {  // x2 = ckm1 x0 + ck x1 + crd (b - A x1) (v_cheb): X[0]
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, q, plane, i, j, k);
      const T r = resid_pt<DIM, T>(g, w, L.X[2], n, i, j, k, L.b[n]);
      L.X[0][n] = fma(L.crd, r, fma(L.ckm1, L.X[1][n], L.ck * L.X[2][n]));
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ the tail in shared memory
// The tail levels' arrays copied into shared memory, compact (pitch mx): a
// tail phase then waits on shared memory instead of an L2 round trip (~25
// phases per V-cycle).  Level 0 keeps b and X[0], the others b, r, X[0..2].
// Only the top level's b comes in and its X[0] goes out: every other tail
// array is written before it is read within the tail, and nothing outside
// the tail reads them.  The compact layout gives the same values: the
// padded layout's extra points are zero and enter no sum (restrict_x reads
// one as 0, where the compact row ends).
__host__ __device__ inline Geom compact_geom(Geom g) {
  g.pitch = g.mx;
  g.plane = (long long)g.mx * g.my;
  return g;
}

// elements of the copy of level l with `pts` nodes per grid
__host__ __device__ inline long long tail_copy_elems(int l, long long pts) { return (l == 0 ? 2 : 5) * pts; }

// The table of the shared-memory copy (sv): level l's entry built by thread
// l (a level's offset is the sum of the sizes below it).  Needs a block
// barrier before use.
template <int DIM, typename T>
__device__ void vtail_prepare(const TailLevel<T> *tl, int top, unsigned char *sm_raw, int copy_off, TailLevel<T> *sv) {
  const int l = threadIdx.x;
  if (l > top) return;
  long long off = 0;
  for (int q = 0; q < l; q++) off += tail_copy_elems(q, level_npts<DIM>(compact_geom(tl[q].g)));
  T *p = reinterpret_cast<T *>(sm_raw + copy_off) + off;
  TailLevel<T> t = tl[l];
  t.g = compact_geom(t.g);
  const long long n = level_npts<DIM>(t.g);
  t.b = p;
  t.X[0] = p + n;
  if (l > 0) {
    t.r = p + 2 * n;
    t.X[1] = p + 3 * n;
    t.X[2] = p + 4 * n;
  }
  sv[l] = t;
}

// The tail from a prepared shared-memory table sv (copy_off >= 0), or in
// global memory (copy_off < 0): the top level's b in, vtail_body, its X[0]
// out.  `smem` as coarse_solve_block takes it.
template <int DIM, typename T>
__device__ void vtail_run(const TailLevel<T> *tl, int top, int plane, const T *S0, const T *S1, const T *S2,
                          const T *ilam, T *work, int n0, int n1, int n2, int smem, T dinv, unsigned char *sm_raw,
                          int copy_off, const TailLevel<T> *sv) {
  if (copy_off < 0) {  // the arrays stay in global memory
    vtail_body<DIM, T>(tl, top, plane, S0, S1, S2, ilam, work, n0, n1, n2, smem, dinv, sm_raw);
    return;
  }
  const int tid = threadIdx.x, nt = blockDim.x;
  const TailLevel<T> &G = tl[top];
  const TailLevel<T> &C = sv[top];
  const int N = level_npts<DIM>(G.g);
  const LevelDiv dv(G.g);
  for (int q = tid; q < N; q += nt) {
    int i, j, k;
    C.b[q] = G.b[level_pos_f<DIM>(G.g, dv, q, plane, i, j, k)];
  }
  __syncthreads();
  vtail_body<DIM, T>(sv, top, 0, S0, S1, S2, ilam, work, n0, n1, n2, smem, dinv, sm_raw);
  for (int q = tid; q < N; q += nt) {
    int i, j, k;
    G.X[0][level_pos_f<DIM>(G.g, dv, q, plane, i, j, k)] = C.X[0][q];
  }
  __syncthreads();
}

// ------------------------------------------------------------------ grid barrier
// A barrier over all blocks of a cooperative launch (every block resident)
// on one monotonic counter: barrier e (1, 2, ...) of the launch is passed
// when the counter reaches e * gridDim.x.  Thread 0 of a block arrives with
// a release reduction (after the block barrier: the block's writes are
// released with it) and waits with acquire loads (the other blocks' writes
// are visible after the closing block barrier) -- one round trip to L2 on
// the critical path.  The wait is bounded in time (kWaitNs): a block that
// gives up records the failure in *fault and returns false, and every later
// barrier of every block gives up at once (the launch's results are void;
// it ends instead of spinning).  *bar must be zero at the launch.
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

struct GridBar {
  unsigned *bar;
  int *fault;
  unsigned epoch;  // barriers passed (thread 0's count)
  int fail;        // this block gave up
};

__device__ __forceinline__ bool grid_sync(GridBar *gb) {
  __syncthreads();
  if (threadIdx.x == 0 && !gb->fail) {
    const unsigned target = ++gb->epoch * gridDim.x;
    red_release_add(gb->bar, 1u);
    if ((int)(ld_acquire(gb->bar) - target) < 0) {
      const unsigned long long t0 = global_ns();
      while ((int)(ld_acquire(gb->bar) - target) < 0) {
        if (*(volatile int *)gb->fault || global_ns() - t0 > kWaitNs) {
          atomicExch(gb->fault, 1);
          gb->fail = 1;
          break;
        }
      }
    }
  }
  __syncthreads();
  return !gb->fail;
}

// n grid barriers and nothing else (the timer's measure of one barrier).
// absent >= 0 (the barrier's self-test): that block leaves without
// arriving, so the others' waits run out and set the fault word.
static __global__ void __launch_bounds__(512, 1) k_grid_sync_probe(unsigned *bar, int *fault, int n, int absent) {
  __shared__ GridBar gb;
  if ((int)blockIdx.x == absent) return;
  if (threadIdx.x == 0) gb = GridBar{bar, fault, 0u, 0};
  __syncthreads();
  for (int q = 0; q < n; q++)
    if (!grid_sync(&gb)) break;
}

// ------------------------------------------------------------------ persistent solve
template <typename T>
struct PersistArgs {
  const TailLevel<T> *lv;  // levels 0 .. top; lv[top] is the fine grid, lv[top].b the CG residual r
  int top;                 // the finest level
  int btop;                // levels btop .. 0 run in block 0 (the one-block tail), btop >= 1
  T *r, *p[2], *w;         // CG vectors: the direction update reads p[i & 1] and writes p[1 - (i & 1)]
  T *y;                    // the solution update y += alpha p (not the ACC form)
  double *y64;             // ACC: y64 += (yscale alpha) p in FP64
  const double *src64;     // mixed form: r = (T)(src64 / ||src64||) with ||src64||^2 at *rr64
  const double *rr64;
  int unprec;              // unpreconditioned norm: r.r tested after each residual update
  int do_pend;             // the last deferred y += alpha p here (else the caller's)
  int max_iters;           // iterations before the launch gives up (the host reports a timeout)
  KspState *st;
  double *part;            // partial sums: [2 slots][2 values][gridDim.x]
  unsigned *bar;           // grid barrier counter (zeroed before the launch)
  int *fault;
  const T *S0, *S1, *S2, *ilam;  // the coarse solve (level 0)
  T *work;
  int n0, n1, n2, smem;
  T dinv;
  int copy_off;            // offset of the tail's shared-memory copy in the dynamic shared memory (-1: none)
};

// Per-thread partial sums -> one partial per block -> barrier -> every block
// sums the partials in the same order and thread 0 calls fin(sums) (on the
// block's copy of the solver state).  Returns false when a barrier gave up.
template <int NV, class FN>
__device__ __forceinline__ bool grid_reduce_fn(double (&v)[NV], double *part, int &slot, GridBar *gb, const FN &fin) {
  block_sum<NV>(v);
  const int nb = gridDim.x;
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) part[(slot * 2 + q) * nb + blockIdx.x] = v[q];
  if (!grid_sync(gb)) return false;
  if (threadIdx.x < 32) {
    double s[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
      s[q] = 0.0;
      for (int b = threadIdx.x; b < nb; b += 32) s[q] += __ldcg(&part[(slot * 2 + q) * nb + b]);
    }
    warp_sum<NV>(s);
    if (threadIdx.x == 0) fin(s);
  }
  __syncthreads();
  slot ^= 1;  // the next reduction writes the other slot: no block still reads this one after the next barrier
  return true;
}

// grid_reduce_fn with a KSP finaliser on the block's copy of the KSP state
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *part, int &slot, GridBar *gb, KspState *ks,
                                            Fin fin, double *out = nullptr) {
  return grid_reduce_fn<NV>(v, part, slot, gb, [&](double *t) { ksp_finalize(ks, fin, t, NV, out); });
}

// b - A x at (i, j, k) from values by coordinates (resid_at's operations;
// xf(ii, jj, kk) is called for the centre and its interior neighbours only)
template <int DIM, typename T, class XF>
__device__ __forceinline__ T resid_ijk(const Geom &g, const Wv<T> &w, const XF &xf, int i, int j, int k, T bv) {
  const T xc = xf(i, j, k);
  const bool bd = jk_bdry(g, DIM, j, k) || i == 0 || i == g.mx - 1;
  if (bd) return fma(-w.sd, xc, bv);
  const T a = (i - 1 > 0 ? xf(i - 1, j, k) : T(0)) + (i + 1 < g.mx - 1 ? xf(i + 1, j, k) : T(0));
  T s = fma(w.sx, a, bv);
  if (DIM >= 2) s = fma(w.sy, (j - 1 > 0 ? xf(i, j - 1, k) : T(0)) + (j + 1 < g.my - 1 ? xf(i, j + 1, k) : T(0)), s);
  if (DIM >= 3) s = fma(w.sz, (k - 1 > 0 ? xf(i, j, k - 1) : T(0)) + (k + 1 < g.mz - 1 ? xf(i, j, k + 1) : T(0)), s);
  return fma(-w.sd, xc, s);
}

// (P^T r_f) at coarse point (I, J, K) from fine values by coordinates
// (restrict_pt's operations; rf(fi, fj, fk) is 0 for fi >= mx, the padding)
template <int DIM, typename T, class RF>
__device__ __forceinline__ T restrict_ijk(const Geom &g, const RF &rf, int I, int J, int K) {
  const T h = T(0.5);
  auto row = [&](int fj, int fk) -> T {
    const int fi = 2 * I;
    const T L = fi > 0 ? rf(fi - 1, fj, fk) : T(0);
    const T R = fi + 1 < g.pitch ? rf(fi + 1, fj, fk) : T(0);
    return fma(h, L + R, rf(fi, fj, fk));
  };
  auto rowsum = [&](int fk) -> T {
    const int fj = 2 * J;
    const T c = row(fj, fk);
    if (DIM < 2) return c;
    const T sr = fj - 1 >= 0 ? row(fj - 1, fk) : T(0);
    const T nr = fj + 1 < g.my ? row(fj + 1, fk) : T(0);
    return fma(h, sr + nr, c);
  };
  if (DIM >= 3) {
    const T below = K > 0 ? rowsum(2 * K - 1) : T(0);
    const T mid = rowsum(2 * K);
    const T above = 2 * K + 1 < g.mz ? rowsum(2 * K + 1) : T(0);
    return fma(h, below + above, mid);
  }
  return rowsum(K);
}

constexpr int kMaxPersistLevels = 24;

// The whole CG solve of run_ksp (its set-up, the iterations until the state
// stops, the last deferred update) for grids whose phases are too small for a
// launch each.  Launched cooperatively with one block per SM at most; the
// state in global memory is read at the start and written back by block 0 at
// the end.  ACC: the accurate inner form of the mixed solve (difference-form
// apply, FP64 accumulation of the correction).
//
// Phases of one iteration, each ended by a grid barrier: the kernels of the
// launch-per-phase form, in their order (p = z + (beta/beta_old) p_old with
// w = A p and p.w; r -= alpha w; per level two smoothing steps from zero,
// the residual, its restriction; block 0: the levels of at most
// persist_tail nodes (vtail_body); per level upwards the prolongation and
// two smoothing steps, the last one with z.z and z.r on the finest level),
// some of them fused in FP32 (FUSE_* below).  Values formed on the fly are
// the same operations as their stored forms, so every point's value is the
// launch-per-phase form's.  A phase never writes an array that another point
// of the same phase reads.
// The shared state of a persistent launch's blocks.
template <typename T>
struct PersistShared {
  KspState ks;                           // this block's copy of the KSP state
  GridBar gb;
  TailLevel<T> lv[kMaxPersistLevels];  // the level table, read at every phase
  TailLevel<T> sv[kMaxPersistLevels];  // block 0: the tail's shared-memory copy
};

// The barrier, the level table, and block 0's tail tables (once per launch).
template <int DIM, typename T>
__device__ void persist_setup(const PersistArgs<T> &a, PersistShared<T> &sh, unsigned char *fg_tail_sm) {
  const int tid = threadIdx.x;
  if (tid == 0) sh.gb = GridBar{a.bar, a.fault, 0u, 0};
  for (int l = tid; l <= a.top; l += blockDim.x) sh.lv[l] = a.lv[l];
  __syncthreads();
  if (blockIdx.x == 0) {
    if (a.copy_off >= 0) vtail_prepare<DIM, T>(sh.lv, a.btop, fg_tail_sm, a.copy_off, sh.sv);
    if (a.smem) coarse_stage<DIM, T>(a.S0, a.S1, a.S2, a.ilam, a.n0, a.n1, a.n2, fg_tail_sm);
    __syncthreads();
  }
}

// Calls f(n, i, j, k) for this thread's points of a level: points are dealt
// to the blocks of a persistent launch in warp-sized runs, round robin, so a
// small level's points spread over all SMs (FP64 work on one SM is slow) and
// every warp still reads consecutive points.
template <int DIM, class F>
__device__ __forceinline__ void persist_each(const Geom &g, F &&f) {
  const int tid = threadIdx.x;
  const long long gt = ((long long)(tid >> 5) * gridDim.x + blockIdx.x) * 32 + (tid & 31);
  const long long G = (long long)gridDim.x * blockDim.x;
  const int N = level_npts<DIM>(g);
  if (N < (1 << 24)) {
    const LevelDiv dv(g);
    for (long long q = gt; q < N; q += G) {
      int i, j, k;
      const long long n = level_pos_f<DIM>(g, dv, (int)q, 0, i, j, k);
      f(n, i, j, k);
    }
  } else {
    for (long long q = gt; q < N; q += G) {
      int i, j, k;
      const long long n = level_pos<DIM>(g, (int)q, 0, i, j, k);
      f(n, i, j, k);
    }
  }
}

// The V-cycle from zero of a persistent launch (enq_pc's V-cycle, two
// Chebyshev/Jacobi steps per level) into lv[top].X[0], on the fine
// right-hand side bfin(m): an array, or values formed on the fly (bfin is
// read at the points and their neighbours in the finest level's passes, so
// what it reads may change only in its last pass, at the point itself).
//   first(rr) runs after the first pass of the finest level (rr: this
//     thread's sum of bfin^2 there); it ends that phase and returns 0 when a
//     barrier gave up, 1 to go on, 2 when the rest is not needed;
//   last(n, i, j, k, v, bv) runs for every fine point in the last pass (v the
//     V-cycle's value, bv = bfin(n)); end() ends that phase (a reduction or a
//     barrier) and returns false when a barrier gave up.
// Returns false when a barrier gave up, true at the end or when first
// returned 2.  Levels btop .. 0 run in block 0 (vtail_run); FUSE_RR fuses the
// residual with its restriction, FUSE_PC the prolongation with the first
// post-smoothing step (FP32 2D only: their 3D forms repeat 27 and 7 point
// evaluations and measured slower).  Values formed on the fly are the same
// operations as their stored forms, so every point's value is the
// launch-per-phase V-cycle's.
template <int DIM, typename T, class BF, class FIRST, class LAST, class END>
__device__ bool persist_vcycle(const PersistArgs<T> &a, PersistShared<T> &sh, unsigned char *fg_tail_sm,
                               const BF &bfin, const FIRST &first, const LAST &last, const END &end) {
  constexpr bool FUSE_RR = sizeof(T) == 4 && DIM == 2, FUSE_PC = FUSE_RR;
  const TailLevel<T> *lv = sh.lv;
  auto sync = [&]() { return grid_sync(&sh.gb); };
  for (int l = a.top; l > a.btop; l--) {
    const TailLevel<T> &L = lv[l];
    const TailLevel<T> &C = lv[l - 1];
    const Geom &g = L.g;
    const Wv<T> w(g);
    const bool fine = l == a.top;
    auto bval = [&](long long m) -> T { return fine ? bfin(m) : L.b[m]; };
    T rr = T(0);
    persist_each<DIM>(g, [&](long long n, int i, int j, int k) {  // x1 = a0 b - a1 A b (v_cheb2_zero)
      const T bc = bval(n);
      T mab;
      if (fine) mab = resid_at<DIM, T>(g, w, bfin, n, i, j, k, T(0));
      else mab = resid_pt<DIM, T>(g, w, L.b, n, i, j, k, T(0));
      L.X[1][n] = fma(L.a1, mab, L.a0 * bc);
      rr = fma(bc, bc, rr);
    });
    if (fine) {
      const int f = first(rr);
      if (f != 1) return f == 2;
    } else if (!sync()) {
      return false;
    }
    if constexpr (FUSE_RR) {
      auto rf = [&](int ii, int jj, int kk) -> T {  // the fine residual b - A x1 (v_resid)
        if (ii >= g.mx) return T(0);
        const long long m = (long long)kk * g.plane + (long long)jj * g.pitch + ii;
        return resid_pt<DIM, T>(g, w, L.X[1], m, ii, jj, kk, bval(m));
      };
      persist_each<DIM>(C.g, [&](long long m, int I, int J, int K) { C.b[m] = restrict_ijk<DIM, T>(g, rf, I, J, K); });
    } else {
      persist_each<DIM>(g, [&](long long n, int i, int j, int k) {  // r = b - A x1 (v_resid)
        L.r[n] = resid_pt<DIM, T>(g, w, L.X[1], n, i, j, k, bval(n));
      });
      if (!sync()) return false;
      persist_each<DIM>(C.g, [&](long long m, int I, int J, int K) { C.b[m] = restrict_pt<DIM, T>(g, L.r, I, J, K); });
    }
    if (!sync()) return false;
  }
  if (blockIdx.x == 0)  // smem 2: the coarse tables are staged
    vtail_run<DIM, T>(lv, a.btop, 0, a.S0, a.S1, a.S2, a.ilam, a.work, a.n0, a.n1, a.n2, a.smem ? 2 : 0, a.dinv,
                      fg_tail_sm, a.copy_off, sh.sv);
  if (!sync()) return false;
  for (int l = a.btop + 1; l <= a.top; l++) {
    const TailLevel<T> &L = lv[l];
    const TailLevel<T> &C = lv[l - 1];
    const Geom &g = L.g;
    const Wv<T> w(g);
    const bool fine = l == a.top;
    auto bval = [&](long long m) -> T { return fine ? bfin(m) : L.b[m]; };
    // x1' = x1 + P x_c and x2 = x1' + c1 (b - A x1'); x1' ends in xs
    T *xs;
    if constexpr (FUSE_PC) {
      // x1' formed at the neighbours too, kept in X[0] (X[1] is still read there)
      auto x1p = [&](int ii, int jj, int kk) -> T {
        const long long m = (long long)(DIM >= 3 ? kk : 0) * g.plane + (long long)jj * g.pitch + ii;
        return prolong_add<DIM, T>(C.g, C.X[0], ii, jj, kk, L.X[1][m]);
      };
      persist_each<DIM>(g, [&](long long n, int i, int j, int k) {
        const T xc = x1p(i, j, k);
        const T r = resid_ijk<DIM, T>(g, w, x1p, i, j, k, bval(n));
        L.X[0][n] = xc;
        L.X[2][n] = fma(L.c1, r, T(1) * xc);
      });
      xs = L.X[0];
    } else {
      persist_each<DIM>(g, [&](long long n, int i, int j, int k) {  // v_prolong, in place
        L.X[1][n] = prolong_add<DIM, T>(C.g, C.X[0], i, j, k, L.X[1][n]);
      });
      if (!sync()) return false;
      persist_each<DIM>(g, [&](long long n, int i, int j, int k) {  // v_cheb without x_{k-1}
        const T r = resid_pt<DIM, T>(g, w, L.X[1], n, i, j, k, bval(n));
        L.X[2][n] = fma(L.c1, r, T(1) * L.X[1][n]);
      });
      xs = L.X[1];
    }
    if (!sync()) return false;
    persist_each<DIM>(g, [&](long long n, int i, int j, int k) {  // x0 = ckm1 x1' + ck x2 + crd (b - A x2)
      const T bv = bval(n);
      const T r = resid_pt<DIM, T>(g, w, L.X[2], n, i, j, k, bv);
      const T v = fma(L.crd, r, fma(L.ckm1, xs[n], L.ck * L.X[2][n]));
      L.X[0][n] = v;
      if (fine) last(n, i, j, k, v, bv);
    });
    if (fine) {
      if (!end()) return false;
    } else if (!sync()) {
      return false;
    }
  }
  return true;
}

// One CG solve (run_ksp's work) on the state in sh.ks: the set-up from r (or
// from src64 scaled by 1/sqrt(*rr64), when src64 is given), the iterations
// until the state stops (or a.max_iters ran: false in *it_out's count), and
// with a.do_pend the last deferred update.  Returns false when a barrier gave
// up.  Every block runs it with identical state.
template <int DIM, typename T, bool ACC>
__device__ bool persist_cg(const PersistArgs<T> &a, const double *src64, const double *rr64, PersistShared<T> &sh,
                           int &slot, unsigned char *fg_tail_sm) {
  const int tid = threadIdx.x;
  KspState &ks = sh.ks;
  GridBar &gb = sh.gb;
  const TailLevel<T> *lv = sh.lv;
  auto sync = [&]() { return grid_sync(&gb); };
  auto each = [&](const Geom &g, auto &&f) { persist_each<DIM>(g, f); };
  const TailLevel<T> &F = lv[a.top];
  const Geom &gf = F.g;
  const Wv<T> wf(gf);
  T *z = F.X[0];

  // FUSE_R: the CG residual update r - alpha w inside the first smoothing pass
  // of the V-cycle (FP32 only: a neighbour's value is formed by every point
  // that reads it, and FP64 throughput on this part is 1/64 of FP32's).
  constexpr bool FUSE_R = sizeof(T) == 4;

  // V-cycle from zero into z on r.  upd (FUSE_R): on r - al w, the CG
  // residual update of this iteration, stored by the last pass; unprec: its
  // r.r reduced after the first pass (FIN_RR).  The last smoothing step's z.z
  // and z.r are reduced and finalised as `fin`.  Returns false when a
  // barrier gave up; true early when FIN_RR stopped the solve.
  auto vcycle = [&](Fin fin, bool upd, T al, bool unprec) -> bool {
    auto bfin = [&](long long m) -> T { return upd ? fma(-al, a.w[m], a.r[m]) : a.r[m]; };
    auto first = [&](T rr) -> int {
      if (upd && unprec) {
        double v1[1] = {(double)rr};
        if (!grid_reduce<1>(v1, a.part, slot, &gb, &ks, FIN_RR)) return 0;
        if (ks.done) {  // r stored; the rest of the V-cycle is not needed
          each(gf, [&](long long n, int, int, int) { a.r[n] = bfin(n); });
          return 2;
        }
        return 1;
      }
      return sync() ? 1 : 0;
    };
    T zz = T(0), zr = T(0);
    auto last = [&](long long n, int, int, int, T v, T bv) {
      zz = fma(v, v, zz);
      zr = fma(v, bv, zr);
      if (upd) a.r[n] = bv;
    };
    auto end = [&]() -> bool {
      double v2[2] = {(double)zz, (double)zr};
      return grid_reduce<2>(v2, a.part, slot, &gb, &ks, fin);
    };
    return persist_vcycle<DIM, T>(a, sh, fg_tail_sm, bfin, first, last, end);
  };

  // ---- set-up (enq_cg_init)
  bool ok = true;
  if (src64) {  // r = r64 / ||r64|| rounded to T as v_demote_init rounds it, r.r
    const double is = 1.0 / sqrt(*rr64);
    T rr = T(0);
    each(gf, [&](long long n, int, int, int) {
      T o;
      if constexpr (sizeof(T) == 4) o = d2f_bits(src64[n]) * (float)is;
      else o = (T)(src64[n] * is);
      a.r[n] = o;
      rr = fma(o, o, rr);
    });
    double v1[1] = {(double)rr};
    ok = grid_reduce<1>(v1, a.part, slot, &gb, &ks, FIN_INIT_RR);
  } else if (a.unprec) {
    T rr = T(0);
    each(gf, [&](long long n, int, int, int) {
      const T v = a.r[n];
      rr = fma(v, v, rr);
    });
    double v1[1] = {(double)rr};
    ok = grid_reduce<1>(v1, a.part, slot, &gb, &ks, FIN_INIT_RR);
  }
  if (ok && !ks.done) ok = vcycle(FIN_INIT_ZZZR, false, T(0), false);

  // ---- iterations (enq_cg_iter)
  int it = 0;
  while (ok && !ks.done && it < a.max_iters) {
    it++;
    const int par = ks.i & 1;
    const T *pold = a.p[par];
    T *pnew = a.p[1 - par];
    const bool first = ks.i == 0;
    const bool pend = ks.pend && (ACC ? (void *)a.y64 : (void *)a.y);
    const bool yfresh = pend && ks.i == 1 && (!ACC || ks.yfresh);
    const T bb = (T)ks.bratio;
    auto pf = [&](long long m) -> T { return first ? z[m] : fma(bb, pold[m], z[m]); };
    T acc = T(0);
    if constexpr (ACC) {
      const double ya = pend ? ks.yscale * ks.alpha : 0.0;
      each(gf, [&](long long n, int i, int j, int k) {
        const T pc = pf(n);
        const T v = apply_diff_at<DIM, T>(gf, wf, pf, n, i, j, k);
        acc = fma(pc, v, acc);
        pnew[n] = pc;
        a.w[n] = v;
        if (pend) a.y64[n] = fma(ya, to_y<double>(pold[n]), yfresh ? 0.0 : a.y64[n]);
      });
    } else {
      const T ya = pend ? (T)ks.alpha : T(0);
      each(gf, [&](long long n, int i, int j, int k) {
        const T pc = pf(n);
        const T v = -resid_at<DIM, T>(gf, wf, pf, n, i, j, k, T(0));
        acc = fma(pc, v, acc);
        pnew[n] = pc;
        a.w[n] = v;
        if (pend) a.y[n] = fma(ya, pold[n], yfresh ? T(0) : a.y[n]);
      });
    }
    double v1[1] = {(double)acc};
    if (!(ok = grid_reduce<1>(v1, a.part, slot, &gb, &ks, FIN_PW)) || ks.done) break;
    const T al = (T)ks.alpha;
    if constexpr (FUSE_R) {  // r -= alpha w (v_cg_r) inside the V-cycle's first pass
      ok = vcycle(FIN_ZZZR, true, al, a.unprec != 0);
    } else {
      T rr = T(0);
      each(gf, [&](long long n, int, int, int) {  // r -= alpha w, r.r (v_cg_r)
        const T rn = fma(-al, a.w[n], a.r[n]);
        a.r[n] = rn;
        rr = fma(rn, rn, rr);
      });
      if (a.unprec) {
        double v2[1] = {(double)rr};
        ok = grid_reduce<1>(v2, a.part, slot, &gb, &ks, FIN_RR);
      } else {
        ok = sync();
      }
      if (!ok || ks.done) break;
      ok = vcycle(FIN_ZZZR, false, T(0), false);
    }
  }

  // ---- the last deferred y += alpha p (v_cg_pend), when the caller does not take it
  if (ok && a.do_pend && !ACC) {
    const bool written = ksp_y_written(&ks);
    const int pend = ks.pend;
    if (!written || pend) {
      const T al = pend ? (T)ks.alpha : T(0);
      const T *pv = pend == 1 ? a.p[0] : a.p[1];
      each(gf, [&](long long n, int, int, int) {
        const T yy = written ? a.y[n] : T(0);
        a.y[n] = pend ? fma(al, pv[n], yy) : yy;
      });
    }
  }
  __syncthreads();
  if (tid == 0) ks.loops = (unsigned)it;
  __syncthreads();
  return ok;
}

// The whole CG solve of run_ksp in one cooperative launch (one block per SM
// at most): the state read from a.st at the start, written back by block 0.
template <int DIM, typename T, bool ACC>
__global__ void __launch_bounds__(512, 1) k_ksp_persist(PersistArgs<T> a) {
  extern __shared__ __align__(16) unsigned char fg_tail_sm[];
  __shared__ PersistShared<T> sh;
  if (threadIdx.x == 0) {
    sh.ks = *a.st;
    sh.ks.ndone = nullptr;
  }
  persist_setup<DIM, T>(a, sh, fg_tail_sm);
  if (sh.ks.done) return;  // every block sees the same state
  int slot = 0;
  persist_cg<DIM, T, ACC>(a, a.src64, a.rr64, sh, slot, fg_tail_sm);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sh.ks.ndone = a.st->ndone;
    *a.st = sh.ks;
  }
}

// ------------------------------------------------------------------ the V-cycle tail in one cooperative launch
// Levels a.top .. 0 of a launch-per-phase V-cycle from zero (enq_vcycle below
// the levels that keep a launch per phase): persist_vcycle on level top's
// stored b, its result in X[0] of every level (as k_vtail leaves it).  The
// KSP state is read once: it does not change inside a V-cycle, so every block
// returns, or runs every barrier.  *a.bar must be zero at the launch.
template <int DIM, typename T>
__global__ void __launch_bounds__(512, 1) k_vtail_coop(PersistArgs<T> a, const KspState *st) {
  extern __shared__ __align__(16) unsigned char fg_tail_sm[];
  __shared__ PersistShared<T> sh;
  if (ksp_done(st)) return;
  persist_setup<DIM, T>(a, sh, fg_tail_sm);
  const T *b = sh.lv[a.top].b;
  auto bf = [&](long long m) -> T { return b[m]; };
  auto first = [&](T) -> int { return grid_sync(&sh.gb) ? 1 : 0; };
  auto last = [](long long, int, int, int, T, T) {};
  auto end = []() -> bool { return true; };  // the launch's end orders the writes for the next kernel
  persist_vcycle<DIM, T>(a, sh, fg_tail_sm, bf, first, last, end);
}

// ------------------------------------------------------------------ the mixed solve in one launch
// FP64 iterative refinement around the FP32 inner CG (solve_dim's mixed
// loop), all on the device: the stop tests and inner tolerances in every
// block from identical values, the inner solves by persist_cg, the last
// deferred update of each (v_pend_acc / v_pend_promote) and the FP64 true
// residual r64 = b64 - A y64 with its norm as grid phases.  What the host
// learns at the end is in MixedOut.
struct MixedArgs {
  const double *b64;  // the right-hand side of J y = b
  double *y64, *r64;  // the solution (zeroed here if no step runs) and the FP64 residual
  float *y32;         // the standard inner form's correction (not ACC)
  const double *bb;   // b64.b64, stored by the kernel that formed b64
  double rtol, atol, inner_rtol, first_floor;
  int outer_max_it, max_it, inner_max_it;
  double dtol;
  struct MixedOut *out;
};

struct MixedOut {
  int status;  // 0, or FISHGPU_ERR_TIMEOUT when an inner solve's iteration cap ran out
  int its, outer, reason, nhist;
  int inner_its[FISHGPU_MAX_OUTER];
  double bn;
  double hist[FISHGPU_MAX_HIST];
};

template <int DIM, bool ACC>
__global__ void __launch_bounds__(512, 1) k_mixed_persist(PersistArgs<float> a, MixedArgs m) {
  extern __shared__ __align__(16) unsigned char fg_tail_sm[];
  __shared__ PersistShared<float> sh;
  __shared__ double s_rr, s_sum;
  persist_setup<DIM, float>(a, sh, fg_tail_sm);
  const int tid = threadIdx.x;
  const long long gt = ((long long)(tid >> 5) * gridDim.x + blockIdx.x) * 32 + (tid & 31);
  const long long G = (long long)gridDim.x * blockDim.x;
  const Geom &gf = sh.lv[a.top].g;
  const int N = level_npts<DIM>(gf);
  const LevelDiv dv(gf);
  auto each = [&](auto &&f) {
    for (long long q = gt; q < N; q += G) {
      int i, j, k;
      const long long n = N < (1 << 24) ? level_pos_f<DIM>(gf, dv, (int)q, 0, i, j, k)
                                         : level_pos<DIM>(gf, (int)q, 0, i, j, k);
      f(n, i, j, k);
    }
  };
  MixedOut *out = m.out;
  const bool b0 = blockIdx.x == 0 && tid == 0;
  const double bn = sqrt(*m.bb);
  const double ttol = fmax(m.rtol * bn, m.atol);
  double rn = bn;
  int reason = 0, its = 0, outer = 0, nh = 0, status = 0, slot = 0;
  if (b0) {
    out->bn = bn;
    out->hist[nh] = rn;
  }
  nh++;
  bool ok = true;
  while (ok) {
    if (isnan(rn) || isinf(rn)) { reason = R_DIVERGED_NANORINF; break; }
    if (rn <= ttol) { reason = rn < m.atol ? R_CONVERGED_ATOL : R_CONVERGED_RTOL; break; }
    if (outer >= m.outer_max_it || its >= m.max_it) { reason = R_DIVERGED_ITS; break; }
    double irtol = fmax(m.inner_rtol, 0.5 * ttol / rn);
    if (outer == 0) irtol = fmax(irtol, m.first_floor);
    if (irtol > 0.5) irtol = 0.5;
    if (tid == 0) {  // the inner solve's fresh state (reset_state)
      memset(&sh.ks, 0, sizeof(sh.ks));
      sh.ks.rtol = irtol;
      sh.ks.atol = m.atol;
      sh.ks.dtol = m.dtol;
      sh.ks.max_it = m.inner_max_it;
      sh.ks.norm_type = FISHGPU_NORM_UNPRECONDITIONED;
      sh.ks.betaold = 1.0;
      sh.ks.yscale = rn;
      sh.ks.yfresh = outer == 0 ? 1 : 0;
      s_rr = outer == 0 ? *m.bb : s_sum;
    }
    __syncthreads();
    // r32 = r / ||r|| (r: b64 in the first step, r64 after) inside the set-up
    if (!(ok = persist_cg<DIM, float, ACC>(a, outer == 0 ? m.b64 : m.r64, &s_rr, sh, slot, fg_tail_sm))) break;
    const KspState &ks = sh.ks;
    if (!ks.done) {  // the inner iteration cap ran out (the device loop's cap)
      status = FISHGPU_ERR_TIMEOUT;
      break;
    }
    its += ks.its;
    if (b0 && outer < FISHGPU_MAX_OUTER) out->inner_its[outer] = ks.its;
    if (ks.reason == R_DIVERGED_NANORINF || ks.reason == R_DIVERGED_INDEFINITE_MAT ||
        ks.reason == R_DIVERGED_INDEFINITE_PC) {
      reason = ks.reason;
      break;
    }
    {  // the last deferred update into y64 (v_pend_acc / v_pend_promote)
      const int pend = ks.pend;
      if constexpr (ACC) {
        const bool keep = ksp_y_written(&ks) || !ks.yfresh;
        if (!keep || pend) {
          const double ya = pend ? ks.yscale * ks.alpha : 0.0;
          const float *pv = pend == 1 ? a.p[0] : a.p[1];
          each([&](long long n, int, int, int) {
            const double yy = keep ? m.y64[n] : 0.0;
            m.y64[n] = pend ? fma(ya, f2d_bits(pv[n]), yy) : yy;
          });
        }
      } else {
        const bool written = ksp_y_written(&ks);
        const float al = pend ? (float)ks.alpha : 0.f;
        const float *pv = pend == 1 ? a.p[0] : a.p[1];
        const bool fresh = outer == 0;
        each([&](long long n, int, int, int) {
          float ev = written ? m.y32[n] : 0.f;
          if (pend) ev = fmaf(al, pv[n], ev);
          m.y64[n] = fma(rn, (double)ev, fresh ? 0.0 : m.y64[n]);
        });
      }
    }
    if (!(ok = grid_sync(&sh.gb))) break;
    {  // r64 = b64 - A y64 and its norm (v_resid<double, NORM>)
      const Wv<double> w(gf);
      double rr = 0.0;
      each([&](long long n, int i, int j, int k) {
        const double v = resid_pt<DIM, double>(gf, w, m.y64, n, i, j, k, m.b64[n]);
        m.r64[n] = v;
        rr = fma(v, v, rr);
      });
      double v1[1] = {rr};
      if (!(ok = grid_reduce<1>(v1, a.part, slot, &sh.gb, &sh.ks, FIN_STORE, &s_sum))) break;
    }
    rn = sqrt(s_sum);
    outer++;
    if (b0 && nh < FISHGPU_MAX_HIST) out->hist[nh] = rn;
    nh++;
  }
  if (ok && outer == 0) {  // no step ran: the correction is zero
    each([&](long long n, int, int, int) { m.y64[n] = 0.0; });
  }
  if (b0) {
    out->status = ok ? status : FISHGPU_ERR_TIMEOUT;
    out->its = its;
    out->outer = outer;
    out->reason = reason;
    out->nhist = nh;
  }
}

}  // namespace fg
