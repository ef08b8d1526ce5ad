// kernels.cuh -- the point-wise operator kernels of the call-back entry
// points (any owned sub-box, global indexing) and the exact coarse solve.
//
// Templated on the dimension DIM (1,2,3) and on the storage and arithmetic
// type T.  A thread owns one (i,j) column and marches `zc` consecutive
// k-planes; blocks are (32,8) threads over (i,j) (256 x 1 in 1D).  The
// solver's own whole-grid kernels (vectorised, padded layout) live in
// vkernels.cuh.
//
// The operator is the Jacobian the reference assembles
// (c/ch6/poissonfunctions.c:117-258), applied matrix-free: boundary rows
// are scdiag*p; interior rows are scdiag*p - sum_d sc_d * (neighbours along d
// that are NOT boundary nodes).  The FP64 instruction count is kept minimal
// (GB300's FP64 pipe, not HBM, bounds the FP64 form): 1 + 2*DIM per apply.
#pragma once

#include "fishgpu_internal.cuh"

namespace fg {

struct Range {   // owned box [xs,xe) x [ys,ye) x [zs,ze)
  int xs, ys, zs, xe, ye, ze;
};

__host__ __device__ inline Range full_range(const Geom &g) { return Range{0, 0, 0, g.mx, g.my, g.mz}; }

template <typename T>
struct Wt {
  T sx, sy, sz, sd;
  __device__ __forceinline__ explicit Wt(const Geom &g) {
    if constexpr (sizeof(T) == 4) {  // FP32 weights rounded on the host (Geom::scf)
      sx = g.scf[0];
      sy = g.scf[1];
      sz = g.scf[2];
      sd = g.scdiagf;
    } else {
      sx = g.sc[0];
      sy = g.sc[1];
      sz = g.sc[2];
      sd = g.scdiag;
    }
  }
};

template <int DIM>
__device__ __forceinline__ bool on_bdry(const Geom &g, int i, int j, int k) {
  bool b = (i == 0) | (i == g.mx - 1);
  if (DIM >= 2) b |= (j == 0) | (j == g.my - 1);
  if (DIM >= 3) b |= (k == 0) | (k == g.mz - 1);
  return b;
}

// s0 + sum_d sc_d * (interior neighbours of n along d); n must be interior.
template <int DIM, typename T>
__device__ __forceinline__ T nbr_sum(const T *__restrict__ p, long long n, int i, int j, int k,
                                     const Geom &g, const Wt<T> &w, T s0) {
  T a = (i - 1 > 0 ? p[n - 1] : T(0)) + (i + 1 < g.mx - 1 ? p[n + 1] : T(0));
  T s = fma(w.sx, a, s0);
  if (DIM >= 2) {
    T b = (j - 1 > 0 ? p[n - g.pitch] : T(0)) + (j + 1 < g.my - 1 ? p[n + g.pitch] : T(0));
    s = fma(w.sy, b, s);
  }
  if (DIM >= 3) {
    T c = (k - 1 > 0 ? p[n - g.plane] : T(0)) + (k + 1 < g.mz - 1 ? p[n + g.plane] : T(0));
    s = fma(w.sz, c, s);
  }
  return s;
}

// (A p)_n
template <int DIM, typename T>
__device__ __forceinline__ T apply_at(const T *__restrict__ p, long long n, int i, int j, int k,
                                      const Geom &g, const Wt<T> &w) {
  T pn = p[n];
  if (on_bdry<DIM>(g, i, j, k)) return w.sd * pn;
  return fma(w.sd, pn, -nbr_sum<DIM, T>(p, n, i, j, k, g, w, T(0)));
}

// (b - A x)_n
template <int DIM, typename T>
__device__ __forceinline__ T resid_at(const T *__restrict__ b, const T *__restrict__ x, long long n,
                                      int i, int j, int k, const Geom &g, const Wt<T> &w) {
  T xn = x[n], bn = b[n];
  if (on_bdry<DIM>(g, i, j, k)) return fma(-w.sd, xn, bn);
  return fma(-w.sd, xn, nbr_sum<DIM, T>(x, n, i, j, k, g, w, bn));
}

__device__ __forceinline__ bool ksp_done(const KspState *st) {
  return st && __ldcg(&st->done);
}

// Grid-stride loop over tiles of blockDim.x x blockDim.y columns x tm.zc
// planes (x fastest); a thread marches k through its tile's planes.
#define FG_POINT_LOOP_BEGIN(R)                                                  \
  for (int t_ = blockIdx.x; t_ < tm.tx * tm.ty * tm.tz; t_ += gridDim.x) {      \
    const int i = (R).xs + (t_ % tm.tx) * blockDim.x + threadIdx.x;             \
    const int j = (R).ys + ((t_ / tm.tx) % tm.ty) * blockDim.y + threadIdx.y;   \
    const int kbeg = (R).zs + (t_ / (tm.tx * tm.ty)) * tm.zc;                   \
    const int kend = min(kbeg + tm.zc, (R).ze);                                 \
    if (i < (R).xe && j < (R).ye) {                                             \
      for (int k = kbeg; k < kend; k++) {                                       \
        const long long n = gidx(g, i, j, k);

#define FG_POINT_LOOP_END \
  }                       \
  }                       \
  }

// ------------------------------------------------------------------ apply
// q = A p on the range; DOT: p.q reduced, finalised by `fin`.
template <int DIM, typename T, bool DOT>
__global__ void __launch_bounds__(256) k_apply(Geom g, Range R, Tiles tm, KspState *st,
                                               const T *__restrict__ p, T *__restrict__ q,
                                               Reducer red, int slot, Fin fin, double *out) {
  if (ksp_done(st)) return;
  const Wt<T> w(g);
  T acc = T(0);
  FG_POINT_LOOP_BEGIN(R)
  T v = apply_at<DIM, T>(p, n, i, j, k, g, w);
  q[n] = v;
  if (DOT) acc = fma(p[n], v, acc);
  FG_POINT_LOOP_END
  if (DOT) {
    double v1[1] = {(double)acc};
    reduce_and_finalize<1>(v1, red, slot, st, fin, out);
  }
}

// ------------------------------------------------------------------ coarse solve
// Exact solve on the coarsest level in ONE block: boundary rows x = b/scdiag;
// interior by sine-transform diagonalisation x = S (Lambda^{-1} (S b)) with
// S_d[i][k] = sqrt(2/(n+1)) sin(ik pi/(n+1)) (symmetric, orthogonal) and
// Lambda = sum_d sc_d (2 - 2cos(k_d pi/(n_d+1))).  S and 1/Lambda come from
// the host (setup).  With `smem` the transform matrices, 1/Lambda and the two
// work arrays are staged in dynamic shared memory (coarse_smem_bytes); else
// `work` (global, 2 * prod(n_d) entries per block) holds the work arrays.
// Every output is the same FMA chain in either form.
template <typename T>
inline size_t coarse_smem_bytes(int dim, int n0, int n1, int n2) {
  const size_t ni = (size_t)n0 * n1 * n2;
  size_t e = 3 * ni + (size_t)n0 * n0;
  if (dim >= 2) e += (size_t)n1 * n1;
  if (dim >= 3) e += (size_t)n2 * n2;
  return e * sizeof(T);
}

// Stages 1/Lambda and the transform matrices in the shared-memory layout of
// coarse_solve_block (after its two work arrays).  No barrier.
template <int DIM, typename T>
__device__ __forceinline__ void coarse_stage(const T *S0, const T *S1, const T *S2, const T *ilam, int n0, int n1,
                                             int n2, unsigned char *sm_raw) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int ni = n0 * n1 * n2;
  T *sl = reinterpret_cast<T *>(sm_raw) + 2 * ni, *s0 = sl + ni, *s1 = s0 + n0 * n0;
  T *s2 = s1 + (DIM >= 2 ? n1 * n1 : 0);
  for (int q = tid; q < ni; q += nt) sl[q] = ilam[q];
  for (int q = tid; q < n0 * n0; q += nt) s0[q] = S0[q];
  if (DIM >= 2)
    for (int q = tid; q < n1 * n1; q += nt) s1[q] = S1[q];
  if (DIM >= 3)
    for (int q = tid; q < n2 * n2; q += nt) s2[q] = S2[q];
}

// The solve of one block: b, x already offset to the block's plane (1D/2D),
// `sm` the block's dynamic shared memory, `work` its global work area.
template <int DIM, typename T>
__device__ __forceinline__ void coarse_solve_block(const Geom &g, const T *__restrict__ b, T *__restrict__ x,
                                                   const T *__restrict__ S0, const T *__restrict__ S1,
                                                   const T *__restrict__ S2, const T *__restrict__ ilam, T *work,
                                                   int n0, int n1, int n2, int smem, T dinv, unsigned char *sm_raw) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mzl = DIM < 3 ? 1 : g.mz;
  const int N = g.mx * g.my * mzl;
  for (int q = tid; q < N; q += nt) {  // dinv = (T)(1 / scdiag), from the host
    const int i = q % g.mx, r = q / g.mx, j = r % g.my, k = r / g.my;
    const long long n = gidx(g, i, j, k);
    x[n] = b[n] * dinv;
  }
  const int ni = n0 * n1 * n2;
  if (ni <= 0) return;
  T *A, *B;
  const T *Sd[3] = {S0, S1, S2};
  const T *il = ilam;
  if (smem) {
    T *sm = reinterpret_cast<T *>(sm_raw);
    A = sm;
    B = A + ni;
    T *sl = B + ni, *s0 = sl + ni, *s1 = s0 + n0 * n0, *s2 = s1 + (DIM >= 2 ? n1 * n1 : 0);
    if (smem != 2) coarse_stage<DIM, T>(S0, S1, S2, ilam, n0, n1, n2, sm_raw);  // 2: staged by the caller
    Sd[0] = s0;
    Sd[1] = s1;
    Sd[2] = s2;
    il = sl;
  } else {
    A = work + (size_t)blockIdx.x * 2 * ni;
    B = A + ni;
  }
  const int oj = DIM >= 2 ? 1 : 0, ok = DIM >= 3 ? 1 : 0;
  __syncthreads();
  for (int q = tid; q < ni; q += nt) {
    const int i = q % n0, j = (q / n0) % n1, k = q / (n0 * n1);
    A[q] = b[gidx(g, i + 1, j + oj, k + ok)];
  }
  __syncthreads();
  for (int pass = 0; pass < 2; pass++) {
    for (int d = 0; d < DIM; d++) {
      const T *S = Sd[d];
      const int nd = d == 0 ? n0 : d == 1 ? n1 : n2;
      const int st_d = d == 0 ? 1 : d == 1 ? n0 : n0 * n1;
      for (int q = tid; q < ni; q += nt) {
        const int c = d == 0 ? q % n0 : d == 1 ? (q / n0) % n1 : q / (n0 * n1);
        const int base = q - c * st_d;
        T s = T(0);
        for (int kk = 0; kk < nd; kk++) s = fma(S[c * nd + kk], A[base + kk * st_d], s);
        B[q] = s;
      }
      __syncthreads();
      T *t = A;
      A = B;
      B = t;
    }
    if (pass == 0) {
      for (int q = tid; q < ni; q += nt) A[q] *= il[q];
      __syncthreads();
    }
  }
  for (int q = tid; q < ni; q += nt) {
    const int i = q % n0, j = (q / n0) % n1, k = q / (n0 * n1);
    x[gidx(g, i + 1, j + oj, k + ok)] = A[q];
  }
}

template <int DIM, typename T>
__global__ void __launch_bounds__(1024) k_coarse(Geom g, KspState *st, int batch, const T *__restrict__ b,
                                                 T *__restrict__ x, const T *__restrict__ S0,
                                                 const T *__restrict__ S1, const T *__restrict__ S2,
                                                 const T *__restrict__ ilam, T *work, int n0, int n1, int n2,
                                                 int smem, T dinv) {
  extern __shared__ __align__(16) unsigned char fg_coarse_sm[];
  // 3D: one block for the grid; 1D/2D: block q solves k-plane q (a batch of
  // independent instances when batch != 0, else the single plane)
  const int plane = DIM < 3 ? (int)blockIdx.x : 0;
  if (batch && st) st += plane;
  if (ksp_done(st)) return;
  if (DIM < 3) {
    b += (long long)plane * g.plane;
    x += (long long)plane * g.plane;
  }
  coarse_solve_block<DIM, T>(g, b, x, S0, S1, S2, ilam, work, n0, n1, n2, smem, dinv, fg_coarse_sm);
}

}  // namespace fg
