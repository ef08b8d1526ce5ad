// vkernels.cuh -- the solver's hot kernels on the padded, vectorised layout.
//
// Layout of every solver vector (all levels, both precisions): row pitch a
// multiple of 4 points, base aligned to 16 B (FP32) / 32 B (FP64); the padding
// points i >= mx are kept at zero by every kernel that writes a vector, so
// pointwise kernels and dot products may run over the flat padded array.
//
// Work decomposition: a thread owns a "slot" of 4 consecutive x-points
// (one float4, or two double2).  The slots of one k-plane are numbered
// row-major; a block of `chunk` threads (256 by default) takes that many consecutive slots (crossing
// rows, so its loads per plane are one contiguous run of 4 KB (FP32)) and
// marches `zc` planes in k with the k-1/k/k+1 values of its slot in
// registers.  x-neighbours across slots come from warp shuffles (the warp's
// edge lanes load one scalar); y-neighbours are two vector loads (L1/L2
// hits); z-neighbours are the register window.  Grid = chunks x z-chunks,
// one block per (chunk, z-chunk): no grid-stride tail.  Batched 2D instances
// (planes) march rows instead: a thread owns one x-slot of a strip of rows
// with the rows j-1, j, j+1 in registers (march_rows).
#pragma once

#include "bitconv.cuh"
#include "fishgpu_internal.cuh"
#include "tma.cuh"

namespace fg {

template <typename T>
struct V4 {
  T x, y, z, w;
};

__device__ __forceinline__ V4<float> ld4(const float *p) {
  float4 v = *reinterpret_cast<const float4 *>(p);
  return V4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ V4<double> ld4(const double *p) {
  double2 a = *reinterpret_cast<const double2 *>(p);
  double2 b = *reinterpret_cast<const double2 *>(p + 2);
  return V4<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(float *p, const V4<float> &v) {
  *reinterpret_cast<float4 *>(p) = make_float4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void st4(double *p, const V4<double> &v) {
  *reinterpret_cast<double2 *>(p) = make_double2(v.x, v.y);
  *reinterpret_cast<double2 *>(p + 2) = make_double2(v.z, v.w);
}
template <typename T>
__device__ __forceinline__ V4<T> zero4() {
  return V4<T>{T(0), T(0), T(0), T(0)};
}
template <typename T>
__device__ __forceinline__ V4<T> add4(const V4<T> &a, const V4<T> &b) {
  return V4<T>{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w};
}
// (c - a) + (c - b) per element: the y- or z-part of the operator in
// difference form (see apply_diff_el)
template <typename T>
__device__ __forceinline__ V4<T> dsum4(const V4<T> &c, const V4<T> &a, const V4<T> &b) {
  return V4<T>{(c.x - a.x) + (c.x - b.x), (c.y - a.y) + (c.y - b.y), (c.z - a.z) + (c.z - b.z),
               (c.w - a.w) + (c.w - b.w)};
}
template <typename T>
__device__ __forceinline__ T el(const V4<T> &v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
template <typename T>
__device__ __forceinline__ void set_el(V4<T> &v, int e, T a) {
  if (e == 0) v.x = a; else if (e == 1) v.y = a; else if (e == 2) v.z = a; else v.w = a;
}

// Launch shape of the slot decomposition of one level.  Batched grids
// (batch = 1) are 2D instances stacked as k-planes: one block covers part of
// one plane, the KSP state, early exit and reductions are per plane.
struct Slots {
  int P4;         // slots per row (pitch / 4)
  int per_plane;  // slots per k-plane (P4 * my)
  int chunk;      // slots per block = threads per block (multiple of 32, <= 256)
  int nchunk;     // chunks per plane
  int zc, nz;     // planes per block, z-chunks
  int batch;      // 1: planes are independent instances
  long long tot4; // slots in the whole array
  int ry;         // 2D row march: a thread owns one x-slot of ry consecutive rows (0: one slot)
};

// zc_max planes per block at most, fewer when needed to keep at least
// `min_blocks` blocks (small levels, and the coarse-grid launches of the
// grid transfers, would otherwise leave SMs idle).
// ry > 1 (2D stencils only): a thread marches ry rows of one x-slot, with
// the rows j-1, j, j+1 in registers (the 2D counterpart of the z-march); a
// plane then holds P4 * ceil(my / ry) thread slots.  Pointwise kernels keep
// the plain form (ry = 0).
inline Slots make_slots(const Geom &g, int zc_max, int min_blocks = 2432, int chunk = 256, int batch = 0,
                        int ry = 0) {
  Slots s;
  s.P4 = g.pitch / 4;
  s.ry = (g.dim == 2 && ry > 1) ? ry : 0;
  s.per_plane = s.P4 * (s.ry ? (g.my + s.ry - 1) / s.ry : g.my);
  s.chunk = chunk;
  s.batch = batch;
  s.nchunk = (s.per_plane + chunk - 1) / chunk;
  int zc = 1;
  if (g.dim == 3 && !batch) {
    const long long want = ((long long)s.nchunk * g.mz) / (min_blocks > 0 ? min_blocks : 1);
    zc = (int)(want < 1 ? 1 : want > zc_max ? zc_max : want);
    if (zc > g.mz) zc = g.mz;
  }
  s.zc = zc;
  s.nz = (g.mz + s.zc - 1) / s.zc;
  s.tot4 = (long long)s.P4 * g.my * g.mz;  // vector slots, whatever the thread decomposition
  return s;
}
inline unsigned slot_blocks(const Slots &s) { return (unsigned)s.nchunk * (unsigned)s.nz; }

// Per-thread slot coordinates.
struct SlotPos {
  int i4, j, k0, k1;
  bool in;   // slot exists (within the plane)
  long long col;
};

__device__ __forceinline__ SlotPos slot_pos(const Geom &g, const Slots &s) {
  SlotPos p;
  const int c = blockIdx.x % s.nchunk, kz = blockIdx.x / s.nchunk;
  const int f = c * s.chunk + threadIdx.x;
  p.in = f < s.per_plane;
  p.j = p.in ? f / s.P4 : 0;  // row (the strip of a 2D row march: slot_pos_st)
  p.i4 = p.in ? (f - p.j * s.P4) * 4 : 0;
  p.k0 = kz * s.zc;
  p.k1 = min(p.k0 + s.zc, g.mz);
  p.col = (long long)p.j * g.pitch + p.i4;
  return p;
}

// Slot coordinates of a stencil thread: in a 2D row march p.j is the first
// row of the thread's strip.  A compile-time split, so that the 3D stencils
// carry no trace of it (a runtime test in slot_pos cost the 3D CG update
// kernel 6%).
template <int DIM>
__device__ __forceinline__ SlotPos slot_pos_st(const Geom &g, const Slots &s) {
  SlotPos p = slot_pos(g, s);
  if constexpr (DIM == 2) {
    if (s.ry) {
      p.j *= s.ry;
      p.col = (long long)p.j * g.pitch + p.i4;
    }
  }
  return p;
}

// Resident blocks per SM the compiler is asked to fit: 4 x 256 threads for
// the FP32 stencils that keep more streams or a reduction in flight (up to 64
// registers; see MinBlocksLean for the others).  FP64 stencils are
// FP64-pipe-bound and keep their registers.
template <typename T>
struct MinBlocks {
  static constexpr int value = sizeof(T) == 4 ? 4 : 1;
};

// Stencils with at most two input streams and no reduction fit 48 registers
// without spills: 5 blocks per SM.  Measured at 513^3: the two-step smoother
// from zero 0.248 -> 0.228 ms (6 blocks: no further gain), the residual
// 0.288 -> 0.267 ms; the Chebyshev step with x_{k-1} (three streams) is
// slower at 5 blocks (0.339 -> 0.377 ms) and keeps 4.  Of the kernels that
// reduce, the fused CG direction update + apply gains a little at 5 blocks
// (0.670 -> 0.657 ms) while the Chebyshev step with fused dots is 2.2x slower
// there (0.361 -> 0.803 ms) and keeps 4.
template <typename T>
struct MinBlocksLean {
  static constexpr int value = sizeof(T) == 4 ? 5 : 1;
};

template <typename T>
struct Wv {
  T sx, sy, sz, sd;
  __device__ __forceinline__ explicit Wv(const Geom &g) {
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

// Neighbour data of a slot at plane k.
template <typename T>
struct Nb {
  V4<T> c;   // centre values
  T l, r;    // x-neighbours of element 0 (i4-1) and element 3 (i4+4)
  V4<T> ys;  // sum of the y-neighbours that are interior nodes (difference form: (c - s) + (c - n))
  V4<T> zs;  // sum of the z-neighbours that are interior nodes (difference form: (c - d) + (c - u))
  bool jkb;  // the slot's row or plane is on the boundary
};

// Stencil input read from one array.
template <typename T>
struct ArraySrc {
  const T *__restrict__ x;
  __device__ __forceinline__ V4<T> v4(long long n) const { return ld4(x + n); }
  __device__ __forceinline__ T s(long long n) const { return x[n]; }
};

// Stencil input p = z + bb * q formed on the fly (the first CG iteration,
// p = z, marches z itself through ArraySrc: no load here tests for it).
template <typename T>
struct AxpySrc {
  const T *__restrict__ z;
  const T *__restrict__ q;
  T bb;
  __device__ __forceinline__ V4<T> v4(long long n) const {
    const V4<T> a = ld4(z + n), b = ld4(q + n);
    return V4<T>{fma(bb, b.x, a.x), fma(bb, b.y, a.y), fma(bb, b.z, a.z), fma(bb, b.w, a.w)};
  }
  __device__ __forceinline__ T s(long long n) const { return fma(bb, q[n], z[n]); }
};

// Loads everything but the z-window for plane k; shuffles need all lanes.
// DIFF: ys holds the difference form (c - s) + (c - n) of the y-part, with
// neighbours that are boundary nodes taken as 0 (see apply_diff_el).
template <int DIM, typename T, class Src, bool DIFF = false>
__device__ __forceinline__ void load_xy(const Geom &g, const SlotPos &p, const Src &x, long long n, const V4<T> &c,
                                        Nb<T> &nb) {
  const int lane = threadIdx.x & 31;
  T l = __shfl_up_sync(0xffffffffu, c.w, 1);
  T r = __shfl_down_sync(0xffffffffu, c.x, 1);
  if (lane == 0) l = (p.in && p.i4 > 0) ? x.s(n - 1) : T(0);
  if (lane == 31) r = (p.in && p.i4 + 4 < g.mx) ? x.s(n + 4) : T(0);
  nb.c = c;
  nb.l = l;
  nb.r = r;
  if (DIM >= 2) {
    const bool hs = p.j - 1 > 0, hn = p.j + 1 < g.my - 1;
    V4<T> s4 = (p.in && hs) ? x.v4(n - g.pitch) : zero4<T>();
    V4<T> n4 = (p.in && hn) ? x.v4(n + g.pitch) : zero4<T>();
    nb.ys = DIFF ? dsum4(c, s4, n4) : add4(s4, n4);
  } else {
    nb.ys = zero4<T>();
  }
}

// b - A x at element e (A: the Jacobian, boundary rows diagonal, boundary
// columns eliminated); `bd` true for a boundary node.  Padding points are
// not evaluated by the callers.
template <int DIM, typename T>
__device__ __forceinline__ T resid_el(const Geom &g, const Wv<T> &w, const Nb<T> &nb, int e, int i, bool jkb, T bv) {
  const T xc = el(nb.c, e);
  const bool bd = jkb || i == 0 || i == g.mx - 1;
  if (bd) return fma(-w.sd, xc, bv);
  const T xl = e == 0 ? nb.l : el(nb.c, e - 1);
  const T xr = e == 3 ? nb.r : el(nb.c, e + 1);
  const T a = (i - 1 > 0 ? xl : T(0)) + (i + 1 < g.mx - 1 ? xr : T(0));
  T s = fma(w.sx, a, bv);
  if (DIM >= 2) s = fma(w.sy, el(nb.ys, e), s);
  if (DIM >= 3) s = fma(w.sz, el(nb.zs, e), s);
  return fma(-w.sd, xc, s);
}

// (A x) at element e in difference form, from neighbour data assembled with
// DIFF: interior rows sum_d sc_d ((x - x_-) + (x - x_+)) with neighbours on the
// boundary taken as 0, which is A x exactly because scdiag = 2 sum_d sc_d.
// For the smooth vectors of an inner Krylov solve the differences of nearby
// values are exact in FP32, so the rounding error is of the order eps * h
// |grad x| instead of eps * scdiag |x|: the FP32 apply keeps its accuracy
// when the result is small against its terms (a smooth x, whose A x cancels
// to O(h^2) of them).  Boundary rows: scdiag x.
template <int DIM, typename T>
__device__ __forceinline__ T apply_diff_el(const Geom &g, const Wv<T> &w, const Nb<T> &nb, int e, int i, bool jkb) {
  const T xc = el(nb.c, e);
  if (jkb || i == 0 || i == g.mx - 1) return w.sd * xc;
  const T xl = e == 0 ? nb.l : el(nb.c, e - 1);
  const T xr = e == 3 ? nb.r : el(nb.c, e + 1);
  const T a = (xc - (i - 1 > 0 ? xl : T(0))) + (xc - (i + 1 < g.mx - 1 ? xr : T(0)));
  T s = w.sx * a;
  if (DIM >= 2) s = fma(w.sy, el(nb.ys, e), s);
  if (DIM >= 3) s = fma(w.sz, el(nb.zs, e), s);
  return s;
}

__device__ __forceinline__ bool ksp_done_v(const KspState *st) { return st && __ldcg(&st->done); }

// The KSP state a block works for: the whole grid's, or its plane's in a batch.
__device__ __forceinline__ KspState *block_state(KspState *st, const Slots &s) {
  if (!st || !s.batch) return st;
  return st + blockIdx.x / s.nchunk;
}

// Batched form of reduce_and_finalize: sum over the blocks of one plane
// (tickets and the finaliser are per plane).  Not inlined, so that the
// register allocation of the single-grid stencils does not carry it.
template <int NV>
__device__ __noinline__ void reduce_planes(double (&v)[NV], Reducer red, int slot, KspState *st, Fin fin,
                                           double *out, int nchunk) {
  __shared__ bool am_last;
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  const int plane = blockIdx.x / nchunk, first = plane * nchunk, nb = nchunk;
  block_sum<NV>(v);
  unsigned int *ticket = red.tickets + (size_t)slot * red.tcap + plane;
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) red.partials[(slot * NV + q) * red.cap + blockIdx.x] = v[q];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == (unsigned)(nb - 1));
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double sum[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) {
    sum[q] = 0.0;
    for (int b = tid; b < nb; b += nt) sum[q] += __ldcg(&red.partials[(slot * NV + q) * red.cap + first + b]);
  }
  block_sum<NV>(sum);
  if (tid == 0) {
    *ticket = 0u;
    if (st || fin == FIN_STORE) ksp_finalize(st, fin, sum, NV, out ? out + plane * NV : nullptr);
  }
}

// Sum over the blocks of a launch (or, for a batch, over the blocks of one
// plane) and run `fin`.
template <int NV>
__device__ __forceinline__ void reduce_slots(double (&v)[NV], Reducer red, int slot, KspState *st, Fin fin,
                                             double *out, const Slots &s) {
  if (!s.batch) reduce_and_finalize<NV>(v, red, slot, st, fin, out);
  else reduce_planes<NV>(v, red, slot, st, fin, out, s.nchunk);
}

// The same with the batch flag fixed at compile time: the stencil kernels
// that reduce are instantiated twice, so the single-grid form carries no
// per-plane code (a runtime branch there cost registers and spills in the
// z-march).
template <int NV, bool PL>
__device__ __forceinline__ void reduce_sel(double (&v)[NV], Reducer red, int slot, KspState *st, Fin fin,
                                           double *out, const Slots &s) {
  if constexpr (PL) reduce_planes<NV>(v, red, slot, st, fin, out, s.nchunk);
  else reduce_and_finalize<NV>(v, red, slot, st, fin, out);
}

template <bool PL>
__device__ __forceinline__ KspState *block_state_sel(KspState *st, const Slots &s) {
  if constexpr (PL) return st ? st + blockIdx.x / s.nchunk : st;
  else return st;
}

// Generic z-march over the slot's planes.  `Op` is called once per plane
// with (k, n, nb) after the neighbour data is assembled; it performs its own
// loads/stores of other arrays at n.  `x` is the stencil input.
__device__ __forceinline__ bool jk_bdry(const Geom &g, int dim, int j, int k) {
  return (dim >= 2 && (j == 0 || j == g.my - 1)) || (dim >= 3 && (k == 0 || k == g.mz - 1));
}

// 2D row march (s.ry rows of one x-slot): the same neighbour data as the
// plain form, the y-neighbour rows from the register window instead of
// loads, in the plain form's order (south + north).  Every thread runs ry
// steps (the shuffles need all lanes); rows past the grid are skipped.
template <typename T, bool DIFF, class Op, class Src>
__device__ __forceinline__ void march_rows(const Geom &g, const Slots &s, const SlotPos &p, const Src &x, Op &op) {
  const int lane = threadIdx.x & 31;
  const long long base = (long long)p.k0 * g.plane + p.i4;
  V4<T> xs = zero4<T>(), xc = zero4<T>();
  if (p.in && p.j - 1 >= 0) xs = x.v4(base + (long long)(p.j - 1) * g.pitch);
  if (p.in && p.j < g.my) xc = x.v4(base + (long long)p.j * g.pitch);
  for (int t = 0; t < s.ry; t++) {
    const int j = p.j + t;
    const bool valid = p.in && j < g.my;
    const long long n = base + (long long)j * g.pitch;
    V4<T> xn = zero4<T>();
    if (valid && j + 1 < g.my) xn = x.v4(n + g.pitch);
    Nb<T> nb;
    T l = __shfl_up_sync(0xffffffffu, xc.w, 1);
    T r = __shfl_down_sync(0xffffffffu, xc.x, 1);
    if (lane == 0) l = (valid && p.i4 > 0) ? x.s(n - 1) : T(0);
    if (lane == 31) r = (valid && p.i4 + 4 < g.mx) ? x.s(n + 4) : T(0);
    nb.c = xc;
    nb.l = l;
    nb.r = r;
    const bool hs = j - 1 > 0, hn = j + 1 < g.my - 1;
    nb.ys = DIFF ? dsum4(xc, hs ? xs : zero4<T>(), hn ? xn : zero4<T>())
                 : add4(hs ? xs : zero4<T>(), hn ? xn : zero4<T>());
    nb.zs = zero4<T>();
    nb.jkb = j == 0 || j == g.my - 1;
    if (valid) op(p.k0, n, nb);
    xs = xc;
    xc = xn;
  }
}

// DIFF: the y- and z-sums of the neighbour data in difference form (load_xy)
template <int DIM, typename T, bool DIFF, class Op, class Src>
__device__ __forceinline__ void march_core(const Geom &g, const Slots &s, const SlotPos &p, const Src &x, Op &op) {
  if constexpr (DIM == 2) {
    if (s.ry) {
      march_rows<T, DIFF>(g, s, p, x, op);
      return;
    }
  }
  V4<T> zd = zero4<T>(), zc = zero4<T>();
  if (p.in) {
    if (DIM >= 3 && p.k0 > 0) zd = x.v4((long long)(p.k0 - 1) * g.plane + p.col);
    zc = x.v4((long long)p.k0 * g.plane + p.col);
  }
  long long n = (long long)p.k0 * g.plane + p.col;  // advanced by a plane per step
  for (int k = p.k0; k < p.k1; k++, n += g.plane) {
    V4<T> zu = zero4<T>();
    if (DIM >= 3 && p.in && k + 1 < g.mz) zu = x.v4(n + g.plane);
    Nb<T> nb;
    load_xy<DIM, T, Src, DIFF>(g, p, x, n, zc, nb);
    if (DIM >= 3) {
      const bool hd = k - 1 > 0, hu = k + 1 < g.mz - 1;
      nb.zs = DIFF ? dsum4(zc, hd ? zd : zero4<T>(), hu ? zu : zero4<T>())
                   : add4(hd ? zd : zero4<T>(), hu ? zu : zero4<T>());
    } else {
      nb.zs = zero4<T>();
    }
    nb.jkb = jk_bdry(g, DIM, p.j, k);
    if (p.in) op(k, n, nb);
    zd = zc;
    zc = zu;
  }
}

template <int DIM, typename T, class Op, class Src>
__device__ __forceinline__ void march_src(const Geom &g, const Slots &s, const SlotPos &p, const Src &x, Op &op) {
  march_core<DIM, T, false>(g, s, p, x, op);
}

template <int DIM, typename T, class Op>
__device__ __forceinline__ void march(const Geom &g, const Slots &s, const SlotPos &p, const T *__restrict__ x,
                                      Op &op) {
  march_src<DIM, T>(g, s, p, ArraySrc<T>{x}, op);
}



// ------------------------------------------------------------------ stencil ops
// out = ckm1*xkm1 + ck*xk + crd*(b - A xk)   (Chebyshev / Richardson step)
// HAS_KM1=false drops the xkm1 term.  out must not alias any input (the
// smoother rotates three buffers per level).
// DOTS: also reduces out.out and out.b (the preconditioned residual's z.z and
// z.r when this is the last smoothing step on the finest level) and runs `fin`.
template <int DIM, typename T, bool HAS_KM1, bool DOTS = false, bool PL = false>
__global__ void __launch_bounds__(256, ((DOTS || HAS_KM1) ? MinBlocks<T>::value : MinBlocksLean<T>::value)) v_cheb(Geom g, Slots s, KspState *st, const T *__restrict__ b,
                                              const T *__restrict__ xkm1, const T *__restrict__ xk,
                                              T *__restrict__ out, T ckm1, T ck, T crd, Reducer red = Reducer{},
                                              int slot = 0, Fin fin = FIN_STORE) {
  st = DOTS ? block_state_sel<PL>(st, s) : block_state(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos_st<DIM>(g, s);
  const Wv<T> w(g);
  T zz = T(0), zr = T(0);
  auto op = [&](int k, long long n, const Nb<T> &nb) {
    const V4<T> bv = ld4(b + n);
    V4<T> km = HAS_KM1 ? ld4(xkm1 + n) : zero4<T>();
    const bool jkb = nb.jkb;
    V4<T> o;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int i = p.i4 + e;
      T v = T(0);
      if (i < g.mx) {
        const T r = resid_el<DIM, T>(g, w, nb, e, i, jkb, el(bv, e));
        T base = ck * el(nb.c, e);
        if (HAS_KM1) base = fma(ckm1, el(km, e), base);
        v = fma(crd, r, base);
        if (DOTS) {
          zz = fma(v, v, zz);
          zr = fma(v, el(bv, e), zr);
        }
      }
      set_el(o, e, v);
    }
    st4(out + n, o);
  };
  march<DIM, T>(g, s, p, xk, op);
  if (DOTS) {
    double v2[2] = {(double)zz, (double)zr};
    reduce_sel<2, PL>(v2, red, slot, st, fin, nullptr, s);
  }
}

// Two Chebyshev steps from a zero iterate in one pass over b:
//   x1 = c1 b,  x2 = omega x1 + omega c1 (b - A x1) = a0 b - a1 (A b)
// with a0 = 2 omega c1, a1 = omega c1^2 (c1 = scale/scdiag).
// RUPD (the finest level of a CG iteration's V-cycle): b is the CG residual
// after this iteration's update, r_new = r - alpha w, formed on the fly from
// r (`b`) and w exactly as v_cg_r forms it and stored to rnew (another
// buffer: neighbours still read r); RR: r_new.r_new reduced as v_cg_r
// reduces it (same slots, same order) and finalised as FIN_RR.  Replaces
// v_cg_r + v_cheb2_zero, bit-identical.
template <int DIM, typename T, bool RUPD = false, bool RR = false>
__global__ void __launch_bounds__(256, MinBlocksLean<T>::value) v_cheb2_zero(Geom g, Slots s, KspState *st, const T *__restrict__ b,
                                                    T *__restrict__ out, T a0, T a1,
                                                    const T *__restrict__ wv = nullptr, T *__restrict__ rnew = nullptr,
                                                    Reducer red = Reducer{}, int slot = 0) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos_st<DIM>(g, s);
  const Wv<T> w(g);
  T acc = T(0);
  auto op = [&](int k, long long n, const Nb<T> &nb) {
    const bool jkb = nb.jkb;
    V4<T> o;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int i = p.i4 + e;
      T v = T(0);
      if (i < g.mx) {
        // -(A b) = (0 - A b): resid_el with bv = 0
        const T mab = resid_el<DIM, T>(g, w, nb, e, i, jkb, T(0));
        v = fma(a1, mab, a0 * el(nb.c, e));
      }
      set_el(o, e, v);
    }
    st4(out + n, o);
    if constexpr (RUPD) {
      const V4<T> &rn = nb.c;
      st4(rnew + n, rn);
      if (RR) acc = fma(rn.x, rn.x, fma(rn.y, rn.y, fma(rn.z, rn.z, fma(rn.w, rn.w, acc))));
    }
  };
  if constexpr (RUPD) {
    const T a = st ? (T)st->alpha : T(0);  // no state: alpha = 0
    march_src<DIM, T>(g, s, p, AxpySrc<T>{b, wv, -a}, op);
    if (RR) {
      double v1[1] = {(double)acc};
      reduce_slots<1>(v1, red, slot, st, FIN_RR, nullptr, s);
    }
  } else {
    march<DIM, T>(g, s, p, b, op);
  }
}

// r = b - A x; NORM: r.r reduced into *out as v_dots(r, r) reduces it (same
// per-thread order over the slot's planes, same block order)
template <int DIM, typename T, bool NORM = false>
__global__ void __launch_bounds__(256, (NORM ? MinBlocks<T>::value : MinBlocksLean<T>::value)) v_resid(Geom g, Slots s, KspState *st, const T *__restrict__ b,
                                               const T *__restrict__ x, T *__restrict__ r, Reducer red = Reducer{},
                                               int slot = 0, double *out = nullptr) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos_st<DIM>(g, s);
  const Wv<T> w(g);
  T rr = T(0);
  auto op = [&](int k, long long n, const Nb<T> &nb) {
    const V4<T> bv = ld4(b + n);
    const bool jkb = nb.jkb;
    V4<T> o;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int i = p.i4 + e;
      set_el(o, e, i < g.mx ? resid_el<DIM, T>(g, w, nb, e, i, jkb, el(bv, e)) : T(0));
    }
    st4(r + n, o);
    if (NORM) rr = fma(o.x, o.x, fma(o.y, o.y, fma(o.z, o.z, fma(o.w, o.w, rr))));
  };
  march<DIM, T>(g, s, p, x, op);
  if (NORM) {
    double v1[1] = {(double)rr};
    reduce_sel<1, false>(v1, red, slot, nullptr, FIN_STORE, out, s);
  }
}


// w = A p; p.w reduced (per-thread partials in T, blocks in FP64)
template <int DIM, typename T>
__global__ void __launch_bounds__(256, MinBlocks<T>::value) v_apply_dot(Geom g, Slots s, KspState *st, const T *__restrict__ pv,
                                                   T *__restrict__ wv, Reducer red, int slot, Fin fin,
                                                   double *out) {
  st = block_state_sel<false>(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos_st<DIM>(g, s);
  const Wv<T> w(g);
  T acc = T(0);
  auto op = [&](int k, long long n, const Nb<T> &nb) {
    const bool jkb = nb.jkb;
    V4<T> o;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int i = p.i4 + e;
      T v = T(0);
      if (i < g.mx) {
        v = -resid_el<DIM, T>(g, w, nb, e, i, jkb, T(0));
        acc = fma(el(nb.c, e), v, acc);
      }
      set_el(o, e, v);
    }
    st4(wv + n, o);
  };
  march<DIM, T>(g, s, p, pv, op);
  double v1[1] = {(double)acc};
  reduce_sel<1, false>(v1, red, slot, st, fin, out, s);
}

// p_new = z + (beta/betaold) p_old (p_new = z on the first CG iteration),
// w = A p_new, p_new.w reduced: the CG direction update fused into the apply.
// p_old and p_new are different buffers (neighbours read p_old).  The
// solution update of the previous iteration, y += alpha p_old, is deferred
// to here (the state's `pend`): this kernel reads p_old anyway, so the
// update costs y's read and write only, and v_cg_r no longer reads p and y.
// alpha is still the previous iteration's: FIN_PW replaces it only after
// every block has finished.
// ACC (FP32 inner solves of the mixed form): w = A p in difference form
// (apply_diff_el) and the solution update in FP64 straight into the outer
// solution, y64 += (yscale * alpha) p_old (the state's yscale and yfresh), so
// that neither the apply nor the FP32 storage of the correction limits the
// true residual an inner solve reaches to ~kappa * 2^-24.
// YM (the ACC form's y updates in pairs): 1 leaves y alone and keeps the owed
// update (FIN_PW_DEFER); 2 applies both owed updates, the older one first,
// y = fma(a, p_old, fma(a2, p_older, y)) -- the values of applying them one
// per iteration, as the FP64 intermediate is what y would have held.  The
// older direction is in the buffer this launch overwrites with p_new: each
// thread reads it at its own points before its store, and no other thread
// reads it.  Iterations alternate 1, 2 (the graphs' parity), so y moves
// every other iteration: 16 + 36 instead of 2 x 32 bytes per node.
// float -> double on the integer pipe (bitconv.cuh: the cast's value)
template <typename YT, typename T>
__device__ __forceinline__ YT to_y(T v) {
  if constexpr (sizeof(YT) == 8 && sizeof(T) == 4) return f2d_bits(v);
  else return (YT)v;
}

template <typename T, bool ACC>
struct CgY {
  using type = T;
};
template <typename T>
struct CgY<T, true> {
  using type = double;
};

template <int DIM, typename T, bool PL = false, bool ACC = false, int YM = 0>
__global__ void __launch_bounds__(256, MinBlocksLean<T>::value) v_cgp_apply(Geom g, Slots s, KspState *st, const T *__restrict__ z,
                                                   const T *__restrict__ pold, T *__restrict__ pnew,
                                                   T *__restrict__ wv, typename CgY<T, ACC>::type *__restrict__ y,
                                                   Reducer red, int slot) {
  using YT = typename CgY<T, ACC>::type;
  static_assert(YM == 0 || (ACC && !PL), "paired y updates: the accurate form of one grid");
  st = block_state_sel<PL>(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos_st<DIM>(g, s);
  const Wv<T> w(g);
  const bool first = !st || st->i == 0;  // no state: p = z
  const bool pend = YM != 1 && st && st->pend && y;
  const bool pend2 = YM == 2 && pend && st->pend2;
  const YT a2 = pend2 ? (YT)(st->yscale * st->alpha2) : YT(0);
  // no update has reached y yet (it is not zero-filled); ACC: nor has an
  // earlier refinement step
  const bool yfresh = pend && st->i == 1 && (!ACC || st->yfresh);
  const YT a = pend ? (ACC ? (YT)(st->yscale * st->alpha) : (YT)st->alpha) : YT(0);
  T acc = T(0);
  auto op = [&](int k, long long n, const Nb<T> &nb) {
    const bool jkb = nb.jkb;
    V4<T> o;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int i = p.i4 + e;
      T v = T(0);
      if (i < g.mx) {
        if constexpr (ACC) v = apply_diff_el<DIM, T>(g, w, nb, e, i, jkb);
        else v = -resid_el<DIM, T>(g, w, nb, e, i, jkb, T(0));
        acc = fma(el(nb.c, e), v, acc);
      }
      set_el(o, e, v);
    }
    if (pend) {  // the first update (iteration 1) starts y from 0 without reading it
      const V4<T> pp = ld4(pold + n);
      V4<YT> yy = yfresh ? zero4<YT>() : ld4(y + n);
      if (pend2) {  // the older direction, read before p_new replaces it
        const V4<T> qq = ld4(pnew + n);
        yy = V4<YT>{fma(a2, to_y<YT>(qq.x), yy.x), fma(a2, to_y<YT>(qq.y), yy.y), fma(a2, to_y<YT>(qq.z), yy.z),
                    fma(a2, to_y<YT>(qq.w), yy.w)};
      }
      st4(y + n, V4<YT>{fma(a, to_y<YT>(pp.x), yy.x), fma(a, to_y<YT>(pp.y), yy.y), fma(a, to_y<YT>(pp.z), yy.z),
                        fma(a, to_y<YT>(pp.w), yy.w)});
    }
    st4(pnew + n, nb.c);
    st4(wv + n, o);
  };
  // the first iteration (p = z) and the others (p = z + beta/betaold p_old)
  // march separately, so that no load of the common case tests `first`
  if (first) march_core<DIM, T, ACC>(g, s, p, ArraySrc<T>{z}, op);
  else march_core<DIM, T, ACC>(g, s, p, AxpySrc<T>{z, pold, (T)st->bratio}, op);
  double v1[1] = {(double)acc};
  reduce_sel<1, PL>(v1, red, slot, st, YM == 1 ? FIN_PW_DEFER : FIN_PW, nullptr, s);
}

// The accurate form of v_cgp_apply (3D, FP32, one grid) fed by a TMA ring.
// A block owns a tile of 43 slots (172 points) by 8 rows and a chunk of
// planes.  Its producer warp streams each plane's tile of z and p_old (with
// one row and one slot of halo on every side) and of y64 (the tile alone)
// into a 3-stage shared-memory ring with bulk tensor copies; eleven consumer
// warps (one thread per slot of the tile) form p = z + beta/betaold p_old for
// their slot and its x- and y-neighbours from the ring, keep p of planes
// k-1, k, k+1 of their slot in registers, and write p, w = A p (difference
// form) and the deferred y64 += (yscale alpha) p_old, summing p.w.  No
// consumer reads shared memory another consumer wrote, so the warps never
// wait for one another: only for their planes to arrive.  Every value of p,
// w and y64 is the same operation on the same operands as in v_cgp_apply;
// p.w is summed in another order (other blocks).
struct CgTile {
  int ntx, nty, nzt, zc;  // x-tiles (43 slots), y-tiles (8 rows), plane chunks, planes per chunk
  unsigned blocks() const { return (unsigned)ntx * (unsigned)nty * (unsigned)nzt; }
};

inline CgTile cg_tile_shape(const Geom &g, int zc = 32) {
  CgTile q;
  q.ntx = (g.pitch / 4 + 42) / 43;
  q.nty = (g.my + 7) / 8;
  q.zc = zc < g.mz ? zc : g.mz;
  q.nzt = (g.mz + q.zc - 1) / q.zc;
  return q;
}

struct CgRing {
  static constexpr int NS = 3;
  static constexpr int SL = 43, RY = 8;         // slots and rows of a tile
  static constexpr int ZW = 180, ZR = 10;       // z, p_old box: points 172 tx - 4 .. + 179, rows j0 - 1 .. j0 + 8
  static constexpr int YW = 172, YR = 8;        // y64 box: points 172 tx .. + 171, rows j0 .. j0 + 7
  static constexpr unsigned ZBYTES = ZW * ZR * 4, YBYTES = YW * YR * 8;
  static constexpr unsigned ZSTR = (ZBYTES + 127) / 128 * 128, YSTR = (YBYTES + 127) / 128 * 128;
  static constexpr unsigned STAGE = 2 * ZSTR + YSTR;
  static constexpr int CONSUMERS = 11, THREADS = 32 * (CONSUMERS + 1);
  static constexpr size_t SMEM = 128 + NS * STAGE + 2 * NS * sizeof(uint64_t);
};

static __global__ void __launch_bounds__(CgRing::THREADS, 2)
    v_cgp_apply_tma(const __grid_constant__ CUtensorMap zmap, const __grid_constant__ CUtensorMap pmap,
                    const __grid_constant__ CUtensorMap ymap, Geom g, CgTile q, KspState *st,
                    float *__restrict__ pnew, float *__restrict__ wv, double *__restrict__ y, Reducer red, int slot,
                    int *fault) {
  using R = CgRing;
  if (ksp_done_v(st)) return;
  extern __shared__ unsigned char cg_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(cg_raw) + 127) & ~uintptr_t(127));
  uint64_t *full = reinterpret_cast<uint64_t *>(base + R::NS * R::STAGE), *empty = full + R::NS;
  auto zs = [&](int s) { return reinterpret_cast<const float *>(base + s * R::STAGE); };
  auto ps = [&](int s) { return reinterpret_cast<const float *>(base + s * R::STAGE + R::ZSTR); };
  auto ys = [&](int s) { return reinterpret_cast<const double *>(base + s * R::STAGE + 2 * R::ZSTR); };
  const bool first = !st || st->i == 0;  // p = z
  const bool pend = st && st->pend;
  const bool yfresh = pend && st->i == 1 && st->yfresh;  // y64 written without reading
  const bool yread = pend && !yfresh;
  const double a = pend ? st->yscale * st->alpha : 0.0;
  const float bb = first ? 0.f : (float)st->bratio;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tx = blockIdx.x % q.ntx, tr = blockIdx.x / q.ntx, ty = tr % q.nty, tz = tr / q.nty;
  const int k0 = tz * q.zc, k1 = min(k0 + q.zc, g.mz);
  const int nq = k1 - k0 + 2;  // ring planes k0 - 1 .. k1
  if (threadIdx.x == 0) {
    for (int s = 0; s < R::NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], R::CONSUMERS);
    }
    mbar_init_fence();
  }
  __syncthreads();
  float acc = 0.f;
  if (warp == R::CONSUMERS) {  // producer
    if (lane == 0) {
      for (int qq = 0; qq < nq; qq++) {
        const int s = qq % R::NS, u = qq / R::NS;
        if (u > 0) mbar_wait(&empty[s], (u - 1) & 1, fault);
        const int pl = k0 - 1 + qq;
        const bool yl = yread && pl >= k0 && pl < k1;
        mbar_arrive_tx(&full[s], R::ZBYTES + (first ? 0u : R::ZBYTES) + (yl ? R::YBYTES : 0u));
        tma_load_3d(base + s * R::STAGE, &zmap, 172 * tx - 4, 8 * ty - 1, pl, &full[s]);
        if (!first) tma_load_3d(base + s * R::STAGE + R::ZSTR, &pmap, 172 * tx - 4, 8 * ty - 1, pl, &full[s]);
        if (yl) tma_load_3d(base + s * R::STAGE + 2 * R::ZSTR, &ymap, 172 * tx, 8 * ty, pl, &full[s]);
      }
      for (int qq = max(0, nq - R::NS); qq < nq; qq++) mbar_wait(&full[qq % R::NS], (qq / R::NS) & 1, fault, true);
    }
  } else {  // consumers: thread t owns slot t % 43 of tile row t / 43
    const int t = threadIdx.x, row = t / R::SL, sl = t - R::SL * (t / R::SL);
    const int j = 8 * ty + row, i4 = 4 * (R::SL * tx + sl);
    const bool act = t < R::SL * R::RY && j < g.my && i4 < g.pitch;
    const int zr = (row + 1) * R::ZW + 4 * sl + 4;  // ring offset of the slot's element 0
    const bool hs = j - 1 > 0, hn = j + 1 < g.my - 1;
    const Wv<float> w(g);
    auto pv4 = [&](int s, int off) -> V4<float> {  // p = z + bb p_old (p = z on the first iteration)
      const V4<float> zz = *reinterpret_cast<const V4<float> *>(zs(s) + off);
      if (first) return zz;
      const V4<float> pp = *reinterpret_cast<const V4<float> *>(ps(s) + off);
      return V4<float>{fmaf(bb, pp.x, zz.x), fmaf(bb, pp.y, zz.y), fmaf(bb, pp.z, zz.z), fmaf(bb, pp.w, zz.w)};
    };
    auto pv1 = [&](int s, int off) -> float { return first ? zs(s)[off] : fmaf(bb, ps(s)[off], zs(s)[off]); };
    mbar_wait(&full[0], 0, fault);  // planes k0 - 1 and k0
    mbar_wait(&full[1], 0, fault);
    V4<float> pd = (act && k0 > 0) ? pv4(0, zr) : zero4<float>();
    V4<float> pc = act ? pv4(1, zr) : zero4<float>();
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[0]);  // plane k0 - 1 is no longer read
    for (int k = k0; k < k1; k++) {
      const int qq = k - k0 + 1, sc = qq % R::NS, su = (qq + 1) % R::NS;
      mbar_wait(&full[su], ((qq + 1) / R::NS) & 1, fault);
      const V4<float> pu = (act && k + 1 < g.mz) ? pv4(su, zr) : zero4<float>();
      if (act) {
        Nb<float> nb;
        nb.c = pc;
        nb.l = pv1(sc, zr - 1);
        nb.r = pv1(sc, zr + 4);
        nb.ys = dsum4(pc, hs ? pv4(sc, zr - R::ZW) : zero4<float>(), hn ? pv4(sc, zr + R::ZW) : zero4<float>());
        const bool hd = k - 1 > 0, hu = k + 1 < g.mz - 1;
        nb.zs = dsum4(pc, hd ? pd : zero4<float>(), hu ? pu : zero4<float>());
        nb.jkb = jk_bdry(g, 3, j, k);
        V4<float> o;
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const int i = i4 + e;
          float v = 0.f;
          if (i < g.mx) {
            v = apply_diff_el<3, float>(g, w, nb, e, i, nb.jkb);
            acc = fmaf(el(pc, e), v, acc);
          }
          set_el(o, e, v);
        }
        const long long n = (long long)k * g.plane + (long long)j * g.pitch + i4;
        st4(pnew + n, pc);
        st4(wv + n, o);
        if (pend) {
          const V4<float> pp = *reinterpret_cast<const V4<float> *>(ps(sc) + zr);
          const V4<double> yy =
              yfresh ? zero4<double>() : *reinterpret_cast<const V4<double> *>(ys(sc) + row * R::YW + 4 * sl);
          st4(y + n, V4<double>{fma(a, f2d_bits(pp.x), yy.x), fma(a, f2d_bits(pp.y), yy.y), fma(a, f2d_bits(pp.z), yy.z),
                                fma(a, f2d_bits(pp.w), yy.w)});
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[sc]);  // plane k is no longer read
      pd = pc;
      pc = pu;
    }
  }
  double v1[1] = {(double)acc};
  reduce_and_finalize<1>(v1, red, slot, st, FIN_PW, nullptr);
}

// ------------------------------------------------------------------ temporally blocked smoothing
// Two Chebyshev steps from a nonzero iterate in one pass (3D, FP32):
//   x1 = x0 + c1 (b - A x0)
//   x2 = ckm1 x0 + ck x1 + crd (b - A x1)
// (the post-smoothing of a V-cycle level), reading x0 and b once and writing
// x2 only: 3 arrays instead of the 7 of two separate steps.  The arithmetic
// of every point is that of v_cheb (same operations in the same order), so
// x2 is bit-identical to the two-kernel form; DOTS reduces x2.x2 and x2.b as
// the last v_cheb step of the finest level does.  Measured at 513^3 it is
// slower than the two v_cheb launches (0.92 ms against 0.34 + 0.36 ms: one
// block of ~900 threads per SM, a barrier per plane and 64 registers leave
// the loads' latency exposed), so the solver uses it only on request
// (-fsh_fuse_smooth 1).
__device__ __forceinline__ float f4e(const float4 &v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
__device__ __forceinline__ void f4set(float4 &v, int e, float a) {
  if (e == 0) v.x = a; else if (e == 1) v.y = a; else if (e == 2) v.z = a; else v.w = a;
}

// b - A x for the 4 points of one slot from preloaded neighbours: c (the
// slot), xl / xr (the points left of element 0 and right of element 3), ys / zs
// (y and z neighbour slots, already masked to interior neighbours and summed in
// the order of load_xy / march_src).  The operations of resid_el, in order.
__device__ __forceinline__ float4 resid4(const Wv<float> &w, const Geom &g, int i4, bool jkb, const float4 &c,
                                         float xl, float xr, const float4 &ys, const float4 &zs, const float4 &bv) {
  float4 o;
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int i = i4 + e;
    const float xc = f4e(c, e);
    float v;
    if (jkb || i == 0 || i == g.mx - 1) {
      v = fmaf(-w.sd, xc, f4e(bv, e));
    } else {
      const float l = e == 0 ? xl : f4e(c, e - 1);
      const float r = e == 3 ? xr : f4e(c, e + 1);
      const float a = (i - 1 > 0 ? l : 0.f) + (i + 1 < g.mx - 1 ? r : 0.f);
      float sm = fmaf(w.sx, a, f4e(bv, e));
      sm = fmaf(w.sy, f4e(ys, e), sm);
      sm = fmaf(w.sz, f4e(zs, e), sm);
      v = fmaf(-w.sd, xc, sm);
    }
    f4set(o, e, v);
  }
  return o;
}

// A block owns R full rows (all P4 slots of each) of a z-chunk plus one halo
// row above and below; a thread owns one slot of one of those R+2 rows and
// marches k keeping x0 (planes k..k+2), x1 (planes k-1..k+1) and b in
// registers.  Per plane it computes x1 at plane k+1 for its slot (x0's
// y-neighbours come from L1/L2 like v_cheb's), publishes it in a 3-plane
// shared ring, and after one barrier computes x2 at plane k for the R inner
// rows, taking x1's y-neighbours from the ring.  Threads of the halo rows
// compute x1 only.  Per point: x0 and b read, x2 written (3 arrays).
struct Post2Z {
  int R, P4, threads, nyb, zc, nz;
  size_t smem;
  bool ok() const { return R > 0; }
  unsigned blocks() const { return (unsigned)nyb * (unsigned)nz; }
};

inline Post2Z post2z_shape(const Geom &g, int min_blocks = 456) {
  Post2Z q{};
  q.P4 = g.pitch / 4;
  if (g.dim != 3 || q.P4 < 33 || g.my < 3 || g.mz < 3) return q;  // small levels: the two-step form
  int R = 1024 / q.P4 - 2;
  if (R > g.my) R = g.my;
  if (R < 2) return q;
  q.R = R;
  q.threads = ((R + 2) * q.P4 + 31) / 32 * 32;
  q.nyb = (g.my + R - 1) / R;
  int zc = (int)(((long long)q.nyb * g.mz) / (min_blocks > 0 ? min_blocks : 1));
  zc = zc < 4 ? 4 : zc > 64 ? 64 : zc;
  if (zc > g.mz) zc = g.mz;
  q.zc = zc;
  q.nz = (g.mz + zc - 1) / zc;
  q.smem = sizeof(float4) * 3 * (size_t)(R + 2) * q.P4;
  return q;
}

template <bool DOTS>
__global__ void __launch_bounds__(1024, 1) v_cheb_post2z(Geom g, Post2Z q, KspState *st, const float *__restrict__ b,
                                                       const float *__restrict__ x0, float *__restrict__ out,
                                                       float c1, float ckm1, float ck, float crd,
                                                       Reducer red = Reducer{}, int slot = 0, Fin fin = FIN_STORE) {
  if (ksp_done_v(st)) return;
  extern __shared__ float4 pz_smem[];  // [3][R+2][P4]: x1 of the block's rows, planes k-1..k+1
  const int t = threadIdx.x, lane = t & 31;
  const int rows = q.R + 2, plane_slots = rows * q.P4;
  const bool act = t < plane_slots;
  const int rho = act ? t / q.P4 : 0, sl = act ? t - rho * q.P4 : 0;  // row in the block (0 = halo), slot
  const int yb = blockIdx.x % q.nyb, zt = blockIdx.x / q.nyb;
  const int j = yb * q.R + rho - 1, i4 = 4 * sl;
  const int k0 = zt * q.zc, k1 = k0 + q.zc < g.mz ? k0 + q.zc : g.mz;
  const bool jin = act && j >= 0 && j < g.my;
  const bool inner = jin && rho >= 1 && rho <= q.R;                     // writes x2
  const bool hs = j - 1 > 0, hn = j + 1 < g.my - 1, jb = j == 0 || j == g.my - 1;
  const long long col = (long long)j * g.pitch + i4;
  const Wv<float> w(g);
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto ld = [&](const float *a, int kk) -> float4 {  // own slot of plane kk (0 outside the grid)
    if (!jin || kk < 0 || kk >= g.mz) return zero;
    return *reinterpret_cast<const float4 *>(a + (long long)kk * g.plane + col);
  };
  auto ldy = [&](int kk, int dj) -> float4 {  // x0 at row j+dj of plane kk, an interior neighbour
    return *reinterpret_cast<const float4 *>(x0 + (long long)kk * g.plane + col + (long long)dj * g.pitch);
  };
  auto add = [](const float4 &a, const float4 &c) { return make_float4(a.x + c.x, a.y + c.y, a.z + c.z, a.w + c.w); };
  // x-neighbours by shuffles (warp edges: the scalar beyond; row starts and ends
  // are boundary or padding points, whose neighbours are never used)
  auto xnb = [&](const float4 &c, const float *arr_plane, float &l, float &r) {
    l = __shfl_up_sync(0xffffffffu, c.w, 1);
    r = __shfl_down_sync(0xffffffffu, c.x, 1);
    if (lane == 0) l = (jin && i4 > 0 && arr_plane) ? arr_plane[col - 1] : 0.f;
    if (lane == 31) r = (jin && i4 + 4 < g.mx && arr_plane) ? arr_plane[col + 4] : 0.f;
  };
  auto ring = [&](int kk, int r) -> float4 & { return pz_smem[(((kk % 3) + 3) % 3 * rows + r) * q.P4 + sl]; };
  // x1 at plane kk for this slot from x0 planes kk-1, kk, kk+1 (xd, xc, xu)
  auto step1 = [&](int kk, const float4 &xd, const float4 &xc, const float4 &xu, const float4 &bv) -> float4 {
    float l, r;
    xnb(xc, (kk >= 0 && kk < g.mz) ? x0 + (long long)kk * g.plane : nullptr, l, r);
    float4 o = zero;
    if (jin && kk >= 0 && kk < g.mz && i4 < g.mx) {
      const float4 ys = add((hs ? ldy(kk, -1) : zero), (hn ? ldy(kk, 1) : zero));
      const float4 zs = add((kk - 1 > 0 ? xd : zero), (kk + 1 < g.mz - 1 ? xu : zero));
      const float4 rr = resid4(w, g, i4, jb || kk == 0 || kk == g.mz - 1, xc, l, r, ys, zs, bv);
#pragma unroll
      for (int e = 0; e < 4; e++) f4set(o, e, i4 + e < g.mx ? fmaf(c1, f4e(rr, e), 1.f * f4e(xc, e)) : 0.f);
    }
    return o;
  };
  // prologue: x1 at planes k0-1 (registers) and k0 (registers and ring)
  float4 xa = ld(x0, k0 - 2), xb = ld(x0, k0 - 1), xcur = ld(x0, k0), xn = ld(x0, k0 + 1);
  float4 x1d = step1(k0 - 1, xa, xb, xcur, ld(b, k0 - 1));
  float4 bk = ld(b, k0);
  float4 x1c = step1(k0, xb, xcur, xn, bk);
  if (act) ring(k0, rho) = x1c;
  // window: xcur = x0(k), xn = x0(k+1)
  float zz = 0.f, zr = 0.f;
  for (int k = k0; k < k1; k++) {
    const float4 xnn = ld(x0, k + 2);
    const float4 bn = ld(b, k + 1);
    const float4 x1n = step1(k + 1, xcur, xn, xnn, bn);
    if (act) ring(k + 1, rho) = x1n;
    __syncthreads();  // x1 planes k and k+1 of every row are in the ring
    // x2 = ckm1 x0 + ck x1 + crd (b - A x1) at plane k
    float l, r;
    {
      l = __shfl_up_sync(0xffffffffu, x1c.w, 1);
      r = __shfl_down_sync(0xffffffffu, x1c.x, 1);
      const float4 *rowp = pz_smem + ((((k % 3) + 3) % 3) * rows + rho) * q.P4;  // x1 plane k, this row
      if (lane == 0) l = (act && sl > 0) ? rowp[sl - 1].w : 0.f;
      if (lane == 31) r = (act && sl + 1 < q.P4) ? rowp[sl + 1].x : 0.f;
    }
    if (inner && i4 < g.pitch) {
      float4 o = zero;
      if (i4 < g.mx) {
        const float4 ys = add((hs ? ring(k, rho - 1) : zero), (hn ? ring(k, rho + 1) : zero));
        const float4 zs = add((k - 1 > 0 ? x1d : zero), (k + 1 < g.mz - 1 ? x1n : zero));
        const float4 rr = resid4(w, g, i4, jb || k == 0 || k == g.mz - 1, x1c, l, r, ys, zs, bk);
#pragma unroll
        for (int e = 0; e < 4; e++) {
          float v = 0.f;
          if (i4 + e < g.mx) {
            float base = ck * f4e(x1c, e);
            base = fmaf(ckm1, f4e(xcur, e), base);
            v = fmaf(crd, f4e(rr, e), base);
            if (DOTS) {
              zz = fmaf(v, v, zz);
              zr = fmaf(v, f4e(bk, e), zr);
            }
          }
          f4set(o, e, v);
        }
      }
      *reinterpret_cast<float4 *>(out + (long long)k * g.plane + col) = o;
    }
    x1d = x1c;
    x1c = x1n;
    xcur = xn;
    xn = xnn;
    bk = bn;
  }
  if (DOTS) {
    double v2[2] = {(double)zz, (double)zr};
    reduce_and_finalize<2>(v2, red, slot, st, fin, nullptr);
  }
}

// ------------------------------------------------------------------ grid transfers
// b_c = P^T r_f (full weighting; weights 1, 1/2 per offset and dimension).
// A thread owns a coarse slot (I4..I4+3) and marches coarse planes; the fine
// x-values 2I4-1 .. 2I4+7 come from two fine slots and a shuffle.
template <int DIM, typename T>
__device__ __forceinline__ V4<T> restrict_row(const Geom &gf, const T *__restrict__ rf, long long m, int I4, bool ok) {
  // fine row values at 2I-1, 2I, 2I+1 weighted (1/2, 1, 1/2) for I = I4..I4+3
  const int lane = threadIdx.x & 31;
  const int fi = 2 * I4;
  V4<T> A = zero4<T>(), B = zero4<T>();
  if (ok) {
    A = ld4(rf + m);
    if (fi + 4 < gf.pitch) B = ld4(rf + m + 4);
  }
  T L = __shfl_up_sync(0xffffffffu, B.w, 1);
  if (lane == 0) L = (ok && fi > 0) ? rf[m - 1] : T(0);
  if (fi == 0) L = T(0);
  const T h = T(0.5);
  return V4<T>{fma(h, L + A.y, A.x), fma(h, A.y + A.w, A.z), fma(h, A.w + B.y, B.x), fma(h, B.y + B.w, B.z)};
}

template <int DIM, typename T>
__global__ void __launch_bounds__(256) v_restrict(Geom gf, Geom g, Slots s, KspState *st, const T *__restrict__ rf,
                                                  T *__restrict__ bc) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos(g, s);
  const T h = T(0.5);
  // fine row offset of fine row fj, plane fk
  auto rowsum = [&](int fk) -> V4<T> {  // sum over fj = 2J-1..2J+1 with weights (1/2,1,1/2)
    const long long base = (long long)fk * gf.plane + 2LL * p.i4;
    const int fj = 2 * p.j;
    V4<T> c = restrict_row<DIM, T>(gf, rf, base + (long long)fj * gf.pitch, p.i4, p.in);
    if (DIM < 2) return c;
    const bool hs = fj - 1 >= 0, hn = fj + 1 < gf.my;
    V4<T> sr = restrict_row<DIM, T>(gf, rf, base + (long long)(fj - 1) * gf.pitch, p.i4, p.in && hs);
    V4<T> nr = restrict_row<DIM, T>(gf, rf, base + (long long)(fj + 1) * gf.pitch, p.i4, p.in && hn);
    return V4<T>{fma(h, sr.x + nr.x, c.x), fma(h, sr.y + nr.y, c.y), fma(h, sr.z + nr.z, c.z),
                 fma(h, sr.w + nr.w, c.w)};
  };
  V4<T> below = zero4<T>();  // row sums of fine plane 2K-1
  if (DIM >= 3 && p.k0 > 0) below = rowsum(2 * p.k0 - 1);
  for (int k = p.k0; k < p.k1; k++) {
    V4<T> mid = rowsum(DIM >= 3 ? 2 * k : k);  // 2D: k is the instance of a batch
    V4<T> above = zero4<T>();
    if (DIM >= 3 && 2 * k + 1 < gf.mz) above = rowsum(2 * k + 1);
    V4<T> o = mid;
    if (DIM >= 3)
      o = V4<T>{fma(h, below.x + above.x, mid.x), fma(h, below.y + above.y, mid.y),
                fma(h, below.z + above.z, mid.z), fma(h, below.w + above.w, mid.w)};
    if (p.in) {
#pragma unroll
      for (int e = 0; e < 4; e++)
        if (p.i4 + e >= g.mx) set_el(o, e, T(0));
      st4(bc + (long long)k * g.plane + p.col, o);
    }
    below = above;
  }
}

// Fused residual and restriction of a 3D level: b_c = P^T (b - A x) without
// storing the fine residual (2s + s/8 bytes per fine node instead of the
// 3s + s + s/8 of v_resid and v_restrict).  A block owns a tile of 31 fine
// x-slots (124 points) by 8 fine rows and a chunk of coarse planes.  Its
// producer warp streams the tile's planes of x (11 rows: the tile's, the row
// below them and their y-neighbours) and b (9 rows) into a 4-stage
// shared-memory ring with bulk tensor copies, one or two planes ahead; nine
// consumer warps compute the residual of nine fine rows (the tile's rows and
// the one below) on 32 slots (the tile's and the one left of it) of one fine
// plane, every neighbour taken from the ring, exactly as v_resid computes it,
// into a shared-memory plane (double-buffered: one barrier of the consumers
// per fine plane); 248 of them, one per coarse point of the tile (4 coarse
// rows by 62), then weight the plane in x and y as v_restrict does and
// combine consecutive fine planes in z in registers.  Every residual and
// every weighted sum is the same operation in the same order as in the two
// kernels, so b_c is bit-identical.
struct RRShape {
  int nxt, nyt, nzt, zc;  // x-tiles (31 fine slots), y-tiles (8 fine rows), coarse-plane chunks, planes per chunk
  unsigned blocks() const { return (unsigned)nxt * (unsigned)nyt * (unsigned)nzt; }
};

inline RRShape rr_shape(const Geom &gf, const Geom &gc, int zc = 16) {
  RRShape q;
  q.nxt = (gf.pitch / 4 + 30) / 31;
  q.nyt = (gc.my + 3) / 4;
  q.zc = zc < gc.mz ? zc : gc.mz;
  q.nzt = (gc.mz + q.zc - 1) / q.zc;
  return q;
}

// Shared-memory layout of the ring (offsets from a 128-byte aligned base)
template <typename T>
struct RRRing {
  static constexpr int NS = 4;                   // stages (planes)
  static constexpr int XW = 136, XR = 11;        // x box: points 124 tx - 4 .. + 135, rows j0 - 2 .. j0 + 8
  static constexpr int BW = 128, BR = 9;         // b box: points 124 tx - 4 .. + 127, rows j0 - 1 .. j0 + 7
  static constexpr unsigned XBYTES = XW * XR * sizeof(T), BBYTES = BW * BR * sizeof(T);
  static constexpr unsigned XSTR = (XBYTES + 127) / 128 * 128, BSTR = (BBYTES + 127) / 128 * 128;
  static constexpr unsigned STAGE = XSTR + BSTR;
  static constexpr unsigned RS = 2 * 9 * 32 * sizeof(V4<T>);  // the residual planes
  static constexpr unsigned BARS = NS * STAGE + RS;            // full[NS], empty[NS]
  static constexpr size_t SMEM = 128 + BARS + 2 * NS * sizeof(uint64_t);
};

template <typename T>
struct RRBlocks {  // FP32: 4 blocks of 320 threads per SM (51 registers); FP64: 2 (the ring's size)
  static constexpr int value = sizeof(T) == 4 ? 4 : 2;
};

template <typename T>
__global__ void __launch_bounds__(320, RRBlocks<T>::value)
    v_resid_restrict(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap bmap, Geom gf,
                     Geom gc, RRShape q, KspState *st, T *__restrict__ bc, int *fault) {
  using R = RRRing<T>;
  if (ksp_done_v(st)) return;
  extern __shared__ unsigned char rr_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(rr_raw) + 127) & ~uintptr_t(127));
  V4<T>(*rs)[9][32] = reinterpret_cast<V4<T>(*)[9][32]>(base + R::NS * R::STAGE);
  uint64_t *full = reinterpret_cast<uint64_t *>(base + R::BARS), *empty = full + R::NS;
  auto xs = [&](int s) { return reinterpret_cast<const T *>(base + s * R::STAGE); };
  auto bs = [&](int s) { return reinterpret_cast<const T *>(base + s * R::STAGE + R::XSTR); };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tx = blockIdx.x % q.nxt, tr = blockIdx.x / q.nxt, ty = tr % q.nyt, tz = tr / q.nyt;
  const int K0 = tz * q.zc, K1 = min(K0 + q.zc, gc.mz);
  const int fbeg = max(2 * K0 - 1, 0), fend = min(2 * K1 - 1, gf.mz - 1);  // fine planes, inclusive
  const int nq = fend - fbeg + 3;                                          // ring planes fbeg - 1 .. fend + 1
  if (threadIdx.x == 0) {
    for (int s = 0; s < R::NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 9);
    }
    mbar_init_fence();
  }
  __syncthreads();
  if (warp == 9) {  // producer
    if (lane == 0) {
      for (int qq = 0; qq < nq; qq++) {
        const int s = qq % R::NS, u = qq / R::NS;
        if (u > 0) mbar_wait(&empty[s], (u - 1) & 1, fault);  // the plane that used the stage is done
        const int pl = fbeg - 1 + qq;
        mbar_arrive_tx(&full[s], R::XBYTES + R::BBYTES);
        tma_load_3d(base + s * R::STAGE, &xmap, 124 * tx - 4, 8 * ty - 2, pl, &full[s]);
        tma_load_3d(base + s * R::STAGE + R::XSTR, &bmap, 124 * tx - 4, 8 * ty - 1, pl, &full[s]);
      }
      // no copy may still be in flight when the block ends
      for (int qq = max(0, nq - R::NS); qq < nq; qq++) mbar_wait(&full[qq % R::NS], (qq / R::NS) & 1, fault, true);
    }
    return;
  }
  const int row = warp;
  const int slot = 31 * tx - 1 + lane, j = 8 * ty - 1 + row, i4 = 4 * slot;
  const bool in = slot >= 0 && i4 < gf.pitch && j >= 0 && j < gf.my;
  const bool hs = j - 1 > 0, hn = j + 1 < gf.my - 1;
  const int c0 = 4 * lane;  // box column of the slot's element 0
  const Wv<T> w(gf);
  const T h = T(0.5);
  const int t = threadIdx.x;
  const bool rt = t < 248;
  const int Jl = t / 62, Il = t - 62 * (t / 62);
  const int J = 4 * ty + Jl, I = 62 * tx + Il;
  const bool rst = rt && J < gc.my && I < gc.pitch;  // stores (points past mx_c are padding: 0)
  T below = T(0), mid = T(0);
  mbar_wait(&full[0], 0, fault);  // planes fbeg - 1 and fbeg
  mbar_wait(&full[1], 0, fault);
  for (int f = fbeg; f <= fend; f++) {
    const int qq = f - fbeg + 1;  // ring index of plane f
    mbar_wait(&full[(qq + 1) % R::NS], ((qq + 1) / R::NS) & 1, fault);
    const T *xm = xs((qq - 1) % R::NS), *xc = xs(qq % R::NS), *xp = xs((qq + 1) % R::NS);
    V4<T> o = zero4<T>();
    if (in) {
      const int ro = (row + 1) * R::XW + c0;
      Nb<T> nb;
      nb.c = *reinterpret_cast<const V4<T> *>(xc + ro);
      nb.l = xc[ro - 1];  // lane 0 (the slot left of the tile): element 0 is not used
      nb.r = xc[ro + 4];
      nb.ys = add4(hs ? *reinterpret_cast<const V4<T> *>(xc + ro - R::XW) : zero4<T>(),
                   hn ? *reinterpret_cast<const V4<T> *>(xc + ro + R::XW) : zero4<T>());
      const bool hd = f - 1 > 0, hu = f + 1 < gf.mz - 1;
      nb.zs = add4(hd ? *reinterpret_cast<const V4<T> *>(xm + ro) : zero4<T>(),
                   hu ? *reinterpret_cast<const V4<T> *>(xp + ro) : zero4<T>());
      nb.jkb = jk_bdry(gf, 3, j, f);
      const V4<T> bv = *reinterpret_cast<const V4<T> *>(bs(qq % R::NS) + row * R::BW + c0);
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int i = i4 + e;
        set_el(o, e, i < gf.mx ? resid_el<3, T>(gf, w, nb, e, i, nb.jkb, el(bv, e)) : T(0));
      }
    }
    rs[f & 1][row][lane] = o;
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[(qq - 1) % R::NS]);  // plane f - 1 is no longer read
    bar_sync(1, 288);
    if (rt) {
      // fine points 2I-1, 2I, 2I+1 are elements 2Il+3 .. 2Il+5 of the row (slot 0 is the halo slot)
      const T *r0 = reinterpret_cast<const T *>(&rs[f & 1][0][0]);
      auto rowv = [&](int rr) -> T {
        const T *a = r0 + rr * 128 + 2 * Il + 3;
        return fma(h, a[0] + a[2], a[1]);
      };
      // fine rows 2J-1, 2J, 2J+1 are tile rows 2Jl, 2Jl+1, 2Jl+2
      const T v = fma(h, rowv(2 * Jl) + rowv(2 * Jl + 2), rowv(2 * Jl + 1));
      if ((f & 1) == 0) {
        mid = v;
        if (f + 1 >= gf.mz && rst)  // no fine plane 2K+1: the last coarse plane
          bc[(long long)(f >> 1) * gc.plane + (long long)J * gc.pitch + I] = I < gc.mx ? fma(h, below + T(0), mid) : T(0);
      } else {
        const int K = f >> 1;  // coarse plane whose upper fine plane this is
        if (f > 2 * K0 - 1 && rst)
          bc[(long long)K * gc.plane + (long long)J * gc.pitch + I] = I < gc.mx ? fma(h, below + v, mid) : T(0);
        below = v;
      }
    }
  }
}

// x_f += P x_c (Q1 interpolation).  A thread owns a coarse slot I4..I4+3 and
// writes the 8 fine x-points 2I4 .. 2I4+7 of fine rows 2J, 2J+1 and planes
// 2K, 2K+1 (those inside the fine grid).  The x-interpolated coarse rows J and
// J+1 of plane K+1 are kept for the next plane (one plane window).
template <typename T>
struct ProlongBlocks {  // FP32: 4 x 256 threads per SM; FP64: no cap (a cap of 64 spilled)
  static constexpr int value = sizeof(T) == 4 ? 4 : 1;
};

template <int DIM, typename T, int MB = ProlongBlocks<T>::value>
__global__ void __launch_bounds__(256, MB) v_prolong(Geom gf, Geom g, Slots s, KspState *st, const T *__restrict__ xc,
                                                 T *__restrict__ xf) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  const SlotPos p = slot_pos(g, s);
  const int lane = threadIdx.x & 31;
  const T h = T(0.5);
  const int fi = 2 * p.i4;
  const bool ok0 = p.in;
  const bool ok1 = p.in && DIM >= 2 && p.j + 1 < g.my;  // coarse row J+1 (fine row 2J+1) exists
  // coarse row (k, jj) x-interpolated to 8 fine values; every lane calls it
  auto xrow = [&](int k, int jj, bool ok, V4<T> &lo, V4<T> &hi) {
    const long long m = (long long)k * g.plane + (long long)jj * g.pitch + p.i4;
    V4<T> C = ok ? ld4(xc + m) : zero4<T>();
    T nx = __shfl_down_sync(0xffffffffu, C.x, 1);
    if (lane == 31) nx = (ok && p.i4 + 4 < g.mx) ? xc[m + 4] : T(0);
    lo = V4<T>{C.x, h * (C.x + C.y), C.y, h * (C.y + C.z)};
    hi = V4<T>{C.z, h * (C.z + C.w), C.w, h * (C.w + nx)};
  };
  // x_f[fk][fj][fi..fi+7] += wgt * (lo, hi): the current values of a batch of
  // fine rows are loaded together (no load waits behind another row's store),
  // then updated and stored; points past mx_f are padding
  const bool lo_ok = fi < gf.mx, hi_ok = fi + 4 < gf.mx;
  auto fload = [&](long long fm, bool ok, V4<T> &l, V4<T> &h2) {
    l = (ok && lo_ok) ? ld4(xf + fm) : zero4<T>();
    h2 = (ok && hi_ok) ? ld4(xf + fm + 4) : zero4<T>();
  };
  auto fstore = [&](long long fm, bool ok, V4<T> l, V4<T> h2, const V4<T> &lo, const V4<T> &hi, T wgt) {
    if (!ok) return;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      if (fi + e < gf.mx) set_el(l, e, fma(wgt, el(lo, e), el(l, e)));
      if (fi + 4 + e < gf.mx) set_el(h2, e, fma(wgt, el(hi, e), el(h2, e)));
    }
    if (lo_ok) st4(xf + fm, l);
    if (hi_ok) st4(xf + fm + 4, h2);
  };
  V4<T> a0l, a0h, a1l, a1h;  // plane k: rows J, J+1
  xrow(p.k0, p.j, ok0, a0l, a0h);
  xrow(p.k0, p.j + (ok1 ? 1 : 0), ok1, a1l, a1h);
  for (int k = p.k0; k < p.k1; k++) {
    const bool up = DIM >= 3 && k + 1 < g.mz;  // fine plane 2k+1 exists (uniform in the block)
    const int fk = DIM >= 3 ? 2 * k : k, fj = DIM >= 2 ? 2 * p.j : 0;
    const long long fa = (long long)fk * gf.plane + (long long)fj * gf.pitch + fi;
    // fine plane fk: rows fj, fj+1
    V4<T> r0l, r0h, r1l, r1h;
    fload(fa, ok0, r0l, r0h);
    fload(fa + gf.pitch, ok1, r1l, r1h);
    V4<T> b0l = zero4<T>(), b0h = zero4<T>(), b1l = zero4<T>(), b1h = zero4<T>();
    if (up) {
      xrow(k + 1, p.j, ok0, b0l, b0h);
      xrow(k + 1, p.j + (ok1 ? 1 : 0), ok1, b1l, b1h);
    }
    fstore(fa, ok0, r0l, r0h, a0l, a0h, T(1));
    fstore(fa + gf.pitch, ok1, r1l, r1h, add4(a0l, a1l), add4(a0h, a1h), h);
    if (up) {  // fine plane fk+1: rows fj, fj+1
      fload(fa + gf.plane, ok0, r0l, r0h);
      fload(fa + gf.plane + gf.pitch, ok1, r1l, r1h);
      fstore(fa + gf.plane, ok0, r0l, r0h, add4(a0l, b0l), add4(a0h, b0h), h);
      fstore(fa + gf.plane + gf.pitch, ok1, r1l, r1h, add4(add4(a0l, a1l), add4(b0l, b1l)),
             add4(add4(a0h, a1h), add4(b0h, b1h)), T(0.25));
    }
    a0l = b0l; a0h = b0h; a1l = b1l; a1h = b1h;
  }
}

// ------------------------------------------------------------------ pointwise
// Slot decomposition as the stencils (one vec4 of points per thread per
// plane); padding points stay zero because every input's padding is zero.
#define FG_PW_BEGIN                                        \
  const SlotPos p = slot_pos(g, s);                        \
  if (p.in)                                                \
    for (int k = p.k0; k < p.k1; k++) {                    \
      const long long n = (long long)k * g.plane + p.col;
#define FG_PW_END }

// r -= alpha w; RR: r.r reduced (unpreconditioned norm test).  The matching
// y += alpha p is deferred to the next v_cgp_apply, or to v_cg_pend when the
// solve stops.
template <typename T, bool RR>
__global__ void __launch_bounds__(256) v_cg_r(Geom g, Slots s, KspState *st, const T *__restrict__ wv,
                                              T *__restrict__ r, Reducer red, int slot) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  const T a = st ? (T)st->alpha : T(0);  // no state: alpha = 0
  T acc = T(0);
  FG_PW_BEGIN
  const V4<T> ww = ld4(wv + n), rr = ld4(r + n);
  const V4<T> rn{fma(-a, ww.x, rr.x), fma(-a, ww.y, rr.y), fma(-a, ww.z, rr.z), fma(-a, ww.w, rr.w)};
  st4(r + n, rn);
  if (RR) acc = fma(rn.x, rn.x, fma(rn.y, rn.y, fma(rn.z, rn.z, fma(rn.w, rn.w, acc))));
  FG_PW_END
  if (RR) {
    double v1[1] = {(double)acc};
    reduce_slots<1>(v1, red, slot, st, FIN_RR, nullptr, s);
  }
}

// The deferred y += alpha p of the last CG iteration, after the loop has
// stopped (the state is done): `pend` names the buffer, 1 for p0, 2 for p1.
// y is not zero-filled when a solve starts: an update reached it only if a
// direction update ran after a successful FIN_PW (its >= 2), otherwise y is
// written here from 0 (alpha p, or zeros).
__device__ __forceinline__ bool ksp_y_written(const KspState *st) { return st->its >= 2; }

template <typename T>
__global__ void __launch_bounds__(256) v_cg_pend(Geom g, Slots s, const KspState *st, const T *__restrict__ p0,
                                                 const T *__restrict__ p1, T *__restrict__ y) {
  st = block_state(const_cast<KspState *>(st), s);
  if (!st) return;
  const bool written = ksp_y_written(st);
  const int pend = st->pend;
  if (written && !pend) return;
  const T a = pend ? (T)st->alpha : T(0);
  const T *__restrict__ pv = pend == 1 ? p0 : p1;
  FG_PW_BEGIN
  V4<T> yy = written ? ld4(y + n) : zero4<T>();
  if (pend) {
    const V4<T> pp = ld4(pv + n);
    yy = V4<T>{fma(a, pp.x, yy.x), fma(a, pp.y, yy.y), fma(a, pp.z, yy.z), fma(a, pp.w, yy.w)};
  }
  st4(y + n, yy);
  FG_PW_END
}

// z.z and z.r reduced together (out: per plane for a batch)
template <typename T>
__global__ void __launch_bounds__(256) v_dots(Geom g, Slots s, KspState *st, const T *__restrict__ z,
                                              const T *__restrict__ r, Reducer red, int slot, Fin fin, double *out) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  T zz = T(0), zr = T(0);
  FG_PW_BEGIN
  const V4<T> a = ld4(z + n), b = ld4(r + n);
  zz = fma(a.x, a.x, fma(a.y, a.y, fma(a.z, a.z, fma(a.w, a.w, zz))));
  zr = fma(a.x, b.x, fma(a.y, b.y, fma(a.z, b.z, fma(a.w, b.w, zr))));
  FG_PW_END
  double v2[2] = {(double)zz, (double)zr};
  reduce_slots<2>(v2, red, slot, st, fin, out, s);
}

// out = c * in (Jacobi apply, or scaled copy)
template <typename T>
__global__ void __launch_bounds__(256) v_scale(Geom g, Slots s, KspState *st, const T *__restrict__ in, T c,
                                               T *__restrict__ out) {
  st = block_state(st, s);
  if (ksp_done_v(st)) return;
  FG_PW_BEGIN
  const V4<T> a = ld4(in + n);
  st4(out + n, V4<T>{c * a.x, c * a.y, c * a.z, c * a.w});
  FG_PW_END
}

template <typename T>
__global__ void __launch_bounds__(256) v_zero(Geom g, Slots s, T *__restrict__ a) {
  FG_PW_BEGIN
  st4(a + n, zero4<T>());
  FG_PW_END
}

// The FP64 residual b - A u0 of an initial iterate that is zero on every
// interior node (the zero initial state, with or without g on the boundary),
// and its r.r as v_dots reduces it.  The Jacobian's interior rows do not see
// boundary columns, so there r = b - A 0 = b + 0 (the value resid_el returns:
// its fused terms all add +0); boundary rows keep fma(-scdiag, u0, b).  A
// pointwise pass instead of the FP64 stencil, with identical results.
template <int DIM>
__global__ void __launch_bounds__(256) v_resid_zero0(Geom g, Slots s, const double *__restrict__ b,
                                                     const double *__restrict__ u0, double *__restrict__ r,
                                                     Reducer red, int slot, double *out) {
  const double sd = g.scdiag;
  double rr = 0.0;
  FG_PW_BEGIN
  const bool jkb = jk_bdry(g, DIM, p.j, k);
  const V4<double> bv = ld4(b + n), uv = ld4(u0 + n);
  V4<double> o;
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int i = p.i4 + e;
    double v = 0.0;
    if (i < g.mx) v = (jkb || i == 0 || i == g.mx - 1) ? fma(-sd, el(uv, e), el(bv, e)) : el(bv, e) + 0.0;
    set_el(o, e, v);
  }
  st4(r + n, o);
  rr = fma(o.x, o.x, fma(o.y, o.y, fma(o.z, o.z, fma(o.w, o.w, rr))));
  FG_PW_END
  double v1[1] = {rr};
  reduce_slots<1>(v1, red, slot, nullptr, FIN_STORE, out, s);
}

// is[0] = 1 / sqrt(rr[0]) (one thread: the FP64 square root and division
// once per inner solve instead of once per block of v_demote_init)
static __global__ void k_inv_norm(const double *__restrict__ rr, double *__restrict__ is) { *is = 1.0 / sqrt(*rr); }

// The set-up of an inner FP32 solve from an FP64 residual in one pass:
// r32 = (float)r64 * (float)is with is = 1 / sqrt(rr), rr = r64.r64 as
// stored by the residual kernel (k_inv_norm, once), and r32.r32 reduced as
// v_dots<float> reduces it, finalised as FIN_INIT_RR.  The scaling is done
// in FP32 after rounding r64 to FP32 on the integer pipe (d2f_bits): the
// FP64 multiply and conversion per element made the pass FP64-bound (ncu:
// FP64 pipe 87%, 0.53 ms at 513^3); the inner solve only needs r32 close to
// unit norm, and its own norm is the one it starts from.  Replaces v_demote
// and v_dots (y32 is not zero-filled: see v_cg_pend).
static __global__ void __launch_bounds__(256) v_demote_init(Geom g, Slots s, KspState *st, const double *__restrict__ r,
                                                     const double *__restrict__ isp, float *__restrict__ r32,
                                                     Reducer red, int slot) {
  if (ksp_done_v(st)) return;
  const float is = (float)*isp;
  float zz = 0.f;
  FG_PW_BEGIN
  const V4<double> a = ld4(r + n);
  const V4<float> o{d2f_bits(a.x) * is, d2f_bits(a.y) * is, d2f_bits(a.z) * is, d2f_bits(a.w) * is};
  st4(r32 + n, o);
  zz = fmaf(o.x, o.x, fmaf(o.y, o.y, fmaf(o.z, o.z, fmaf(o.w, o.w, zz))));
  FG_PW_END
  double v1[1] = {(double)zz};
  reduce_slots<1>(v1, red, slot, st, FIN_INIT_RR, nullptr, s);
}

// The end of an inner FP32 solve whose updates accumulate in FP64 (the ACC
// form of v_cgp_apply): the last deferred update y64 += (yscale * alpha) p,
// after an older one the paired updates still owe (pend2).
// y64 is read unless nothing has reached it yet (no update in this inner
// solve and the state's yfresh: the first refinement step), in which case it
// is written from 0.  Per plane for a batch.
static __global__ void __launch_bounds__(256) v_pend_acc(Geom g, Slots s, const KspState *st,
                                                  const float *__restrict__ p0, const float *__restrict__ p1,
                                                  double *__restrict__ y) {
  st = block_state(const_cast<KspState *>(st), s);
  if (!st) return;
  const bool keep = ksp_y_written(st) || !st->yfresh;
  const int pend = st->pend, pend2 = st->pend2;
  if (keep && !pend && !pend2) return;
  const double a = pend ? st->yscale * st->alpha : 0.0;
  const double a2 = pend2 ? st->yscale * st->alpha2 : 0.0;
  const float *__restrict__ pv = pend == 1 ? p0 : p1;
  const float *__restrict__ qv = pend2 == 1 ? p0 : p1;
  FG_PW_BEGIN
  V4<double> yy = keep ? ld4(y + n) : zero4<double>();
  if (pend2) {  // an older owed update (paired updates): first
    const V4<float> qq = ld4(qv + n);
    yy = V4<double>{fma(a2, f2d_bits(qq.x), yy.x), fma(a2, f2d_bits(qq.y), yy.y), fma(a2, f2d_bits(qq.z), yy.z),
                    fma(a2, f2d_bits(qq.w), yy.w)};
  }
  if (pend) {
    const V4<float> pp = ld4(pv + n);
    yy = V4<double>{fma(a, f2d_bits(pp.x), yy.x), fma(a, f2d_bits(pp.y), yy.y), fma(a, f2d_bits(pp.z), yy.z),
                    fma(a, f2d_bits(pp.w), yy.w)};
  }
  st4(y + n, yy);
  FG_PW_END
}

// r32 = (float)r64 * (float)inv_s, rounded as v_demote_init rounds; inv_s
// per plane for a batch (scale[plane])
static __global__ void __launch_bounds__(256) v_demote(Geom g, Slots s, const double *__restrict__ r, const double *scale,
                                                double inv_s, float *__restrict__ r32) {
  FG_PW_BEGIN
  const float is = (float)(scale ? scale[k] : inv_s);
  const V4<double> a = ld4(r + n);
  st4(r32 + n, V4<float>{d2f_bits(a.x) * is, d2f_bits(a.y) * is, d2f_bits(a.z) * is, d2f_bits(a.w) * is});
  FG_PW_END
}

// y64 += s * (double)e32; s per plane for a batch (scale[plane]); fresh: y64
// is taken as +0 (not read), as after v_zero
static __global__ void __launch_bounds__(256) v_promote_add(Geom g, Slots s, const float *__restrict__ e, const double *scale,
                                                     double sc, double *__restrict__ y, bool fresh = false) {
  FG_PW_BEGIN
  const double f = scale ? scale[k] : sc;
  const V4<float> a = ld4(e + n);
  const V4<double> b = fresh ? zero4<double>() : ld4(y + n);
  st4(y + n, V4<double>{fma(f, (double)a.x, b.x), fma(f, (double)a.y, b.y), fma(f, (double)a.z, b.z),
                        fma(f, (double)a.w, b.w)});
  FG_PW_END
}

// The end of an inner FP32 solve and the FP64 update in one pass: the last
// CG iteration's deferred y32 += alpha p (v_cg_pend), then y64 += sc *
// (double)y32 (v_promote_add, fresh as there); y32 itself is not written back.
static __global__ void __launch_bounds__(256) v_pend_promote(Geom g, Slots s, const KspState *st,
                                                      const float *__restrict__ p0, const float *__restrict__ p1,
                                                      const float *__restrict__ e, double sc, double *__restrict__ y,
                                                      bool fresh) {
  const int pend = st ? st->pend : 0;
  const bool written = st && ksp_y_written(st);  // else the inner solution starts from 0 (not stored)
  const float a = pend ? (float)st->alpha : 0.f;
  const float *__restrict__ pv = pend == 1 ? p0 : p1;
  FG_PW_BEGIN
  V4<float> ev = written ? ld4(e + n) : zero4<float>();
  if (pend) {
    const V4<float> pp = ld4(pv + n);
    ev = V4<float>{fmaf(a, pp.x, ev.x), fmaf(a, pp.y, ev.y), fmaf(a, pp.z, ev.z), fmaf(a, pp.w, ev.w)};
  }
  const V4<double> b = fresh ? zero4<double>() : ld4(y + n);
  st4(y + n, V4<double>{fma(sc, (double)ev.x, b.x), fma(sc, (double)ev.y, b.y), fma(sc, (double)ev.z, b.z),
                        fma(sc, (double)ev.w, b.w)});
  FG_PW_END
}

}  // namespace fg
