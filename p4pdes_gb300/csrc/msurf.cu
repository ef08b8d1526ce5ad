// msurf.cu -- the minimal-surface equation of c/ch7/minimal.c on one GPU.
//
//   -div( (1 + |grad u|^2)^q grad u ) = 0 on the unit square, u = g on the
//   boundary; 9-point finite differences (FormFunctionLocal,
//   minimal.c:210-282), catenoid / tent boundary data (minimal.c:27-42).
//
// Solver: Newton (PETSc SNESNEWTONLS: J Y = F, X <- X - lambda Y with the
// cubic backtracking line search on ||F||^2/2, SNESConvergedDefault), with
// optional grid sequencing (each grid starts from the Q1 interpolation of the
// previous grid's solution).  F(u), the norms, the line search and the update
// are FP64.  The Newton step is solved in FP32: the exact Jacobian of F is
// applied matrix-free from eight FP32 coefficients per node (computed in FP64
// from u once per Newton step), inside BiCGStab right-preconditioned by the
// FP32 Poisson multigrid V-cycle of a 2D fish solver of the same grid (the
// reference preconditions with Poisson2DJacobianLocal, minimal.c:142-145);
// boundary rows of the Jacobian are the identity and are passed through the
// preconditioner unchanged.  The right-hand side is scaled to unit norm, so
// FP32 range is never an issue; the inner solve stops at ksp_rtol on its own
// (unpreconditioned) residual, as PETSc's KSP does at -ksp_rtol.
//
// Layout: the fish solver's padded 2D layout (pitch = mx rounded up to 4,
// padding kept at 0); one thread per node, blocks of 32 x 8; reductions are
// deterministic (block partials, last block sums them in order).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "graph_loop.cuh"
#include "mg_hooks.cuh"

namespace fg {

struct MsP {
  int problem;
  double q, c, H;
  int model;      // FISHGPU_NL_MINIMAL / FISHGPU_NL_BRATU
  double lambda;  // Bratu's coefficient of e^u
  // boundary data of one grid, precomputed (k_ms_gtab): nullptr = evaluate g
  // where it is needed
  const double *gt = nullptr;
  int gtm = 0;  // max(mx, my): the length of each of its 16 rows
};

// boundary data: minimal.c:27-42 (tent, catenoid); bratu2D.c:58-68 (zero, Liouville)
__host__ __device__ inline double ms_gd(const MsP &P, double x, double y) {
  if (P.model == FISHGPU_NL_BRATU) {
    if (P.problem != FISHGPU_BRATU_LIOUVILLE) return 0.0;
    const double r2 = (x + 1.0) * (x + 1.0) + (y + 1.0) * (y + 1.0), qq = r2 * r2 + 1.0, omega = r2 / (qq * qq);
    return log(32.0 * omega);
  }
  if (P.problem == FISHGPU_MS_TENT) return x < 1.0e-8 ? 2.0 * P.H * (y < 0.5 ? y : 1.0 - y) : 0.0;
  return P.c * cosh(x / P.c) * sin(acos((y / P.c) / cosh(x / P.c)));
}

// Obstacle problem (c/ch12/obstacle.c:15-49) on (-2,2)^2: the hemispherical
// obstacle with a C^1 skirt at r0 = 0.9, and the exact solution of the
// radial free-boundary problem (free boundary at r = a).
__host__ __device__ inline double obs_psi(double x, double y) {
  const double r = sqrt(x * x + y * y), r0 = 0.9, psi0 = sqrt(1.0 - r0 * r0), dpsi0 = -r0 / psi0;
  return r <= r0 ? sqrt(1.0 - r * r) : psi0 + dpsi0 * (r - r0);
}

__host__ __device__ inline double obs_uexact(double x, double y) {
  const double afree = 0.697965148223374, A = 0.680259411891719, B = 0.471519893402112;
  const double r = sqrt(x * x + y * y);
  return r <= afree ? obs_psi(x, y) : -A * log(r) + B;
}

constexpr double OBS_ZEROTOL = 1.0e-8;  // PETSc's active-set tolerance (obstacle.c:191)

// Poisson2DFunctionLocal (c/ch6/poissonfunctions.c:27-64) with f = 0 and
// g = the exact solution, on (-2,2)^2: interior rows; boundary neighbours are g
__device__ __forceinline__ double obs_f_interior(const Geom &g, const double *__restrict__ u, long long pitch, int i,
                                                 int j) {
  const double hx = g.h[0], hy = g.h[1], x = -2.0 + i * hx, y = -2.0 + j * hy;
  const double scx = hy / hx, scy = hx / hy, scdiag = 2.0 * (scx + scy);
  const long long n = (long long)j * pitch + i;
  const double ue = (i + 1 == g.mx - 1) ? obs_uexact(x + hx, y) : u[n + 1];
  const double uw = (i - 1 == 0) ? obs_uexact(x - hx, y) : u[n - 1];
  const double un = (j + 1 == g.my - 1) ? obs_uexact(x, y + hy) : u[n + pitch];
  const double us = (j - 1 == 0) ? obs_uexact(x, y - hy) : u[n - pitch];
  return scdiag * u[n] - scx * (uw + ue) - scy * (us + un);
}

// Bratu at interior node (i,j), bratu2D.c:205-211: the neighbours are the array's values
__device__ __forceinline__ double lb_f_interior(const Geom &g, const MsP &P, const double *__restrict__ u,
                                                long long pitch, int i, int j) {
  const double hx = g.h[0], hy = g.h[1], darea = hx * hy, hxhy = hx / hy, hyhx = hy / hx;
  const long long n = (long long)j * pitch + i;
  return hyhx * (2.0 * u[n] - u[n - 1] - u[n + 1]) + hxhy * (2.0 * u[n] - u[n - pitch] - u[n + pitch]) -
         darea * P.lambda * exp(u[n]);
}

__device__ __forceinline__ bool ms_bdry(const Geom &g, int i, int j) {
  return i == 0 || j == 0 || i == g.mx - 1 || j == g.my - 1;
}

// Boundary-data table of one grid (P.gt, rows of length M = P.gtm).  The
// values g(x +- hx, y +- hy) that interior nodes next to the boundary ask for
// are stored by asker: rows 0-2 for the askers of row j = 1 (neighbour row
// j - 1 = 0, x-offsets -1, 0, +1), rows 3-5 for row j = my-2 (neighbour row
// my-1), rows 6-8 for column i = 1 (neighbour column 0, y-offsets -1, 0, +1),
// rows 9-11 for column i = mx-2; rows 12-15 hold g at the boundary nodes
// themselves (bottom, top by i; left, right by j).  Every entry is ms_gd at the
// argument expression of the direct evaluation, so the table changes no bit;
// it keeps FP64 transcendentals out of the residual, whose boundary blocks
// otherwise wait on them.
__device__ __forceinline__ int ms_gt_row(int e, int d) { return e * 3 + d; }

__global__ void __launch_bounds__(128) k_ms_gtab(Geom g, MsP P, double *__restrict__ gt, int M) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M) return;
  const double hx = g.h[0], hy = g.h[1];
  if (t >= 1 && t <= g.mx - 2) {
    const double x = t * hx, ys = 1 * hy, yn = (g.my - 2) * hy;
    for (int d = 0; d < 3; d++) {
      gt[(size_t)ms_gt_row(0, d) * M + t] = ms_gd(P, x + (d - 1) * hx, ys + (-1) * hy);
      gt[(size_t)ms_gt_row(1, d) * M + t] = ms_gd(P, x + (d - 1) * hx, yn + 1 * hy);
    }
  }
  if (t >= 1 && t <= g.my - 2) {
    const double y = t * hy, xw = 1 * hx, xe = (g.mx - 2) * hx;
    for (int d = 0; d < 3; d++) {
      gt[(size_t)ms_gt_row(2, d) * M + t] = ms_gd(P, xw + (-1) * hx, y + (d - 1) * hy);
      gt[(size_t)ms_gt_row(3, d) * M + t] = ms_gd(P, xe + 1 * hx, y + (d - 1) * hy);
    }
  }
  if (t < g.mx) {
    gt[(size_t)12 * M + t] = ms_gd(P, t * hx, 0 * hy);
    gt[(size_t)13 * M + t] = ms_gd(P, t * hx, (g.my - 1) * hy);
  }
  if (t < g.my) {
    gt[(size_t)14 * M + t] = ms_gd(P, 0 * hx, t * hy);
    gt[(size_t)15 * M + t] = ms_gd(P, (g.mx - 1) * hx, t * hy);
  }
}

// g at boundary node (i,j)
__device__ __forceinline__ double ms_gown(const Geom &g, const MsP &P, int i, int j) {
  if (!P.gt) return ms_gd(P, i * g.h[0], j * g.h[1]);
  const size_t M = (size_t)P.gtm;
  return j == 0 ? P.gt[12 * M + i] : j == g.my - 1 ? P.gt[13 * M + i] : i == 0 ? P.gt[14 * M + j] : P.gt[15 * M + j];
}

// The eight neighbours of interior node (i,j) (order e w n s ne nw se sw):
// the array value, or g at x +- hx, y +- hy when the neighbour is a boundary
// node (minimal.c:227-255).
__device__ __forceinline__ void ms_nb(const Geom &g, const MsP &P, const double *__restrict__ u, long long pitch,
                                      int i, int j, double v[8]) {
  const double hx = g.h[0], hy = g.h[1], x = i * hx, y = j * hy;
  const int di[8] = {1, -1, 0, 0, 1, -1, 1, -1}, dj[8] = {0, 0, 1, -1, 1, 1, -1, -1};
  const size_t M = (size_t)P.gtm;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int a = i + di[q], b = j + dj[q];
    if (!ms_bdry(g, a, b)) {
      v[q] = u[(long long)b * pitch + a];
    } else if (!P.gt) {
      v[q] = ms_gd(P, x + di[q] * hx, y + dj[q] * hy);
    } else {
      const int e = (dj[q] == -1 && b == 0) ? 0 : (dj[q] == 1 && b == g.my - 1) ? 1 : (di[q] == -1 && a == 0) ? 2 : 3;
      const int d = e < 2 ? di[q] + 1 : dj[q] + 1, t = e < 2 ? i : j;
      v[q] = P.gt[(size_t)ms_gt_row(e, d) * M + t];
    }
  }
}

// The diffusivity (1 + W)^q (minimal.c:46-48).  For the minimal surface
// equation q = -1/2 and it is the reciprocal square root: CUDA's rsqrt (1 ulp)
// instead of pow (2 ulp), which costs many times the FP64 instructions on a
// part whose FP64 rate is low.
__device__ __forceinline__ double ms_diffusivity(double onepw, double q) {
  return q == -0.5 ? rsqrt(onepw) : pow(onepw, q);
}

// F at interior node (i,j), minimal.c:257-280
__device__ __forceinline__ double ms_f_interior(const Geom &g, const MsP &P, const double *__restrict__ u,
                                                long long pitch, int i, int j) {
  const double hx = g.h[0], hy = g.h[1], hxhy = hx / hy, hyhx = hy / hx;
  double v[8];
  ms_nb(g, P, u, pitch, i, j, v);
  const double uc = u[(long long)j * pitch + i], ue = v[0], uw = v[1], un = v[2], us = v[3];
  const double une = v[4], unw = v[5], use = v[6], usw = v[7];
  double dx, dy;
  dx = (ue - uc) / hx;
  dy = (un + une - us - use) / (4.0 * hy);
  const double De = ms_diffusivity(1.0 + dx * dx + dy * dy, P.q);
  dx = (uc - uw) / hx;
  dy = (unw + un - usw - us) / (4.0 * hy);
  const double Dw = ms_diffusivity(1.0 + dx * dx + dy * dy, P.q);
  dx = (ue + une - uw - unw) / (4.0 * hx);
  dy = (un - uc) / hy;
  const double Dn = ms_diffusivity(1.0 + dx * dx + dy * dy, P.q);
  dx = (ue + use - uw - usw) / (4.0 * hx);
  dy = (uc - us) / hy;
  const double Ds = ms_diffusivity(1.0 + dx * dx + dy * dy, P.q);
  return -hyhx * (De * (ue - uc) - Dw * (uc - uw)) - hxhy * (Dn * (un - uc) - Ds * (uc - us));
}

// Deterministic sum over the blocks of a 2D launch: block partials, the last
// block to arrive sums them in block order and calls fin(total) on thread 0.
template <int NV, class Fin>
__device__ __forceinline__ void ms_reduce(double (&v)[NV], const Reducer &red, Fin fin) {
  __shared__ bool am_last;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nt = blockDim.x * blockDim.y;
  const int bid = blockIdx.x + gridDim.x * blockIdx.y, nb = gridDim.x * gridDim.y;
  block_sum<NV>(v);
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) red.partials[q * red.cap + bid] = v[q];
    __threadfence();
    am_last = atomicAdd(red.tickets, 1u) == (unsigned)(nb - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) {
    s[q] = 0.0;
    for (int b = tid; b < nb; b += nt) s[q] += __ldcg(&red.partials[q * red.cap + b]);
  }
  block_sum<NV>(s);
  if (tid == 0) {
    *red.tickets = 0u;
    fin(s);
  }
}

struct Store2Fin {
  double *out;
  __device__ void operator()(const double *s) const { out[0] = s[0]; out[1] = s[1]; }
};

#define MS_NODE_BEGIN                                               \
  const int i = blockIdx.x * blockDim.x + threadIdx.x;              \
  const int j = blockIdx.y * blockDim.y + threadIdx.y;              \
  const bool in_ = j < g.my && i < g.pitch;                         \
  const long long n = (long long)j * g.pitch + i;                   \
  const bool node = in_ && i < g.mx;                              \
  (void)node;

// F(u) everywhere (boundary rows u - g, padding 0), ||F||^2 -> out[0] and
// ||u||^2 -> out[1] (the Newton step's ||x||; ms_reduce sums each component
// on its own, in the order of a reduction of that component alone)
__global__ void __launch_bounds__(256) k_ms_resid(Geom g, MsP P, const double *__restrict__ u,
                                                  double *__restrict__ F, Reducer red, double *out) {
  MS_NODE_BEGIN
  double acc = 0.0;
  const double uu = node ? u[n] : 0.0;
  if (in_) {
    double f = 0.0;
    if (node && P.model == FISHGPU_NL_OBSTACLE) {
      const double x = -2.0 + i * g.h[0], y = -2.0 + j * g.h[1];
      f = ms_bdry(g, i, j) ? 2.0 * (g.h[1] / g.h[0] + g.h[0] / g.h[1]) * (u[n] - obs_uexact(x, y))
                           : obs_f_interior(g, u, g.pitch, i, j);
      // the VI residual norm is taken over the inactive set (u > psi or F <= 0)
      acc = (u[n] <= obs_psi(x, y) + OBS_ZEROTOL && f > 0.0) ? 0.0 : f * f;
    } else if (node) {
      f = ms_bdry(g, i, j) ? u[n] - ms_gown(g, P, i, j)
          : P.model == FISHGPU_NL_BRATU ? lb_f_interior(g, P, u, g.pitch, i, j) : ms_f_interior(g, P, u, g.pitch, i, j);
      acc = f * f;
    }
    F[n] = f;
  }
  double v2[2] = {acc, uu * uu};
  ms_reduce<2>(v2, red, Store2Fin{out});
}

// Linearisation of one half-point flux D(W) d (d the normal difference):
//   A = D + K dn/hn,  Q = K dt/(4 ht),  K = 2 q D/(1+W) d
__device__ __forceinline__ void ms_half(double q, double d, double hn, double dt, double ht, float &A, float &Q) {
  const double dn = d / hn, W = dn * dn + dt * dt, D = ms_diffusivity(1.0 + W, q);
  const double K = 2.0 * q * D / (1.0 + W) * d;
  A = (float)(D + K * dn / hn);
  Q = (float)(K * dt / (4.0 * ht));
}

// Jacobian coefficients at u: C1 = (Ae, Qe, Aw, Qw), C2 = (An, Qn, As, Qs)
__global__ void __launch_bounds__(256) k_ms_coef(Geom g, MsP P, const double *__restrict__ u,
                                                 const double *__restrict__ F, float4 *__restrict__ C1,
                                                 float4 *__restrict__ C2) {
  MS_NODE_BEGIN
  if (!in_) return;
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
  if (node && P.model == FISHGPU_NL_OBSTACLE) {  // C1.x = 1 on the active set
    a.x = (u[n] <= obs_psi(-2.0 + i * g.h[0], -2.0 + j * g.h[1]) + OBS_ZEROTOL && F[n] > 0.0) ? 1.f : 0.f;
  } else if (node && !ms_bdry(g, i, j) && P.model == FISHGPU_NL_BRATU) {
    a.x = (float)(g.h[0] * g.h[1] * P.lambda * exp(u[n]));  // the diagonal shift darea lambda e^u
  } else if (node && !ms_bdry(g, i, j)) {
    const double hx = g.h[0], hy = g.h[1];
    double v[8];
    ms_nb(g, P, u, g.pitch, i, j, v);
    const double uc = u[n], ue = v[0], uw = v[1], un = v[2], us = v[3];
    const double une = v[4], unw = v[5], use = v[6], usw = v[7];
    ms_half(P.q, ue - uc, hx, (un + une - us - use) / (4.0 * hy), hy, a.x, a.y);
    ms_half(P.q, uc - uw, hx, (unw + un - usw - us) / (4.0 * hy), hy, a.z, a.w);
    ms_half(P.q, un - uc, hy, (ue + une - uw - unw) / (4.0 * hx), hx, b.x, b.y);
    ms_half(P.q, uc - us, hy, (ue + use - uw - usw) / (4.0 * hx), hx, b.z, b.w);
  }
  C1[n] = a;
  C2[n] = b;
}

// (J v) at node n in FP32: identity on boundary rows.  Minimal surface:
// boundary neighbours do not enter interior rows (their values are g).
// Bratu: the 5-point rows couple to every neighbour, diagonal shifted by
// -darea lambda e^u (C1.x).
__device__ __forceinline__ float ms_jv_node(const Geom &g, int model, int i, int j, long long n, float a, float b,
                                            const float4 *__restrict__ C1, const float4 *__restrict__ C2,
                                            const float *__restrict__ v) {
  const long long P = g.pitch;
  if (model == FISHGPU_NL_OBSTACLE) {  // Poisson2DJacobianLocal on the inactive set, identity on the active set
    if (C1[n].x != 0.f) return v[n];
    if (ms_bdry(g, i, j)) return 2.f * (a + b) * v[n];
    const bool E = i + 1 < g.mx - 1, Wb = i - 1 > 0, N = j + 1 < g.my - 1, S = j - 1 > 0;
    return 2.f * (a + b) * v[n] - a * ((E ? v[n + 1] : 0.f) + (Wb ? v[n - 1] : 0.f)) -
           b * ((N ? v[n + P] : 0.f) + (S ? v[n - P] : 0.f));
  }
  if (ms_bdry(g, i, j)) return v[n];
  if (model == FISHGPU_NL_BRATU)
    return (2.f * (a + b) - C1[n].x) * v[n] - a * (v[n - 1] + v[n + 1]) - b * (v[n - P] + v[n + P]);
  const bool E = i + 1 < g.mx - 1, Wb = i - 1 > 0, N = j + 1 < g.my - 1, S = j - 1 > 0;
  const float vc = v[n];
  const float ve = E ? v[n + 1] : 0.f, vw = Wb ? v[n - 1] : 0.f;
  const float vn = N ? v[n + P] : 0.f, vs = S ? v[n - P] : 0.f;
  const float vne = (E && N) ? v[n + P + 1] : 0.f, vnw = (Wb && N) ? v[n + P - 1] : 0.f;
  const float vse = (E && S) ? v[n - P + 1] : 0.f, vsw = (Wb && S) ? v[n - P - 1] : 0.f;
  const float4 c1 = C1[n], c2 = C2[n];
  const float ce = c1.x * (ve - vc) + c1.y * (vn + vne - vs - vse);
  const float cw = c1.z * (vc - vw) + c1.w * (vnw + vn - vsw - vs);
  const float cn = c2.x * (vn - vc) + c2.y * (ve + vne - vw - vnw);
  const float cs = c2.z * (vc - vs) + c2.w * (ve + vse - vw - vsw);
  return -a * (ce - cw) - b * (cn - cs);
}

// ------------------------------------------------------------------ BiCGStab
// Right-preconditioned BiCGStab (van der Vorst) for J x = b with device
// scalars; k.done (read by every kernel, including the V-cycle's) stops it.
struct MsKsp {
  KspState k;  // k.done: every kernel of the inner solve returns at once
  double rho, alpha, omega, beta, rnorm0, ttol, rnorm, rtol, atol;
  int its, max_it, reason, first;
};

enum { MSK_CONVERGED_RTOL = 2, MSK_CONVERGED_ATOL = 3, MSK_DIVERGED_ITS = -3, MSK_DIVERGED_BREAKDOWN = -5,
       MSK_DIVERGED_NANORINF = -9 };

__device__ __forceinline__ bool msk_done(const MsKsp *st) { return __ldcg(&st->k.done) != 0; }

__device__ __forceinline__ void msk_stop(MsKsp *st, int reason) {
  st->reason = reason;
  st->k.done = 1;
}

struct InitFin {
  MsKsp *st;
  __device__ void operator()(const double *s) const {
    st->rho = s[0];
    st->rnorm0 = st->rnorm = sqrt(s[0]);
    st->ttol = fmax(st->rtol * st->rnorm0, st->atol);
    st->its = 0;
    st->first = 1;
    st->reason = 0;
    st->k.done = 0;
    st->k.loops = 0;  // bodies of the device loop, counted per inner solve
    if (!(st->rnorm0 > st->ttol)) msk_stop(st, isfinite(st->rnorm0) ? MSK_CONVERGED_ATOL : MSK_DIVERGED_NANORINF);
  }
};

// r = b, rhat = b, x = p = v = 0; rho = b.b
__global__ void __launch_bounds__(256) k_bi_init(Geom g, MsKsp *st, const float *__restrict__ b, float *__restrict__ r,
                                                 float *__restrict__ rh, float *__restrict__ x, float *__restrict__ p,
                                                 float *__restrict__ v, Reducer red) {
  MS_NODE_BEGIN
  double acc = 0.0;
  if (in_) {
    const float bb = b[n];
    r[n] = bb;
    rh[n] = bb;
    x[n] = 0.f;
    p[n] = 0.f;
    v[n] = 0.f;
    acc = (double)bb * bb;
  }
  double v1[1] = {acc};
  ms_reduce<1>(v1, red, InitFin{st});
}

// p = r (first iteration) or r + beta (p - omega v)
__global__ void __launch_bounds__(256) k_bi_p(Geom g, MsKsp *st, const float *__restrict__ r, float *__restrict__ p,
                                              const float *__restrict__ v) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  if (!in_) return;
  if (st->first) {
    p[n] = r[n];
  } else {
    const float be = (float)st->beta, om = (float)st->omega;
    p[n] = fmaf(be, fmaf(-om, v[n], p[n]), r[n]);
  }
}

// out = M in: the V-cycle's result inside, in itself on boundary rows (z null: no preconditioner)
// Obstacle: the Poisson V-cycle's result everywhere but on the active set
// (boundary rows of its Jacobian are Poisson's too).
__global__ void __launch_bounds__(256) k_bi_pcout(Geom g, int model, const float4 *__restrict__ C1, MsKsp *st,
                                                  const float *__restrict__ z, const float *__restrict__ in,
                                                  float *__restrict__ out) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  if (!in_) return;
  bool use_z;
  if (model == FISHGPU_NL_OBSTACLE) use_z = node && z && C1[n].x == 0.f;
  else use_z = node && z && !ms_bdry(g, i, j);
  out[n] = use_z ? z[n] : in[n];
}

struct AlphaFin {
  MsKsp *st;
  __device__ void operator()(const double *s) const {
    if (!(s[0] != 0.0) || !isfinite(s[0])) {
      msk_stop(st, isfinite(s[0]) ? MSK_DIVERGED_BREAKDOWN : MSK_DIVERGED_NANORINF);
      return;
    }
    st->alpha = st->rho / s[0];
  }
};

struct OmegaFin {
  MsKsp *st;
  __device__ void operator()(const double *s) const { st->omega = s[1] > 0.0 ? s[0] / s[1] : 0.0; }
};

// v = J ph; rhat.v -> alpha
__global__ void __launch_bounds__(256) k_bi_jv1(Geom g, int model, MsKsp *st, float a, float b, const float4 *__restrict__ C1,
                                                const float4 *__restrict__ C2, const float *__restrict__ ph,
                                                float *__restrict__ v, const float *__restrict__ rh, Reducer red) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  double acc = 0.0;
  if (in_) {
    const float o = node ? ms_jv_node(g, model, i, j, n, a, b, C1, C2, ph) : 0.f;
    v[n] = o;
    acc = (double)rh[n] * o;
  }
  double v1[1] = {acc};
  ms_reduce<1>(v1, red, AlphaFin{st});
}

// s = r - alpha v
__global__ void __launch_bounds__(256) k_bi_s(Geom g, MsKsp *st, const float *__restrict__ r,
                                              const float *__restrict__ v, float *__restrict__ s) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  if (!in_) return;
  s[n] = fmaf(-(float)st->alpha, v[n], r[n]);
}

// t = J sh; t.s, t.t -> omega
__global__ void __launch_bounds__(256) k_bi_jv2(Geom g, int model, MsKsp *st, float a, float b, const float4 *__restrict__ C1,
                                                const float4 *__restrict__ C2, const float *__restrict__ sh,
                                                float *__restrict__ t, const float *__restrict__ s, Reducer red) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  double ts = 0.0, tt = 0.0;
  if (in_) {
    const float o = node ? ms_jv_node(g, model, i, j, n, a, b, C1, C2, sh) : 0.f;
    t[n] = o;
    ts = (double)o * s[n];
    tt = (double)o * o;
  }
  double v2[2] = {ts, tt};
  ms_reduce<2>(v2, red, OmegaFin{st});
}

struct XrFin {
  MsKsp *st;
  __device__ void operator()(const double *s) const {
    st->its += 1;
    st->first = 0;
    st->rnorm = sqrt(s[0]);
    if (!isfinite(st->rnorm)) msk_stop(st, MSK_DIVERGED_NANORINF);
    else if (st->rnorm <= st->ttol) msk_stop(st, st->rnorm < st->atol ? MSK_CONVERGED_ATOL : MSK_CONVERGED_RTOL);
    else if (st->its >= st->max_it) msk_stop(st, MSK_DIVERGED_ITS);
    else if (st->omega == 0.0 || s[1] == 0.0) msk_stop(st, MSK_DIVERGED_BREAKDOWN);
    else {
      st->beta = (s[1] / st->rho) * (st->alpha / st->omega);
      st->rho = s[1];
    }
  }
};

// x += alpha ph + omega sh; r = s - omega t; r.r, rhat.r
__global__ void __launch_bounds__(256) k_bi_xr(Geom g, MsKsp *st, const float *__restrict__ ph,
                                               const float *__restrict__ sh, const float *__restrict__ s,
                                               const float *__restrict__ t, const float *__restrict__ rh,
                                               float *__restrict__ x, float *__restrict__ r, Reducer red) {
  if (msk_done(st)) return;
  MS_NODE_BEGIN
  double rr = 0.0, hr = 0.0;
  if (in_) {
    const float al = (float)st->alpha, om = (float)st->omega;
    x[n] = fmaf(om, sh[n], fmaf(al, ph[n], x[n]));
    const float rn = fmaf(-om, t[n], s[n]);
    r[n] = rn;
    rr = (double)rn * rn;
    hr = (double)rh[n] * rn;
  }
  double v2[2] = {rr, hr};
  ms_reduce<2>(v2, red, XrFin{st});
}

// The whole BiCGStab solve of a small grid in ONE block: the iteration of
// k_bi_p .. k_bi_xr above, each kernel a phase of the block (same operations
// on every node), the preconditioner the exact coarse solve that is the whole
// Poisson V-cycle of a grid with one multigrid level (coarse_solve_block), the
// dot products summed over the block's threads in a fixed order.  The inner
// solve of such a grid is ~20 launches per iteration of almost no work each;
// here it is one launch.  Same finalisers, so the state the host reads (its,
// reason) means the same; the dot products are summed in another order than
// the multi-block kernels', so iterates differ from theirs by rounding.
struct BiCoarse {
  Geom g;
  const float *S0, *S1, *ilam;
  float *work, *z;
  int n0, n1, smem;
  float dinv;
};

// Compensated FP32 dot products for the one-block BiCGStab (Ogita, Rump and
// Oishi, "Accurate sum and dot product", 2005: TwoProduct by FMA, Knuth's
// TwoSum): each partial is a pair (s, c) whose sum carries about twice the
// FP32 precision, close to the FP64 accumulation it replaces.  On one SM an
// FP64 warp instruction takes ~17 issue cycles, so the FP64 accumulation and
// shuffle tree cost microseconds per dot product (ncu: FP64 pipe 31% busy);
// plain FP32 sums instead cost the obstacle problem 4% more inner
// iterations.  The _rn intrinsics keep the compiler from contracting the
// error terms into FMAs.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x) {
  const float t = __fadd_rn(s, x);
  const float bp = __fsub_rn(t, s);
  c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp)));
  s = t;
}
__device__ __forceinline__ void dot2_acc(float &s, float &c, float a, float b) {
  const float p = __fmul_rn(a, b);
  two_sum_acc(s, c, p);
  c = __fadd_rn(c, fmaf(a, b, -p));
}

// Block sum of the pairs: the warp tree combines pairs (TwoSum), each warp's
// s + c enters FP64, the warps are summed in FP64 in warp order
// (deterministic); the result in thread 0.
template <int NV>
__device__ __forceinline__ void bi_block_sum(float (&s)[NV], float (&c)[NV], double (&out)[NV]) {
  __shared__ double red_f[NV][32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const float s2 = __shfl_down_sync(0xffffffffu, s[q], o), c2 = __shfl_down_sync(0xffffffffu, c[q], o);
      two_sum_acc(s[q], c[q], s2);
      c[q] = __fadd_rn(c[q], c2);
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) red_f[q][wid] = (double)s[q] + (double)c[q];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = lane < nw ? red_f[q][lane] : 0.0;
    warp_sum<NV>(out);
  }
  __syncthreads();
}

// vsm_off >= 0: the ten work vectors (and the preconditioner's output z)
// live in the dynamic shared memory from that offset for the whole solve,
// so every phase waits on shared memory instead of an L2 round trip; x is
// copied out at the end (the only vector the Newton step reads).  The
// coarse solve's tables are staged in shared memory once per launch.
__global__ void __launch_bounds__(1024) k_bi_block(Geom g, int model, float a, float b, const float4 *__restrict__ C1,
                                                   const float4 *__restrict__ C2, const float *__restrict__ bv,
                                                   float *r, float *rh, float *p, float *v, float *s, float *t,
                                                   float *x_out, float *ph, float *sh, MsKsp *st, BiCoarse pc,
                                                   int use_pc, int max_iters, int vsm_off) {
  extern __shared__ __align__(16) unsigned char bi_sm[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int N = g.pitch * g.my;  // every element of the padded grid, as the node kernels cover it
  float *x = x_out, *zc = pc.z;
  if (vsm_off >= 0) {
    float *q0 = reinterpret_cast<float *>(bi_sm + vsm_off);
    r = q0;
    rh = q0 + N;
    p = q0 + 2 * N;
    v = q0 + 3 * N;
    s = q0 + 4 * N;
    t = q0 + 5 * N;
    x = q0 + 6 * N;
    ph = q0 + 7 * N;
    sh = q0 + 8 * N;
    zc = q0 + 9 * N;
    for (int q = tid; q < N; q += nt) zc[q] = 0.f;  // the coarse solve writes z's interior and boundary nodes
  }
  if (use_pc && pc.smem) coarse_stage<2, float>(pc.S0, pc.S1, pc.S1, pc.ilam, pc.n0, pc.n1, 1, bi_sm);
  __syncthreads();
  auto done = [&]() { return *(volatile int *)&st->k.done != 0; };
  // z = M in into out (k_bi_pcout): the Poisson solve inside, `in` elsewhere
  auto precondition = [&](const float *in, float *out) {
    if (use_pc) {  // smem 2: the tables were staged at the start
      coarse_solve_block<2, float>(pc.g, in, zc, pc.S0, pc.S1, pc.S1, pc.ilam, pc.work, pc.n0, pc.n1, 1,
                                   pc.smem ? 2 : 0, pc.dinv, bi_sm);
      __syncthreads();
    }
    for (int q = tid; q < N; q += nt) {
      const int i = q % g.pitch, j = q / g.pitch;
      const bool node = i < g.mx;
      bool use_z;
      if (model == FISHGPU_NL_OBSTACLE) use_z = node && use_pc && C1[q].x == 0.f;
      else use_z = node && use_pc && !ms_bdry(g, i, j);
      out[q] = use_z ? zc[q] : in[q];
    }
    __syncthreads();
  };
  {  // k_bi_init: r = b, rhat = b, x = p = v = 0; rho = b.b
    float as[1] = {0.f}, ac[1] = {0.f};
    double acc[1];
    for (int q = tid; q < N; q += nt) {
      const float bb = bv[q];
      r[q] = bb;
      rh[q] = bb;
      x[q] = 0.f;
      p[q] = 0.f;
      v[q] = 0.f;
      dot2_acc(as[0], ac[0], bb, bb);
    }
    bi_block_sum<1>(as, ac, acc);
    if (tid == 0) InitFin{st}(acc);
    __syncthreads();
  }
  // max_iters: the iterations the device loop's cap would allow; a solve
  // still running then ends with its state not done (the host reports it)
  for (int iter = 0; !done() && iter < max_iters; iter++) {
    {  // k_bi_p
      const bool first = *(volatile int *)&st->first != 0;
      const float be = (float)*(volatile double *)&st->beta, om = (float)*(volatile double *)&st->omega;
      for (int q = tid; q < N; q += nt) p[q] = first ? r[q] : fmaf(be, fmaf(-om, v[q], p[q]), r[q]);
      __syncthreads();
    }
    precondition(p, ph);
    {  // k_bi_jv1: v = J ph, rhat.v -> alpha
      float as[1] = {0.f}, ac[1] = {0.f};
      double acc[1];
      for (int q = tid; q < N; q += nt) {
        const int i = q % g.pitch, j = q / g.pitch;
        const float o = i < g.mx ? ms_jv_node(g, model, i, j, q, a, b, C1, C2, ph) : 0.f;
        v[q] = o;
        dot2_acc(as[0], ac[0], rh[q], o);
      }
      bi_block_sum<1>(as, ac, acc);
      if (tid == 0) AlphaFin{st}(acc);
      __syncthreads();
    }
    if (done()) break;
    {  // k_bi_s
      const float al = (float)*(volatile double *)&st->alpha;
      for (int q = tid; q < N; q += nt) s[q] = fmaf(-al, v[q], r[q]);
      __syncthreads();
    }
    precondition(s, sh);
    {  // k_bi_jv2: t = J sh; t.s, t.t -> omega
      float as[2] = {0.f, 0.f}, ac[2] = {0.f, 0.f};
      double acc[2];
      for (int q = tid; q < N; q += nt) {
        const int i = q % g.pitch, j = q / g.pitch;
        const float o = i < g.mx ? ms_jv_node(g, model, i, j, q, a, b, C1, C2, sh) : 0.f;
        t[q] = o;
        dot2_acc(as[0], ac[0], o, s[q]);
        dot2_acc(as[1], ac[1], o, o);
      }
      bi_block_sum<2>(as, ac, acc);
      if (tid == 0) OmegaFin{st}(acc);
      __syncthreads();
    }
    {  // k_bi_xr: x += alpha ph + omega sh; r = s - omega t; r.r, rhat.r
      const float al = (float)*(volatile double *)&st->alpha, om = (float)*(volatile double *)&st->omega;
      float as[2] = {0.f, 0.f}, ac[2] = {0.f, 0.f};
      double acc[2];
      for (int q = tid; q < N; q += nt) {
        x[q] = fmaf(om, sh[q], fmaf(al, ph[q], x[q]));
        const float rn = fmaf(-om, t[q], s[q]);
        r[q] = rn;
        dot2_acc(as[0], ac[0], rn, rn);
        dot2_acc(as[1], ac[1], rh[q], rn);
      }
      bi_block_sum<2>(as, ac, acc);
      if (tid == 0) XrFin{st}(acc);
      __syncthreads();
    }
  }
  if (vsm_off >= 0) {  // the Newton step reads x
    __syncthreads();
    for (int q = tid; q < N; q += nt) x_out[q] = x[q];
  }
}

// The whole BiCGStab solve of a multigrid grid in ONE cooperative launch (one
// block of 512 threads per SM at most): the iteration of k_bi_p .. k_bi_xr,
// each kernel a phase ended by a grid barrier, the preconditioner the fish
// solver's FP32 V-cycle run by persist_vcycle (the launch-per-phase
// V-cycle's values).  Two fusions save a phase each: p = r + beta (p - omega
// v) (k_bi_p) and s = r - alpha v (k_bi_s) are formed on the fly as the
// V-cycle's fine right-hand side and stored by its last pass, which also
// stores ph = M p and sh = M s (k_bi_pcout).  Every block sums the dot
// products' block partials in the same order and runs the same finalisers on
// its own copy of the state (block 0 writes it back), so the iteration is
// the launch-per-phase one up to the order of the dot products' sums; each
// point runs the same operations.  Grids whose V-cycle kernels are too small
// to hide a launch each (the inner iteration is ~60 launches) take this form.
struct BiPersist {
  Geom g;  // the fine grid, the fish solver's padded layout
  int model;
  float ja, jb;
  const float4 *C1, *C2;
  const float *b;
  float *r, *rh, *p, *v, *s, *t, *x, *ph, *sh;
  MsKsp *st;
  int max_iters;  // iterations before the launch gives up (the host reports a timeout)
};

__global__ void __launch_bounds__(512, 1) k_bi_persist(PersistArgs<float> a, BiPersist q) {
  extern __shared__ __align__(16) unsigned char fg_tail_sm[];
  __shared__ PersistShared<float> ps;
  __shared__ MsKsp mk;
  const int tid = threadIdx.x;
  if (tid == 0) mk = *q.st;
  persist_setup<2, float>(a, ps, fg_tail_sm);
  const Geom &g = q.g;
  int slot = 0;
  auto each = [&](auto &&f) { persist_each<2>(g, f); };
  auto sync = [&]() { return grid_sync(&ps.gb); };
  // M in = the V-cycle's value inside, in itself on boundary rows (k_bi_pcout)
  auto use_z = [&](long long n, int i, int j) -> bool {
    return q.model == FISHGPU_NL_OBSTACLE ? q.C1[n].x == 0.f : !ms_bdry(g, i, j);
  };
  auto sync_first = [&](float) -> int { return sync() ? 1 : 0; };
  bool ok = true;
  {  // k_bi_init: r = b, rhat = b, x = p = v = 0; rho = b.b.  Every vector's padding is zeroed
     // here and never written again (the node kernels keep it at 0).
    const long long tot = (long long)g.plane;
    const long long G = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + tid; e < tot; e += G)
      if ((int)(e % g.pitch) >= g.mx) {
        q.r[e] = q.rh[e] = q.p[e] = q.v[e] = q.s[e] = q.t[e] = q.x[e] = q.ph[e] = q.sh[e] = 0.f;
      }
    double acc = 0.0;
    each([&](long long n, int, int, int) {
      const float bb = q.b[n];
      q.r[n] = bb;
      q.rh[n] = bb;
      q.x[n] = 0.f;
      q.p[n] = 0.f;
      q.v[n] = 0.f;
      acc += (double)bb * bb;
    });
    double v1[1] = {acc};
    ok = grid_reduce_fn<1>(v1, a.part, slot, &ps.gb, [&](double *t) { InitFin{&mk}(t); });
  }
  int it = 0;
  while (ok && !mk.k.done && it < q.max_iters) {
    it++;
    {  // p (k_bi_p) formed on the fly; ph = M p (k_bi_pcout)
      const bool first = mk.first != 0;
      const float be = (float)mk.beta, om = (float)mk.omega;
      auto pf = [&](long long m) -> float { return first ? q.r[m] : fmaf(be, fmaf(-om, q.v[m], q.p[m]), q.r[m]); };
      auto last = [&](long long n, int i, int j, int, float z, float bv) {
        q.p[n] = bv;
        q.ph[n] = use_z(n, i, j) ? z : bv;
      };
      if (!(ok = persist_vcycle<2, float>(a, ps, fg_tail_sm, pf, sync_first, last, sync))) break;
    }
    {  // k_bi_jv1: v = J ph; rhat.v -> alpha
      double acc = 0.0;
      each([&](long long n, int i, int j, int) {
        const float o = ms_jv_node(g, q.model, i, j, n, q.ja, q.jb, q.C1, q.C2, q.ph);
        q.v[n] = o;
        acc += (double)q.rh[n] * o;
      });
      double v1[1] = {acc};
      if (!(ok = grid_reduce_fn<1>(v1, a.part, slot, &ps.gb, [&](double *t) { AlphaFin{&mk}(t); }))) break;
    }
    if (mk.k.done) break;
    {  // s = r - alpha v (k_bi_s) formed on the fly; sh = M s
      const float al = (float)mk.alpha;
      auto sf = [&](long long m) -> float { return fmaf(-al, q.v[m], q.r[m]); };
      auto last = [&](long long n, int i, int j, int, float z, float bv) {
        q.s[n] = bv;
        q.sh[n] = use_z(n, i, j) ? z : bv;
      };
      if (!(ok = persist_vcycle<2, float>(a, ps, fg_tail_sm, sf, sync_first, last, sync))) break;
    }
    {  // k_bi_jv2: t = J sh; t.s, t.t -> omega
      double ts = 0.0, tt = 0.0;
      each([&](long long n, int i, int j, int) {
        const float o = ms_jv_node(g, q.model, i, j, n, q.ja, q.jb, q.C1, q.C2, q.sh);
        q.t[n] = o;
        ts += (double)o * q.s[n];
        tt += (double)o * o;
      });
      double v2[2] = {ts, tt};
      if (!(ok = grid_reduce_fn<2>(v2, a.part, slot, &ps.gb, [&](double *t) { OmegaFin{&mk}(t); }))) break;
    }
    {  // k_bi_xr: x += alpha ph + omega sh; r = s - omega t; r.r, rhat.r
      const float al = (float)mk.alpha, om = (float)mk.omega;
      double rr = 0.0, hr = 0.0;
      each([&](long long n, int, int, int) {
        q.x[n] = fmaf(om, q.sh[n], fmaf(al, q.ph[n], q.x[n]));
        const float rn = fmaf(-om, q.t[n], q.s[n]);
        q.r[n] = rn;
        rr += (double)rn * rn;
        hr += (double)q.rh[n] * rn;
      });
      double v2[2] = {rr, hr};
      if (!(ok = grid_reduce_fn<2>(v2, a.part, slot, &ps.gb, [&](double *t) { XrFin{&mk}(t); }))) break;
    }
  }
  if (blockIdx.x == 0 && tid == 0) *q.st = mk;  // not done: the iteration cap (or a barrier) ended it
}

// ------------------------------------------------------------------ Newton helpers
// b = F / fnorm (FP32); 0 on the active set of the obstacle problem (C1.x)
__global__ void __launch_bounds__(256) k_ms_demote(Geom g, int model, const float4 *__restrict__ C1,
                                                   const double *__restrict__ F, double inv, float *__restrict__ b) {
  MS_NODE_BEGIN
  if (in_) b[n] = (model == FISHGPU_NL_OBSTACLE && node && C1[n].x != 0.f) ? 0.f : (float)(F[n] * inv);
}

// t = J x (FP32); out = {F.t, x.x}
__global__ void __launch_bounds__(256) k_ms_slope(Geom g, int model, float a, float b, const float4 *__restrict__ C1,
                                                  const float4 *__restrict__ C2, const float *__restrict__ x,
                                                  const double *__restrict__ F, Reducer red, double *out) {
  MS_NODE_BEGIN
  double ft = 0.0, xx = 0.0;
  if (node) {
    const float o = ms_jv_node(g, model, i, j, n, a, b, C1, C2, x);
    ft = (model == FISHGPU_NL_OBSTACLE && C1[n].x != 0.f) ? 0.0 : F[n] * (double)o;
    xx = (double)x[n] * x[n];
  }
  double v2[2] = {ft, xx};
  ms_reduce<2>(v2, red, Store2Fin{out});
}

// W = u - c x, projected onto u >= psi for the obstacle problem
__global__ void __launch_bounds__(256) k_ms_trial(Geom g, int model, const double *__restrict__ u, double c,
                                                  const float *__restrict__ x, double *__restrict__ W) {
  MS_NODE_BEGIN
  if (!in_) return;
  double w = node ? u[n] - c * (double)x[n] : 0.0;
  if (node && model == FISHGPU_NL_OBSTACLE) w = fmax(w, obs_psi(-2.0 + i * g.h[0], -2.0 + j * g.h[1]));
  W[n] = w;
}

// u = max(u, psi) (SNESVIProjectOntoBounds at the start of a VI solve)
__global__ void __launch_bounds__(256) k_obs_project(Geom g, double *__restrict__ u) {
  MS_NODE_BEGIN
  if (node) u[n] = fmax(u[n], obs_psi(-2.0 + i * g.h[0], -2.0 + j * g.h[1]));
}

// the obstacle report: sum and max of |u - u_exact| (sel 0), or the number of
// active nodes (sel 1: u <= psi + zerotol and F > 0, obstacle.c:184-213)
__global__ void __launch_bounds__(256) k_obs_report(Geom g, int sel, const double *__restrict__ u,
                                                    const double *__restrict__ F, double *part, int cap);

// mode 0: u = g on the boundary and 0 inside (InitialState ZEROS with g,
// minimal.c:155-157); 1: g everywhere (FormExactFromG, minimal.c:193-208);
// 2: 0 everywhere (VecSet(u,0), bratu2D.c:133); padding 0
__global__ void __launch_bounds__(256) k_ms_init(Geom g, MsP P, int mode, double *__restrict__ u) {
  MS_NODE_BEGIN
  if (!in_) return;
  u[n] = (node && mode != 2 && (mode == 1 || ms_bdry(g, i, j))) ? ms_gd(P, i * g.h[0], j * g.h[1]) : 0.0;
}

// DMDA Q1 interpolation coarse -> fine, ratio 2
__global__ void __launch_bounds__(256) k_ms_interp(Geom gc, const double *__restrict__ uc, Geom g,
                                                   double *__restrict__ uf) {
  MS_NODE_BEGIN
  if (!in_) return;
  if (!node) {
    uf[n] = 0.0;
    return;
  }
  const int i0 = i / 2, j0 = j / 2, i1 = i0 + (i & 1), j1 = j0 + (j & 1);
  const long long P = gc.pitch;
  uf[n] = 0.25 * (uc[j0 * P + i0] + uc[j0 * P + i1] + uc[j1 * P + i0] + uc[j1 * P + i1]);
}

// Per-block (sum, min, max) of a node quantity, combined by k_ms_fin3.
__device__ __forceinline__ void block_3(double &s, double &lo, double &hi, double *part, int cap) {
  __shared__ double sm[3][32];
  const int tid = threadIdx.x + blockDim.x * threadIdx.y, nt = blockDim.x * blockDim.y;
  const int lane = tid & 31, wid = tid >> 5, nw = (nt + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    sm[0][wid] = s;
    sm[1][wid] = lo;
    sm[2][wid] = hi;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, b = INFINITY, c = -INFINITY;
    for (int w = 0; w < nw; w++) {
      a += sm[0][w];
      b = fmin(b, sm[1][w]);
      c = fmax(c, sm[2][w]);
    }
    const int bid = blockIdx.x + gridDim.x * blockIdx.y;
    part[bid] = a;
    part[cap + bid] = b;
    part[2 * cap + bid] = c;
  }
}

__global__ void __launch_bounds__(256) k_ms_fin3(const double *__restrict__ part, int cap, int nb, double *out) {
  __shared__ double sm[3][256];
  const int t = threadIdx.x;
  double a = 0.0, b = INFINITY, c = -INFINITY;
  for (int k = t; k < nb; k += blockDim.x) {
    a += part[k];
    b = fmin(b, part[cap + k]);
    c = fmax(c, part[2 * cap + k]);
  }
  sm[0][t] = a;
  sm[1][t] = b;
  sm[2][t] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s) {
      sm[0][t] += sm[0][t + s];
      sm[1][t] = fmin(sm[1][t], sm[1][t + s]);
      sm[2][t] = fmax(sm[2][t], sm[2][t + s]);
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = sm[0][0];
    out[1] = sm[1][0];
    out[2] = sm[2][0];
  }
}

// MSEMonitor, minimal.c:286-362: surface area of the Q1 interpolant and the
// range of the diffusivity at Gauss-Legendre points; cell (i,j) has its NE
// corner at node (i,j)
__global__ void __launch_bounds__(256) k_ms_area(Geom g, double q, int degree, const double *__restrict__ u,
                                                 double *part, int cap) {
  const double xi2 = 0.57735026918962576451, xi3 = 0.77459666924148337704;
  const int nq = degree < 1 ? 1 : degree > 3 ? 3 : degree;
  MS_NODE_BEGIN
  double s = 0.0, lo = INFINITY, hi = -INFINITY;
  if (node && i > 0 && j > 0) {
    const double hx = g.h[0], hy = g.h[1], xi_ = i * hx, yj = j * hy;
    const double u00 = u[n - g.pitch - 1], u10 = u[n - g.pitch], u01 = u[n - 1], u11 = u[n];
    for (int r = 0; r < nq; r++) {
      const double pr = nq == 1 ? 0.0 : nq == 2 ? (r ? xi2 : -xi2) : (r == 0 ? -xi3 : r == 1 ? 0.0 : xi3);
      const double wr = nq == 1 ? 2.0 : nq == 2 ? 1.0 : (r == 1 ? 8.0 / 9.0 : 5.0 / 9.0);
      const double x = xi_ - hx + hx * 0.5 * (pr + 1.0);
      for (int t = 0; t < nq; t++) {
        const double pt = nq == 1 ? 0.0 : nq == 2 ? (t ? xi2 : -xi2) : (t == 0 ? -xi3 : t == 1 ? 0.0 : xi3);
        const double wt = nq == 1 ? 2.0 : nq == 2 ? 1.0 : (t == 1 ? 8.0 / 9.0 : 5.0 / 9.0);
        const double y = yj - hy + hy * 0.5 * (pt + 1.0);
        const double ux = ((u11 - u01) * (y - (yj - hy)) + (u10 - u00) * (yj - y)) / (hx * hy);
        const double uy = ((u11 - u10) * (x - (xi_ - hx)) + (u01 - u00) * (xi_ - x)) / (hx * hy);
        const double W = ux * ux + uy * uy, D = ms_diffusivity(1.0 + W, q);
        lo = fmin(lo, D);
        hi = fmax(hi, D);
        s += wr * wt * sqrt(1.0 + W);
      }
    }
  }
  block_3(s, lo, hi, part, cap);
}

// max |u - g| over the nodes (error against the catenoid, minimal.c:170-184)
__global__ void __launch_bounds__(256) k_ms_err(Geom g, MsP P, const double *__restrict__ u, double *part, int cap) {
  MS_NODE_BEGIN
  double s = 0.0, lo = INFINITY, hi = 0.0;
  if (node) hi = fabs(u[n] - ms_gd(P, i * g.h[0], j * g.h[1]));
  block_3(s, lo, hi, part, cap);
}

__global__ void __launch_bounds__(256) k_obs_report(Geom g, int sel, const double *__restrict__ u,
                                                    const double *__restrict__ F, double *part, int cap) {
  MS_NODE_BEGIN
  double s = 0.0, lo = INFINITY, hi = 0.0;
  if (node) {
    const double x = -2.0 + i * g.h[0], y = -2.0 + j * g.h[1];
    if (sel == 0) {
      s = fabs(u[n] - obs_uexact(x, y));
      hi = s;
    } else {
      s = (u[n] <= obs_psi(x, y) + OBS_ZEROTOL && F[n] > 0.0) ? 1.0 : 0.0;
    }
  }
  block_3(s, lo, hi, part, cap);
}

// The call-back: dense whole-grid arrays, owned box
__global__ void __launch_bounds__(256) k_ms_funclocal(Geom g, MsP P, int xs, int ys, int xm, int ym,
                                                      const double *__restrict__ u, double *__restrict__ F) {
  const int i = xs + blockIdx.x * blockDim.x + threadIdx.x, j = ys + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= xs + xm || j >= ys + ym) return;
  const long long n = (long long)j * g.mx + i;
  F[n] = ms_bdry(g, i, j) ? u[n] - ms_gd(P, i * g.h[0], j * g.h[1])
         : P.model == FISHGPU_NL_BRATU ? lb_f_interior(g, P, u, g.mx, i, j) : ms_f_interior(g, P, u, g.mx, i, j);
}

}  // namespace fg

using namespace fg;

// ------------------------------------------------------------------ host
namespace {

struct MsLevel {
  fishgpu_solver *P = nullptr;  // Poisson multigrid of this grid (geometry, V-cycle)
  Geom g;
  double *gt = nullptr;  // boundary-data table (k_ms_gtab), minimal surface and Bratu
  int gtm = 0;
  long long N = 0;
  dim3 grid, block;
  double *u = nullptr, *F = nullptr, *W = nullptr, *G = nullptr;
  float4 *C1 = nullptr, *C2 = nullptr;
  float *b = nullptr, *r = nullptr, *rh = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr,
        *x = nullptr, *ph = nullptr, *sh = nullptr;
  cudaGraphExec_t g_init = nullptr, g_iter = nullptr;
  cudaGraphExec_t g_loop = nullptr;  // g_iter's body repeated on the device until the inner solve stops
  long long n_loop = 0;
  int giters = 2;
  bool block1 = false;  // the inner solve is one launch of k_bi_block
  bool persist = false;  // the inner solve is one cooperative launch of k_bi_persist
  PersistArgs<float> pa{};
  int pblocks = 0;
  size_t psmem = 0;
  BiCoarse bc{};
  int use_pc = 0;
  int max_iters = 0;
  size_t bsm = 0;    // its dynamic shared memory
  int vsm_off = -1;  // offset of its vectors there (-1: in global memory)
};

}  // namespace

struct fishgpu_ms_solver_s {
  fishgpu_ms_opts o;
  MsP P;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<MsLevel> lev;
  Reducer red{};
  double *part3 = nullptr;
  int cap = 0;
  MsKsp *st = nullptr, *st_h = nullptr;
  double *dval = nullptr, *hval = nullptr;
  std::vector<void *> allocs;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evg = nullptr, evg2 = nullptr;
  long long nfuncs = 0;  // residual evaluations of the current solve
};

#define MS_CK(x)                                   \
  do {                                             \
    if ((x) != cudaSuccess) {                      \
      cudaGetLastError();                          \
      return FISHGPU_ERR_CUDA;                     \
    }                                              \
  } while (0)

template <typename T>
static int ms_alloc(fishgpu_ms_solver *S, T **p, long long n) {
  void *q = nullptr;
  if (cudaMalloc(&q, sizeof(T) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) {
    cudaGetLastError();
    return FISHGPU_ERR_NOMEM;
  }
  S->allocs.push_back(q);
  *p = (T *)q;
  return FISHGPU_OK;
}

// The problem parameters with the boundary-data table of grid L
static MsP level_params(const fishgpu_ms_solver *S, const MsLevel &L) {
  MsP P = S->P;
  P.gt = L.gt;
  P.gtm = L.gtm;
  return P;
}

static int ms_levels_for(int mx, int my) {
  int l = 1;
  while (mx > 3 && my > 3 && (mx - 1) % 2 == 0 && (my - 1) % 2 == 0) {
    mx = (mx - 1) / 2 + 1;
    my = (my - 1) / 2 + 1;
    l++;
  }
  return l;
}

// One BiCGStab iteration enqueued on S->stream (captured into a graph).
static void enq_bicg_iter(fishgpu_ms_solver *S, MsLevel &L) {
  cudaStream_t s = S->stream;
  const Geom &g = L.g;
  const float a = (float)(g.h[1] / g.h[0]), b = (float)(g.h[0] / g.h[1]);
  const bool mg = S->o.pc_type == FISHGPU_PC_MG;
  k_bi_p<<<L.grid, L.block, 0, s>>>(g, S->st, L.r, L.p, L.v);
  const float *z = mg ? solver_vcycle32(L.P, L.p, &S->st->k) : nullptr;
  k_bi_pcout<<<L.grid, L.block, 0, s>>>(g, S->P.model, L.C1, S->st, z, L.p, L.ph);
  k_bi_jv1<<<L.grid, L.block, 0, s>>>(g, S->P.model, S->st, a, b, L.C1, L.C2, L.ph, L.v, L.rh, S->red);
  k_bi_s<<<L.grid, L.block, 0, s>>>(g, S->st, L.r, L.v, L.s);
  z = mg ? solver_vcycle32(L.P, L.s, &S->st->k) : nullptr;
  k_bi_pcout<<<L.grid, L.block, 0, s>>>(g, S->P.model, L.C1, S->st, z, L.s, L.sh);
  k_bi_jv2<<<L.grid, L.block, 0, s>>>(g, S->P.model, S->st, a, b, L.C1, L.C2, L.sh, L.t, L.s, S->red);
  k_bi_xr<<<L.grid, L.block, 0, s>>>(g, S->st, L.ph, L.sh, L.s, L.t, L.rh, L.x, L.r, S->red);
}

static int capture(fishgpu_ms_solver *S, MsLevel &L, bool init, cudaGraphExec_t *out) {
  cudaGraph_t gr = nullptr;
  MS_CK(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
  if (init) {
    k_bi_init<<<L.grid, L.block, 0, S->stream>>>(L.g, S->st, L.b, L.r, L.rh, L.x, L.p, L.v, S->red);
  } else {
    for (int k = 0; k < L.giters; k++) enq_bicg_iter(S, L);
  }
  const cudaError_t e = cudaStreamEndCapture(S->stream, &gr);
  if (e != cudaSuccess || !gr) {
    cudaGetLastError();
    return FISHGPU_ERR_CUDA;
  }
  const cudaError_t e2 = cudaGraphInstantiate(out, gr, 0);
  cudaGraphDestroy(gr);
  if (e2 != cudaSuccess) {
    cudaGetLastError();
    return FISHGPU_ERR_CUDA;
  }
  return FISHGPU_OK;
}

static int read_vals(fishgpu_ms_solver *S, int n) {
  MS_CK(cudaMemcpyAsync(S->hval, S->dval, sizeof(double) * n, cudaMemcpyDeviceToHost, S->stream));
  MS_CK(cudaStreamSynchronize(S->stream));
  return FISHGPU_OK;
}

// F = F(u) and ||F||; ||u||^2 into *unorm2 when asked (the same launch)
static int residual(fishgpu_ms_solver *S, MsLevel &L, const double *u, double *F, double *fnorm,
                    double *unorm2 = nullptr) {
  S->nfuncs++;
  k_ms_resid<<<L.grid, L.block, 0, S->stream>>>(L.g, level_params(S, L), u, F, S->red, S->dval);
  MS_CK(cudaGetLastError());
  int rc = read_vals(S, 2);
  if (rc) return rc;
  *fnorm = sqrt(S->hval[0]);
  if (unorm2) *unorm2 = S->hval[1];
  return FISHGPU_OK;
}

static int area(fishgpu_ms_solver *S, MsLevel &L, const double *u, double out[3]) {
  const int nb = (int)(L.grid.x * L.grid.y);
  k_ms_area<<<L.grid, L.block, 0, S->stream>>>(L.g, S->P.q, S->o.monitor_degree, u, S->part3, S->cap);
  k_ms_fin3<<<1, 256, 0, S->stream>>>(S->part3, S->cap, nb, S->dval);
  MS_CK(cudaGetLastError());
  int rc = read_vals(S, 3);
  if (rc) return rc;
  out[0] = S->hval[0] * L.g.h[0] * L.g.h[1] / 4.0;
  out[1] = S->hval[1];
  out[2] = S->hval[2];
  return FISHGPU_OK;
}

// SNES reasons (PETSc values)
enum { SN_CONVERGED_FNORM_ABS = 2, SN_CONVERGED_FNORM_RELATIVE = 3, SN_CONVERGED_SNORM_RELATIVE = 4,
       SN_DIVERGED_FNORM_NAN = -4, SN_DIVERGED_MAX_IT = -5, SN_DIVERGED_LINE_SEARCH = -6 };

// Newton on one grid from L.u; fills the report row `k`.
static int newton(fishgpu_ms_solver *S, MsLevel &L, int k, fishgpu_ms_report *rep) {
  const fishgpu_ms_opts &o = S->o;
  cudaStream_t s = S->stream;
  const Geom &g = L.g;
  const float a = (float)(g.h[1] / g.h[0]), b = (float)(g.h[0] / g.h[1]);
  int rc;
  double fnorm = 0.0;
  if (S->P.model == FISHGPU_NL_OBSTACLE) k_obs_project<<<L.grid, L.block, 0, s>>>(g, L.u);
  if ((rc = residual(S, L, L.u, L.F, &fnorm))) return rc;
  rep->fnorm[k][0] = fnorm;
  if (o.monitor_degree > 0 && (rc = area(S, L, L.u, rep->area[k][0]))) return rc;
  const double ttol = o.rtol * fnorm;
  int reason = 0, its = 0;
  if (fnorm != fnorm) reason = SN_DIVERGED_FNORM_NAN;
  else if (fnorm < o.atol) reason = SN_CONVERGED_FNORM_ABS;
  // inner-solve parameters
  MsKsp h;
  memset(&h, 0, sizeof(h));
  h.rtol = o.ksp_rtol;
  h.atol = 0.0;
  h.max_it = o.ksp_max_it;
  MS_CK(cudaMemcpyAsync(S->st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  while (!reason) {
    if (its >= FISHGPU_MS_MAX_ITS) {
      reason = SN_DIVERGED_MAX_IT;
      break;
    }
    // J Y = F: coefficients at u, b = F/||F||, BiCGStab for x = J^-1 b, Y = ||F|| x
    k_ms_coef<<<L.grid, L.block, 0, s>>>(g, level_params(S, L), L.u, L.F, L.C1, L.C2);
    k_ms_demote<<<L.grid, L.block, 0, s>>>(g, S->P.model, L.C1, L.F, 1.0 / fnorm, L.b);
    MS_CK(cudaGetLastError());
    int kits = 0, kreason = 0;
    // the inner solve, then at once the slope's dot products (k_ms_slope): the
    // host reads them with the solver state in one round trip
    auto enq_slope = [&]() -> int {
      k_ms_slope<<<L.grid, L.block, 0, s>>>(g, S->P.model, a, b, L.C1, L.C2, L.x, L.F, S->red, S->dval);
      MS_CK(cudaGetLastError());
      MS_CK(cudaMemcpyAsync(S->hval, S->dval, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      return FISHGPU_OK;
    };
    if (L.block1) {
      const float ja = (float)(g.h[1] / g.h[0]), jb = (float)(g.h[0] / g.h[1]);
      k_bi_block<<<1, 1024, L.bsm, s>>>(g, S->P.model, ja, jb, L.C1, L.C2, L.b, L.r, L.rh, L.p, L.v, L.s, L.t,
                                        L.x, L.ph, L.sh, S->st, L.bc, L.use_pc, L.max_iters, L.vsm_off);
      MS_CK(cudaGetLastError());
      if ((rc = enq_slope())) return rc;
      MS_CK(cudaMemcpyAsync(S->st_h, S->st, sizeof(MsKsp), cudaMemcpyDeviceToHost, s));
      MS_CK(cudaStreamSynchronize(s));
      if (!S->st_h->k.done) return FISHGPU_ERR_TIMEOUT;  // the iteration cap ended it unfinished
    } else if (L.persist) {
      MS_CK(cudaMemsetAsync(L.pa.bar, 0, 2 * sizeof(unsigned), s));
      BiPersist q{g, S->P.model, a, b, L.C1, L.C2, L.b, L.r, L.rh, L.p, L.v, L.s, L.t, L.x, L.ph, L.sh, S->st,
                  L.max_iters};
      void *args[] = {&L.pa, &q};
      MS_CK(cudaLaunchCooperativeKernel((const void *)k_bi_persist, dim3(L.pblocks), dim3(512), args, L.psmem, s));
      if ((rc = enq_slope())) return rc;
      MS_CK(cudaMemcpyAsync(S->st_h, S->st, sizeof(MsKsp), cudaMemcpyDeviceToHost, s));
      MS_CK(cudaMemcpyAsync(S->hval + 7, L.pa.fault, sizeof(int), cudaMemcpyDeviceToHost, s));
      MS_CK(cudaStreamSynchronize(s));
      int fault = 0;
      memcpy(&fault, S->hval + 7, sizeof(int));
      if (fault) {  // a grid barrier gave up: the state is void; the next solve starts clean
        MS_CK(cudaMemsetAsync(L.pa.fault, 0, sizeof(int), s));
        MS_CK(cudaStreamSynchronize(s));
        return FISHGPU_ERR_TIMEOUT;
      }
      if (!S->st_h->k.done) return FISHGPU_ERR_TIMEOUT;  // the iteration cap ended it unfinished
    } else if (L.g_loop) {
      MS_CK(cudaGraphLaunch(L.g_init, s));
      MS_CK(cudaGraphLaunch(L.g_loop, s));
      if ((rc = enq_slope())) return rc;
      MS_CK(cudaMemcpyAsync(S->st_h, S->st, sizeof(MsKsp), cudaMemcpyDeviceToHost, s));
      MS_CK(cudaStreamSynchronize(s));
      if (!S->st_h->k.done) return FISHGPU_ERR_TIMEOUT;  // the capped device loop ended unfinished
    } else {  // the host-polled graph
      MS_CK(cudaGraphLaunch(L.g_init, s));
      for (;;) {
        MS_CK(cudaMemcpyAsync(S->st_h, S->st, sizeof(MsKsp), cudaMemcpyDeviceToHost, s));
        MS_CK(cudaStreamSynchronize(s));
        if (S->st_h->k.done) break;
        MS_CK(cudaGraphLaunch(L.g_iter, s));
      }
      if ((rc = enq_slope())) return rc;
      MS_CK(cudaStreamSynchronize(s));
    }
    kits = S->st_h->its;
    kreason = S->st_h->reason;
    rep->ksp_its[k][its] = kits;
    rep->ksp_reason[k][its] = kreason;
    rep->total_ksp_its += kits;
    // slope of ||F||^2/2 along -Y: -(F, J Y) = -||F|| (F, J x); ||Y|| = ||F|| ||x|| (read above)
    double initslope = -fnorm * S->hval[0];
    double ynorm = fnorm * sqrt(S->hval[1]);
    if (initslope > 0.0) initslope = -initslope;
    if (initslope == 0.0) initslope = -1.0;
    double scale = fnorm;  // Y = scale * x
    if (ynorm > 1e8) {     // maxstep
      scale *= 1e8 / ynorm;
      ynorm = 1e8;
    }
    // line search: lambda = 1, then cubic backtracking (Dennis & Schnabel A6.3.1)
    double lam = 1.0, gnorm = 0.0, lamprev = 1.0, gprev = 0.0, wnorm2 = 0.0;
    bool ok = false;
    const double alpha = 1e-4;
    for (int ls = 0; ls < 41; ls++) {
      k_ms_trial<<<L.grid, L.block, 0, s>>>(g, S->P.model, L.u, lam * scale, L.x, L.W);
      if ((rc = residual(S, L, L.W, L.G, &gnorm, &wnorm2))) return rc;
      if (!o.line_search || 0.5 * gnorm * gnorm <= 0.5 * fnorm * fnorm + lam * alpha * initslope) {
        ok = true;
        break;
      }
      double lamtemp;
      if (ls == 0) {
        lamtemp = -initslope / (gnorm * gnorm - fnorm * fnorm - 2.0 * lam * initslope);
      } else {
        const double t1 = 0.5 * (gnorm * gnorm - fnorm * fnorm) - lam * initslope;
        const double t2 = 0.5 * (gprev * gprev - fnorm * fnorm) - lamprev * initslope;
        const double ca = (t1 / (lam * lam) - t2 / (lamprev * lamprev)) / (lam - lamprev);
        const double cb = (-lamprev * t1 / (lam * lam) + lam * t2 / (lamprev * lamprev)) / (lam - lamprev);
        double d = cb * cb - 3.0 * ca * initslope;
        if (d < 0.0) d = 0.0;
        lamtemp = ca == 0.0 ? -initslope / (2.0 * cb) : (-cb + sqrt(d)) / (3.0 * ca);
      }
      lamprev = lam;
      gprev = gnorm;
      lam = lamtemp > 0.5 * lam ? 0.5 * lam : (lamtemp <= 0.1 * lam ? 0.1 * lam : lamtemp);
      if (lam < 1e-12) break;
    }
    its++;
    if (!ok) {
      rep->fnorm[k][its] = fnorm;
      reason = SN_DIVERGED_LINE_SEARCH;
      break;
    }
    std::swap(L.u, L.W);
    std::swap(L.F, L.G);
    fnorm = gnorm;
    rep->fnorm[k][its] = fnorm;
    if (o.monitor_degree > 0 && (rc = area(S, L, L.u, rep->area[k][its]))) return rc;
    // ||u|| of the accepted trial, reduced by its residual evaluation
    const double xnorm = sqrt(wnorm2), snorm = lam * ynorm;
    if (fnorm != fnorm) reason = SN_DIVERGED_FNORM_NAN;
    else if (fnorm < o.atol) reason = SN_CONVERGED_FNORM_ABS;
    else if (fnorm <= ttol) reason = SN_CONVERGED_FNORM_RELATIVE;
    else if (snorm < o.stol * xnorm) reason = SN_CONVERGED_SNORM_RELATIVE;
    else if (its >= o.max_it) reason = SN_DIVERGED_MAX_IT;
  }
  rep->its[k] = its;
  rep->reason[k] = reason;
  rep->m[k] = g.mx;
  rep->inner_form[k] = L.block1 ? 1 : L.persist ? 2 : 0;
  return FISHGPU_OK;
}

extern "C" int fishgpu_ms_opts_default(fishgpu_ms_opts *o) {
  if (!o) return FISHGPU_ERR_ARG;
  memset(o, 0, sizeof(*o));
  o->ctx.problem = FISHGPU_MS_CATENOID;
  o->ctx.q = -0.5;
  o->ctx.catenoid_c = 1.1;
  o->ctx.tent_H = 1.0;
  o->ctx.model = FISHGPU_NL_MINIMAL;
  o->ctx.lambda = 1.0;
  o->mx = o->my = 3;
  o->rtol = 1e-8;
  o->atol = 1e-50;
  o->stol = 1e-8;
  o->max_it = 50;
  o->line_search = 1;
  o->ksp_rtol = 1e-5;
  o->ksp_max_it = 10000;
  o->inner_block = 1;
  o->inner_persist = -1;
  o->pc_type = FISHGPU_PC_MG;
  return FISHGPU_OK;
}

extern "C" int fishgpu_bratu_opts_default(fishgpu_ms_opts *o) {
  const int rc = fishgpu_ms_opts_default(o);
  if (rc) return rc;
  o->ctx.model = FISHGPU_NL_BRATU;  // bratu2D.c:87-98: lambda 1, u = 0 on the boundary
  o->ctx.problem = FISHGPU_BRATU_ZERO;
  o->ctx.lambda = 1.0;
  return FISHGPU_OK;
}

extern "C" int fishgpu_obstacle_opts_default(fishgpu_ms_opts *o) {
  const int rc = fishgpu_ms_opts_default(o);
  if (rc) return rc;
  o->ctx.model = FISHGPU_NL_OBSTACLE;  // obstacle.c:89-107: 3x3 grid on (-2,2)^2, u0 = 0
  o->ctx.problem = 0;
  return FISHGPU_OK;
}

extern "C" const char *fishgpu_snes_reason_name(int r) {
  switch (r) {
  case SN_CONVERGED_FNORM_ABS: return "CONVERGED_FNORM_ABS";
  case SN_CONVERGED_FNORM_RELATIVE: return "CONVERGED_FNORM_RELATIVE";
  case SN_CONVERGED_SNORM_RELATIVE: return "CONVERGED_SNORM_RELATIVE";
  case SN_DIVERGED_FNORM_NAN: return "DIVERGED_FNORM_NAN";
  case SN_DIVERGED_MAX_IT: return "DIVERGED_MAX_IT";
  case SN_DIVERGED_LINE_SEARCH: return "DIVERGED_LINE_SEARCH";
  default: return "CONVERGED_ITERATING";
  }
}

extern "C" int fishgpu_ms_opts_parse(fishgpu_ms_opts *o, int argc, const char *const *argv) {
  if (!o || argc < 0 || (argc > 0 && !argv)) return FISHGPU_ERR_ARG;
  int refine = 0, gx = 0, gy = 0, monitor = 0, quaddeg = 3;
  auto num = [&](int &a, double *d, int *iv) -> int {
    if (a + 1 >= argc) return FISHGPU_ERR_ARG;
    char *end = nullptr;
    const char *sv = argv[++a];
    if (d) *d = strtod(sv, &end);
    else *iv = (int)strtol(sv, &end, 10);
    return (end && *end == 0 && end != sv) ? FISHGPU_OK : FISHGPU_ERR_ARG;
  };
  for (int a = 0; a < argc; a++) {
    const char *k = argv[a];
    int rc = FISHGPU_OK;
    if (!strcmp(k, "-ms_problem")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      const char *v = argv[++a];
      if (!strcmp(v, "catenoid")) o->ctx.problem = FISHGPU_MS_CATENOID;
      else if (!strcmp(v, "tent")) o->ctx.problem = FISHGPU_MS_TENT;
      else return FISHGPU_ERR_ARG;
    } else if (!strcmp(k, "-lb_lambda")) rc = num(a, &o->ctx.lambda, nullptr);
    else if (!strcmp(k, "-lb_exact")) o->ctx.problem = FISHGPU_BRATU_LIOUVILLE;
    else if (!strcmp(k, "-lb_showcounts")) {  // the driver prints the counts
    } else if (!strcmp(k, "-ms_q")) rc = num(a, &o->ctx.q, nullptr);
    else if (!strcmp(k, "-ms_catenoid_c")) rc = num(a, &o->ctx.catenoid_c, nullptr);
    else if (!strcmp(k, "-ms_tent_H")) rc = num(a, &o->ctx.tent_H, nullptr);
    else if (!strcmp(k, "-ms_exact_init")) o->exact_init = 1;
    else if (!strcmp(k, "-ms_monitor")) monitor = 1;
    else if (!strcmp(k, "-ms_quaddegree")) {
      rc = num(a, nullptr, &quaddeg);
      if (!rc && (quaddeg < 1 || quaddeg > 3)) return FISHGPU_ERR_ARG;
    } else if (!strcmp(k, "-da_refine")) rc = num(a, nullptr, &refine);
    else if (!strcmp(k, "-da_grid_x")) rc = num(a, nullptr, &gx);
    else if (!strcmp(k, "-da_grid_y")) rc = num(a, nullptr, &gy);
    else if (!strcmp(k, "-snes_grid_sequence")) rc = num(a, nullptr, &o->grid_sequence);
    else if (!strcmp(k, "-snes_rtol")) rc = num(a, &o->rtol, nullptr);
    else if (!strcmp(k, "-snes_atol")) rc = num(a, &o->atol, nullptr);
    else if (!strcmp(k, "-snes_stol")) rc = num(a, &o->stol, nullptr);
    else if (!strcmp(k, "-snes_max_it")) rc = num(a, nullptr, &o->max_it);
    else if (!strcmp(k, "-ksp_rtol")) rc = num(a, &o->ksp_rtol, nullptr);
    else if (!strcmp(k, "-ksp_max_it")) rc = num(a, nullptr, &o->ksp_max_it);
    else if (!strcmp(k, "-ms_loop_cap")) rc = num(a, nullptr, &o->loop_cap);
    else if (!strcmp(k, "-ms_inner_block")) rc = num(a, nullptr, &o->inner_block);
    else if (!strcmp(k, "-ms_inner_persist")) rc = num(a, nullptr, &o->inner_persist);
    else if (!strcmp(k, "-ms_vtail_points")) rc = num(a, nullptr, &o->vtail_points);
    else if (!strcmp(k, "-pc_mg_levels")) rc = num(a, nullptr, &o->mg_levels);
    else if (!strcmp(k, "-pc_type")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      const char *v = argv[++a];
      if (!strcmp(v, "mg")) o->pc_type = FISHGPU_PC_MG;
      else if (!strcmp(v, "none")) o->pc_type = FISHGPU_PC_NONE;
      else return FISHGPU_ERR_UNSUPPORTED;
    } else if (!strcmp(k, "-snes_linesearch_type")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      const char *v = argv[++a];
      if (!strcmp(v, "bt")) o->line_search = 1;
      else if (!strcmp(v, "basic")) o->line_search = 0;
      else return FISHGPU_ERR_UNSUPPORTED;
    } else if (!strcmp(k, "-snes_monitor") || !strcmp(k, "-snes_monitor_short")) o->snes_monitor = 1;
    else if (!strcmp(k, "-snes_converged_reason")) o->converged_reason = 1;
    else if (!strcmp(k, "-ksp_converged_reason")) o->ksp_converged_reason = 1;
    else if (!strcmp(k, "-ksp_type")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      a++;  // the inner solver is BiCGStab whatever is asked
    } else if (!strcmp(k, "-mat_is_symmetric")) {
      if (a + 1 < argc && argv[a + 1][0] != '-') a++;
    } else if (!strcmp(k, "-snes_fd_color") || !strcmp(k, "-snes_mf_operator") || !strcmp(k, "-snes_mf")) {
      // Jacobian handling of PETSc: the exact Jacobian is always used
    } else if (!strcmp(k, "-snes_type")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      const char *v = argv[++a];
      const bool vi = !strcmp(v, "vinewtonrsls") || !strcmp(v, "vinewtonssls");
      // the obstacle problem is solved by the reduced-space method for either VI type
      if (o->ctx.model == FISHGPU_NL_OBSTACLE ? !vi : strcmp(v, "newtonls")) return FISHGPU_ERR_UNSUPPORTED;
    } else if (!strcmp(k, "-obs_dump_binary")) {
      if (a + 1 >= argc) return FISHGPU_ERR_ARG;
      a++;  // written by the driver
    } else if (!strcmp(k, "-snes_view_solution")) {
      if (a + 1 < argc && argv[a + 1][0] != '-') a++;  // written by the driver
    } else if (!strcmp(k, "-log_view")) {
    } else {
      return FISHGPU_ERR_ARG;
    }
    if (rc) return rc;
  }
  o->monitor_degree = monitor ? quaddeg : 0;  // minimal.c:82-87,91-93
  int mx = gx > 0 ? gx : 3, my = gy > 0 ? gy : 3;
  if (mx < 3 || my < 3 || refine < 0 || refine > 14 || o->grid_sequence < 0 ||
      o->grid_sequence >= FISHGPU_MS_MAX_GRIDS)
    return FISHGPU_ERR_ARG;
  for (int r = 0; r < refine; r++) {
    mx = 2 * mx - 1;
    my = 2 * my - 1;
  }
  o->mx = mx;
  o->my = my;
  if (o->ctx.model == FISHGPU_NL_OBSTACLE) return (o->exact_init || o->monitor_degree) ? FISHGPU_ERR_ARG : FISHGPU_OK;
  if (o->ctx.model == FISHGPU_NL_BRATU) {
    if (o->ctx.problem == FISHGPU_BRATU_LIOUVILLE && o->ctx.lambda != 1.0) return FISHGPU_ERR_ARG;  // bratu2D.c:109-113
    if (o->exact_init || o->monitor_degree) return FISHGPU_ERR_ARG;
    return FISHGPU_OK;
  }
  if (o->ctx.problem == FISHGPU_MS_CATENOID && o->ctx.catenoid_c < 1.0) return FISHGPU_ERR_ARG;  // minimal.c:121-124
  if (o->exact_init && (o->ctx.problem != FISHGPU_MS_CATENOID || o->ctx.q != -0.5)) return FISHGPU_ERR_ARG;
  return FISHGPU_OK;
}

extern "C" int fishgpu_ms_solver_destroy(fishgpu_ms_solver *S) {
  if (!S) return FISHGPU_OK;
  if (S->stream) cudaStreamSynchronize(S->stream);
  for (auto &L : S->lev) {
    if (L.g_init) cudaGraphExecDestroy(L.g_init);
    if (L.g_iter) cudaGraphExecDestroy(L.g_iter);
    if (L.g_loop) cudaGraphExecDestroy(L.g_loop);
    if (L.P) fishgpu_solver_destroy(L.P);
  }
  for (void *p : S->allocs) cudaFree(p);
  if (S->st_h) cudaFreeHost(S->st_h);
  if (S->hval) cudaFreeHost(S->hval);
  if (S->ev0) cudaEventDestroy(S->ev0);
  if (S->ev1) cudaEventDestroy(S->ev1);
  if (S->evg) cudaEventDestroy(S->evg);
  if (S->evg2) cudaEventDestroy(S->evg2);
  if (S->own_stream && S->stream) cudaStreamDestroy(S->stream);
  delete S;
  return FISHGPU_OK;
}

extern "C" int fishgpu_ms_solver_create(const fishgpu_ms_opts *o, void *stream, fishgpu_ms_solver **out) {
  if (!o || !out) return FISHGPU_ERR_ARG;
  *out = nullptr;
  if (o->mx < 3 || o->my < 3 || o->grid_sequence < 0 || o->grid_sequence >= FISHGPU_MS_MAX_GRIDS) return FISHGPU_ERR_ARG;
  if (o->ctx.model != FISHGPU_NL_MINIMAL && o->ctx.model != FISHGPU_NL_BRATU && o->ctx.model != FISHGPU_NL_OBSTACLE)
    return FISHGPU_ERR_ARG;
  if (o->ctx.model == FISHGPU_NL_OBSTACLE && (o->monitor_degree || o->exact_init)) return FISHGPU_ERR_ARG;
  if (o->ctx.problem != 0 && o->ctx.problem != 1) return FISHGPU_ERR_ARG;
  if (o->ctx.model == FISHGPU_NL_MINIMAL && o->ctx.problem == FISHGPU_MS_CATENOID && !(o->ctx.catenoid_c >= 1.0))
    return FISHGPU_ERR_ARG;
  if (o->ctx.model == FISHGPU_NL_BRATU && o->ctx.problem == FISHGPU_BRATU_LIOUVILLE && o->ctx.lambda != 1.0)
    return FISHGPU_ERR_ARG;  // bratu2D.c:109-113
  if (o->ctx.model == FISHGPU_NL_BRATU && o->monitor_degree) return FISHGPU_ERR_ARG;
  if (!(o->rtol >= 0) || !(o->atol >= 0) || !(o->stol >= 0) || o->max_it < 0 || !(o->ksp_rtol > 0) ||
      o->ksp_max_it < 1 || o->monitor_degree < 0 || o->monitor_degree > 3 || o->loop_cap < 0)
    return FISHGPU_ERR_ARG;
  if (o->pc_type != FISHGPU_PC_MG && o->pc_type != FISHGPU_PC_NONE) return FISHGPU_ERR_UNSUPPORTED;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FISHGPU_ERR_NODEVICE;
  }
  fishgpu_ms_solver *S = new fishgpu_ms_solver();
  S->o = *o;
  S->P = MsP{o->ctx.problem, o->ctx.q, o->ctx.catenoid_c, o->ctx.tent_H, o->ctx.model, o->ctx.lambda};
  int rc = FISHGPU_OK;
#define MS_FAIL(x)                 \
  do {                             \
    if ((rc = (x)) != FISHGPU_OK) { \
      fishgpu_ms_solver_destroy(S); \
      return rc;                   \
    }                              \
  } while (0)
  if (stream) {
    S->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete S;
      return FISHGPU_ERR_CUDA;
    }
    S->own_stream = true;
  }
  if (cudaMallocHost((void **)&S->st_h, sizeof(MsKsp)) != cudaSuccess ||
      cudaMallocHost((void **)&S->hval, sizeof(double) * 8) != cudaSuccess ||
      cudaEventCreate(&S->ev0) != cudaSuccess || cudaEventCreate(&S->ev1) != cudaSuccess ||
      cudaEventCreate(&S->evg) != cudaSuccess || cudaEventCreate(&S->evg2) != cudaSuccess)
    MS_FAIL(FISHGPU_ERR_CUDA);
  int mx = o->mx, my = o->my;
  S->lev.resize(o->grid_sequence + 1);
  for (size_t k = 0; k < S->lev.size(); k++) {
    MsLevel &L = S->lev[k];
    fishgpu_opts po;
    fishgpu_opts_default(&po);
    po.ctx.dim = 2;
    po.ctx.problem = FISHGPU_ZERO;
    if (o->ctx.model == FISHGPU_NL_OBSTACLE) po.ctx.Lx = po.ctx.Ly = 4.0;  // (-2,2)^2, obstacle.c:97
    po.mx = mx;
    po.my = my;
    po.mz = 1;
    po.pc_type = FISHGPU_PC_MG;
    po.precision = FISHGPU_MIXED;
    // only the hierarchy and its V-cycle are used here (never the fish
    // solver's CG): no persistent-solve tables, no second residual buffer
    po.persist = 0;
    po.fuse_cgr = 0;
    if (o->vtail_points > 0) po.vtail_points = o->vtail_points;
    // default hierarchy: coarsen only down to about 33 x 33 and solve that
    // grid exactly (one block, sine transform): the V-cycle of these 2D grids
    // is launch-bound, and the deepest levels cost launches, not work
    const int lmax = ms_levels_for(mx, my);
    int ldef = 1, cm = std::min(mx, my);
    while (ldef < lmax && cm > 33) {
      cm = (cm - 1) / 2 + 1;
      ldef++;
    }
    po.mg_levels = o->mg_levels > 0 && o->mg_levels < lmax ? o->mg_levels : ldef;
    MS_FAIL(fishgpu_solver_create(&po, (void *)S->stream, &L.P));
    L.g = solver_fine(L.P);
    L.N = (long long)L.g.plane;
    L.block = dim3(32, 8);
    L.grid = dim3((unsigned)((L.g.pitch + 31) / 32), (unsigned)((L.g.my + 7) / 8));
    S->cap = std::max(S->cap, (int)(L.grid.x * L.grid.y));
    MS_FAIL(ms_alloc(S, &L.u, L.N));
    MS_FAIL(ms_alloc(S, &L.F, L.N));
    MS_FAIL(ms_alloc(S, &L.W, L.N));
    MS_FAIL(ms_alloc(S, &L.G, L.N));
    MS_FAIL(ms_alloc(S, &L.C1, L.N));
    MS_FAIL(ms_alloc(S, &L.C2, L.N));
    float **vs[10] = {&L.b, &L.r, &L.rh, &L.p, &L.v, &L.s, &L.t, &L.x, &L.ph, &L.sh};
    for (float **q : vs) MS_FAIL(ms_alloc(S, q, L.N));
    L.giters = L.N >= (1LL << 20) ? 1 : 2;
    {  // grids of up to 4096 nodes whose preconditioner is one exact coarse solve: one-block inner solves
      CoarseView cv;
      const bool one_level = o->pc_type == FISHGPU_PC_MG && solver_coarse32(L.P, &cv);
      if (o->inner_block && (long long)L.g.mx * L.g.my <= 4096 && (o->pc_type != FISHGPU_PC_MG || one_level)) {
        L.block1 = true;
        L.use_pc = one_level ? 1 : 0;
        if (one_level)
          L.bc = BiCoarse{cv.g, cv.S0, cv.S1, cv.ilam, cv.work, cv.x, cv.n0, cv.n1, (int)cv.smem, cv.dinv};
        const long long cap =
            o->loop_cap > 0 ? o->loop_cap : (long long)std::max(1, o->ksp_max_it) / L.giters + 5;
        L.max_iters = (int)std::min<long long>(cap * L.giters, 1 << 30);
        // the work vectors in shared memory when they fit beside the coarse solve's tables
        const size_t coarse = L.use_pc ? (size_t)L.bc.smem : 0;
        const size_t off = (coarse + 15) / 16 * 16;
        const size_t need = off + 10 * sizeof(float) * (size_t)L.g.pitch * L.g.my;
        L.bsm = coarse;
        if (need <= 200 * 1024 &&
            cudaFuncSetAttribute(k_bi_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need) == cudaSuccess) {
          L.bsm = need;
          L.vsm_off = (int)off;
        }
        cudaGetLastError();
      }
      // larger multigrid grids: one cooperative launch per inner solve (the
      // V-cycle's coarse solve in block 0)
      const long long plim = o->inner_persist < 0 ? FISHGPU_MS_PERSIST_POINTS : o->inner_persist;
      if (!L.block1 && o->pc_type == FISHGPU_PC_MG && (long long)L.g.mx * L.g.my <= plim &&
          solver_persist32(L.P, (const void *)k_bi_persist, o->vtail_points, &L.pa, &L.pblocks, &L.psmem)) {
        L.persist = true;
        const long long cap =
            o->loop_cap > 0 ? o->loop_cap : (long long)std::max(1, o->ksp_max_it) / L.giters + 5;
        L.max_iters = (int)std::min<long long>(cap * L.giters, 1 << 30);
      }
    }
    if (S->P.model != FISHGPU_NL_OBSTACLE) {
      L.gtm = std::max(L.g.mx, L.g.my);
      MS_FAIL(ms_alloc(S, &L.gt, 16LL * L.gtm));
      k_ms_gtab<<<(L.gtm + 127) / 128, 128, 0, S->stream>>>(L.g, S->P, L.gt, L.gtm);
      if (cudaGetLastError() != cudaSuccess) MS_FAIL(FISHGPU_ERR_CUDA);
    }
    mx = 2 * mx - 1;
    my = 2 * my - 1;
  }
  MS_FAIL(ms_alloc(S, &S->red.partials, 2LL * S->cap));
  MS_FAIL(ms_alloc(S, &S->red.tickets, 4));
  MS_FAIL(ms_alloc(S, &S->part3, 3LL * S->cap));
  MS_FAIL(ms_alloc(S, &S->dval, 8));
  MS_FAIL(ms_alloc(S, &S->st, 1));
  S->red.cap = S->cap;
  S->red.tcap = 1;
  if (cudaMemsetAsync(S->red.tickets, 0, 16, S->stream) != cudaSuccess ||
      cudaMemsetAsync(S->st, 0, sizeof(MsKsp), S->stream) != cudaSuccess)
    MS_FAIL(FISHGPU_ERR_CUDA);
  for (auto &L : S->lev) {
    MS_FAIL(capture(S, L, true, &L.g_init));
    // the BiCGStab loop on the device (bodies of giters iterations until the
    // inner solve stops, capped); the host-polled graph if the driver refuses
    const unsigned int cap =
        o->loop_cap > 0 ? (unsigned int)o->loop_cap : (unsigned int)(std::max(1, o->ksp_max_it) / L.giters + 5);
    if (!build_loop_graph(S->stream, [&] { for (int k = 0; k < L.giters; k++) enq_bicg_iter(S, L); },
                          &S->st->k.done, nullptr, 0u, &S->st->k.loops, cap, &L.g_loop, &L.n_loop))
      MS_FAIL(capture(S, L, false, &L.g_iter));
  }
  if (cudaStreamSynchronize(S->stream) != cudaSuccess) MS_FAIL(FISHGPU_ERR_CUDA);
#undef MS_FAIL
  *out = S;
  return FISHGPU_OK;
}

extern "C" int fishgpu_ms_solver_solve(fishgpu_ms_solver *S, double *u_host, fishgpu_ms_report *rep) {
  if (!S || !rep) return FISHGPU_ERR_ARG;
  memset(rep, 0, sizeof(*rep));
  cudaStream_t s = S->stream;
  int rc;
  S->nfuncs = 0;
  MS_CK(cudaEventRecord(S->ev0, s));
  for (size_t k = 0; k < S->lev.size(); k++) {
    MsLevel &L = S->lev[k];
    if (k == 0) {
      const int mode = S->P.model != FISHGPU_NL_MINIMAL ? 2 : S->o.exact_init ? 1 : 0;
      k_ms_init<<<L.grid, L.block, 0, s>>>(L.g, S->P, mode, L.u);
    } else {
      MsLevel &C = S->lev[k - 1];
      k_ms_interp<<<L.grid, L.block, 0, s>>>(C.g, C.u, L.g, L.u);
    }
    MS_CK(cudaGetLastError());
    MS_CK(cudaEventRecord(S->evg, s));
    if ((rc = newton(S, L, (int)k, rep))) return rc;
    MS_CK(cudaEventRecord(S->evg2, s));
    MS_CK(cudaEventSynchronize(S->evg2));
    float gms = 0.f;
    MS_CK(cudaEventElapsedTime(&gms, S->evg, S->evg2));
    rep->grid_ms[k] = gms;
    rep->ngrids = (int)k + 1;
  }
  MS_CK(cudaEventRecord(S->ev1, s));
  MsLevel &L = S->lev.back();
  rep->dofs = (long long)L.g.mx * L.g.my;
  rep->errinf = -1.0;
  if (S->P.model == FISHGPU_NL_OBSTACLE) {
    const int nb = (int)(L.grid.x * L.grid.y);
    k_obs_report<<<L.grid, L.block, 0, s>>>(L.g, 0, L.u, L.F, S->part3, S->cap);
    k_ms_fin3<<<1, 256, 0, s>>>(S->part3, S->cap, nb, S->dval);
    k_obs_report<<<L.grid, L.block, 0, s>>>(L.g, 1, L.u, L.F, S->part3, S->cap);
    k_ms_fin3<<<1, 256, 0, s>>>(S->part3, S->cap, nb, S->dval + 3);
    MS_CK(cudaGetLastError());
    if ((rc = read_vals(S, 6))) return rc;
    const double afree = 0.697965148223374, exactarea = M_PI * afree * afree;
    rep->err1 = S->hval[0] / ((double)L.g.mx * L.g.my);
    rep->errinf = S->hval[2];
    rep->n_active = (long long)S->hval[3];
    rep->active_area_err = fabs(L.g.h[0] * L.g.h[1] * S->hval[3] - exactarea) / exactarea;
  }
  const bool has_exact = S->P.model == FISHGPU_NL_BRATU
                             ? S->o.ctx.problem == FISHGPU_BRATU_LIOUVILLE
                             : (S->o.ctx.problem == FISHGPU_MS_CATENOID && S->o.ctx.q == -0.5);
  if (has_exact && S->P.model != FISHGPU_NL_OBSTACLE) {
    k_ms_err<<<L.grid, L.block, 0, s>>>(L.g, S->P, L.u, S->part3, S->cap);
    k_ms_fin3<<<1, 256, 0, s>>>(S->part3, S->cap, (int)(L.grid.x * L.grid.y), S->dval);
    MS_CK(cudaGetLastError());
    if ((rc = read_vals(S, 3))) return rc;
    rep->errinf = S->hval[2];
  }
  if (u_host)
    MS_CK(cudaMemcpy2DAsync(u_host, sizeof(double) * L.g.mx, L.u, sizeof(double) * L.g.pitch,
                            sizeof(double) * L.g.mx, L.g.my, cudaMemcpyDeviceToHost, s));
  MS_CK(cudaStreamSynchronize(s));
  float ms = 0.f;
  MS_CK(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
  rep->solve_ms = ms;
  rep->nfuncs = S->nfuncs;
  for (int k = 0; k < rep->ngrids; k++)
    if (rep->reason[k] <= 0) return FISHGPU_ERR_NOT_CONVERGED;
  return FISHGPU_OK;
}

extern "C" int fishgpu_ms_solve(const fishgpu_ms_opts *o, double *u_host, fishgpu_ms_report *rep) {
  fishgpu_ms_solver *S = nullptr;
  int rc = fishgpu_ms_solver_create(o, nullptr, &S);
  if (rc) return rc;
  rc = fishgpu_ms_solver_solve(S, u_host, rep);
  fishgpu_ms_solver_destroy(S);
  return rc;
}

extern "C" int MinimalFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                                        const fishgpu_ms_ctx *ctx, void *stream) {
  if (!info || !au || !aF || !ctx || info->dim != 2) return FISHGPU_ERR_ARG;
  if (info->mx < 2 || info->my < 2 || info->xs < 0 || info->ys < 0 || info->xm < 0 || info->ym < 0 ||
      info->xs + info->xm > info->mx || info->ys + info->ym > info->my)
    return FISHGPU_ERR_ARG;
  if ((ctx->problem != 0 && ctx->problem != 1) || (ctx->model != FISHGPU_NL_MINIMAL && ctx->model != FISHGPU_NL_BRATU))
    return FISHGPU_ERR_ARG;
  if (info->xm == 0 || info->ym == 0) return FISHGPU_OK;
  Geom g;
  memset(&g, 0, sizeof(g));
  g.dim = 2;
  g.mx = info->mx;
  g.my = info->my;
  g.mz = 1;
  g.pitch = info->mx;
  g.plane = (long long)info->mx * info->my;
  g.h[0] = (info->xmax[0] - info->xmin[0]) / (info->mx - 1);  // minimal.c:221-222
  g.h[1] = (info->xmax[1] - info->xmin[1]) / (info->my - 1);
  const MsP P{ctx->problem, ctx->q, ctx->catenoid_c, ctx->tent_H, ctx->model, ctx->lambda};
  const dim3 block(32, 8), grid((info->xm + 31) / 32, (info->ym + 7) / 8);
  k_ms_funclocal<<<grid, block, 0, (cudaStream_t)stream>>>(g, P, info->xs, info->ys, info->xm, info->ym, au, aF);
  return cudaGetLastError() == cudaSuccess ? FISHGPU_OK : FISHGPU_ERR_CUDA;
}

extern "C" int BratuFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF, double lambda,
                                      int liouville, void *stream) {
  fishgpu_ms_ctx c;
  memset(&c, 0, sizeof(c));
  c.model = FISHGPU_NL_BRATU;
  c.problem = liouville ? FISHGPU_BRATU_LIOUVILLE : FISHGPU_BRATU_ZERO;
  c.lambda = lambda;
  if (liouville && lambda != 1.0) return FISHGPU_ERR_ARG;
  return MinimalFunctionLocal_gpu(info, au, aF, &c, stream);
}
