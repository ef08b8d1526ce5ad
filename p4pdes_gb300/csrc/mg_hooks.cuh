// mg_hooks.cuh -- internal interface of solver.cu for other solvers of the
// library that reuse a 2D mixed-form fish solver's geometry, stream and FP32
// Poisson multigrid hierarchy (the minimal-surface Newton solver
// preconditions its inner Krylov solves with that V-cycle).
#pragma once

#include "common.cuh"
#include "vblock.cuh"

struct fishgpu_solver_s;

namespace fg {

const Geom &solver_fine(const fishgpu_solver_s *S);
const Slots &solver_slots(const fishgpu_solver_s *S);
cudaStream_t solver_stream(const fishgpu_solver_s *S);
// Enqueues z = V-cycle(r) (Poisson operator, FP32, zero initial iterate) on
// the solver's stream; kernels return at once while st->done is set.  Returns
// the hierarchy buffer that holds z (valid until the next V-cycle), or null
// when the solver is not a 2D mixed-form multigrid solver.
const float *solver_vcycle32(fishgpu_solver_s *S, const float *r, KspState *st);

// The exact coarse solve that is the whole V-cycle of a 2D mixed-form
// solver with one multigrid level: its geometry, sine-transform tables,
// work area, shared-memory bytes (0: use `work`) and output buffer.
struct CoarseView {
  Geom g;
  const float *S0, *S1, *ilam;
  float *work, *x;
  int n0, n1;
  size_t smem;
  float dinv;
};
// False unless the solver is a 2D mixed-form multigrid solver with one level.
bool solver_coarse32(const fishgpu_solver_s *S, CoarseView *c);

// The V-cycle of a 2D mixed-form multigrid solver (two Chebyshev/Jacobi
// steps per level) for a persistent cooperative kernel (persist_vcycle):
// fills the level table, the coarse solve, the grid barrier (zero it before
// each launch), the partial sums and the fault word of *a; levels of at most
// tail_pts nodes (the coarsest always) run in block 0.  *blocks and *smem:
// the launch's blocks of 512 threads (one per SM at most) and its dynamic
// shared memory.  False when the solver has no such V-cycle or the kernel
// cannot be launched so.
bool solver_persist32(fishgpu_solver_s *S, const void *kernel, long long tail_pts, PersistArgs<float> *a,
                      int *blocks, size_t *smem);

}  // namespace fg
