// tma.cuh -- bulk tensor copies (TMA) into shared memory and the mbarriers
// that signal them, for the stencil kernels that stage their planes in a
// shared-memory ring (one GPU: a tensor map covers this GPU's own memory and
// no copy is multicast).
//
// Every wait on an mbarrier is bounded in time (%globaltimer): a wait that
// has not seen its phase complete after kWaitNs gives up, records the failure
// in a device word the host reads after the solve, and lets the kernel run
// to its end (with wrong values) instead of spinning forever.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fg {

// ---------------------------------------------------------------- host
// A tiled 3D tensor map of a [nz][ny][nx] array (x fastest) with row and
// plane strides in bytes, boxes of bx * by * bz elements, zero fill outside
// the array.  False if the driver refuses it (alignment, sizes).
bool tma_map_3d(CUtensorMap *map, const void *base, CUtensorMapDataType dtype, long long nx, long long ny,
                long long nz, long long row_bytes, long long plane_bytes, int bx, int by, int bz);

// ---------------------------------------------------------------- device
constexpr unsigned long long kWaitNs = 200ull * 1000 * 1000;  // 0.2 s per wait

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the completion of the phase with the given parity; false (and
// *fault set) if it did not complete within kWaitNs.  Once a wait of the
// launch has given up, later waits give up at once (the launch's results are
// void anyway, and it ends in one wait's time instead of one per plane),
// except the waits for copies still in flight before a block ends (drain).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, int *fault, bool drain = false) {
  if (mbar_try_wait(bar, parity)) return true;
  if (!drain && fault && *(volatile int *)fault) return false;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > kWaitNs) {
      if (fault) atomicExch(fault, 1);
      return false;
    }
  }
  return true;
}

// 3D tile load: box at element coordinates (x, y, z) of `map` into shared
// memory at `dst` (128-byte aligned), completing `bytes` on `bar`.  x times
// the element size must be a multiple of 16 bytes; y and z may lie outside
// the array (zero fill).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// named barrier over `count` threads (a multiple of 32) of the block
__device__ __forceinline__ void bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

}  // namespace fg
