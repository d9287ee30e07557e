// Tensor-memory-accelerator (TMA) tile loads of a padded field into shared
// memory, completed on an mbarrier (sm_90+ PTX, used here on sm_103a).
//
// A field of the common padded box (PX x PY x PZ elements, x fastest) is
// described by a 3-D tiled tensor map; one thread of a CTA issues
// cp.async.bulk.tensor loads of box x by x 1 tiles into shared memory and
// arms the tile's mbarrier with the byte count (expect_tx); the threads that
// read the tile wait on the barrier's phase. Coordinates outside the box read
// zeros (the tensor map's out-of-bounds fill). Every wait is bounded: after
// kTmaWaitLimit polls the waiting thread reports failure, and the kernel
// records it in an error flag and leaves.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mifgpu {

// Tensor maps of the fields one stage kernel stages into its plane ring.
struct StageMaps {
  CUtensorMap m[5];
};

constexpr int kTmaWaitLimit = 1 << 22;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Makes initialised barriers visible to the async proxy (the TMA unit).
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// Orders this thread's earlier shared-memory accesses (and those a CTA
// barrier made visible to it) before its later async-proxy copies.
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of the barrier; false after kTmaWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  for (int it = 0; it < kTmaWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// One box of the 3-D tensor map at element coordinates (x, y, z) into dst
// (16-byte aligned), completing on bar. x * element size must be a multiple
// of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Host: a 3-D tiled tensor map over one field of the padded box (elements
// of `elem` bytes, 4 float or 8 double), box bx x by x 1, zero fill outside.
// Returns false if the driver rejects it.
bool make_field_map(CUtensorMap *map, const void *base, int elem, long PX, long PY, long PZ, int bx, int by);
// The same over any 3-D view: dims[3] elements, byte strides of dims 1 and 2.
bool make_map_3d(CUtensorMap *map, const void *base, int elem, const long dims[3], const long strides[2], int bx,
                 int by);

}  // namespace mifgpu
