// Tensor-memory-accelerator (TMA) loads of field windows into shared memory:
// the host encodes a tiled tensor map of a field array, one thread of a CTA
// arms an mbarrier with the byte count and issues cp.async.bulk.tensor, and
// every thread waits on the barrier with an iteration limit. Inline PTX for
// sm_90 and later (sm_103a here).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pic {

// iterations of mbarrier.try_wait before a wait is declared lost (each
// try_wait blocks for a hardware-defined interval; a window load takes
// microseconds)
constexpr long kTmaWaitLimit = 1L << 22;

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  // make the initialised barrier visible to the async proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0u;
}

// waits for phase `parity` of the barrier; false when the limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
  for (long it = 0; it < kTmaWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// tiled loads of a box at integer coordinates (innermost first); the box
// lands in shared memory innermost-fastest, out-of-range elements as zeros
__device__ __forceinline__ void tma_load_3d(unsigned dst, const void* map, unsigned bar, int c0,
                                            int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(unsigned dst, const void* map, unsigned bar, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

// Encodes a tiled tensor map of a field array with `rank` axes (innermost
// first): dims[] elements per axis, strides[] the element strides of axes
// 1..rank-1 (axis 0 contiguous), box[] the box extent per axis. Returns false
// (and leaves the map unused) when the array does not meet TMA's rules: a
// 16-byte aligned base, byte strides that are multiples of 16, an innermost
// box of a multiple of 16 bytes, box extents of at most 256, or when the
// driver entry point is unavailable.
bool encode_field_map(CUtensorMap* map, const void* base, int real_bytes, int rank,
                      const int64_t* dims, const int64_t* strides, const int* box);

// false when TMA staging is switched off for this process
// (ENTITY_PIC_NO_TMA=1 in the environment, read at each launch)
bool tma_enabled();

}  // namespace pic
