// Tensor-memory-accelerator (TMA) bulk copies and mbarriers, as inline PTX, and
// the host-side encoding of a tiled tensor map (cuTensorMapEncodeTiled, taken
// through the runtime's driver entry point so the library needs no libcuda
// link). Used by the lattice FFT passes to stage their tiles in shared memory.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.hpp"

namespace tprf {

// ---- device side --------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation and earlier generic-proxy shared-memory writes
// visible to the async proxy (the TMA unit).
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// One non-blocking probe of the barrier's phase with the given parity.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase with the given parity for at most limit_ns nanoseconds of
// the global timer (checked before every probe, so limit_ns = 0 gives up at once).
// False when the limit ran out.
__device__ __forceinline__ bool mbar_wait_timed(uint64_t *bar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (global_ns() - t0 >= limit_ns) return false;
    if (mbar_try_wait(bar, parity)) return true;
  }
}

// Bound of the drain after a timed-out wait: a block waits this long for each
// copy it has in flight before it leaves (the copies write its shared memory).
constexpr unsigned long long kTmaDrainNs = 1000000000ull;

// 4-D tiled bulk copy global -> shared, completing on the barrier (bytes counted
// by the barrier's expect_tx). Coordinates innermost first, in elements.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// ---- host side ----------------------------------------------------------------

// Encodes a tiled map of FP64 elements (rank <= 5; dims and box innermost
// first, strides in bytes for dims 1..rank-1). Returns a status; checks the
// documented constraints (16-byte base and strides, box <= 256 per dim, inner
// box a multiple of 16 bytes) before calling the driver.
int encode_tensor_map_f64(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                          const uint64_t *strides_bytes, const uint32_t *box);

}  // namespace tprf
