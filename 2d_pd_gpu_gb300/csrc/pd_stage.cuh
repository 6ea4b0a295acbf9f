// Staging of a warp's SELL-32 chunk of bond indices in shared memory.
//
// The 32 particles of a warp own one chunk: w slots x 32 lanes of int32,
// contiguous in HBM (128 B per slot row, 128 B aligned because chunk bases
// are multiples of 32 slots).  Lane 0 moves the whole chunk with one bulk
// asynchronous copy (TMA, cp.async.bulk) completing on a per-warp mbarrier;
// the walk then reads its indices from shared memory, so each group of
// neighbour gathers waits for one L1/L2 round trip instead of an HBM index
// load followed by the gather.
//
// The wait is bounded: after kStageSpinLimit polls the warp records
// ERR_STAGE_TIMEOUT, waits once more (bounded) for its copy, and the caller
// skips the particle's work; the host reports PD_ERR_TIMEOUT.
#pragma once
#include <cstdint>

namespace pd {

constexpr unsigned kStageSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (unsigned it = 0; it < kStageSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Copies src[0 .. 32 w) (global) to dst (shared) for the calling warp; all 32
// lanes must call it.  Returns false if the copy did not land in time.
__device__ __forceinline__ bool stage_chunk(int32_t* dst, const int32_t* src, int w, uint64_t* bar) {
  if (w <= 0) return true;
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t b = smem_addr(bar);
  const uint32_t bytes = (uint32_t)w * 128u;
  if (lane == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  if (lane == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(b)
        : "memory");
  }
  if (mbar_wait_bounded(b, 0)) return true;
  mbar_wait_bounded(b, 0);  // give the copy in flight one more bounded chance before the warp moves on
  return false;
}

// Index of slot k of lane `lane` in a staged chunk.
struct SharedIdx {
  const int32_t* base;
  int lane;
  __device__ __forceinline__ int operator()(int k) const { return base[k * 32 + lane]; }
};

}  // namespace pd
