// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory,
// completing on an mbarrier, with bounded waits.
//
// Used to stage a warp's SELL-32 chunk of bond indices: the 32 particles of
// a warp own w slot rows x 32 lanes, contiguous in HBM (128 B per row of
// int32 indices, 64 B per row of 16-bit halo indices; chunk bases are
// multiples of 32 slots, so the source is 64 B aligned).  One thread issues
// the whole chunk; the walk then reads its indices from shared memory.
//
// Every wait is bounded: after kStageSpinLimit polls the caller records
// ERR_STAGE_TIMEOUT, waits once more (bounded) for its copy, and skips the
// work; the host reports PD_ERR_TIMEOUT.
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

// One thread: arms `bar` (phase 0) for `bytes` and issues the copy
// global src -> shared dst.  bytes > 0, a multiple of 16; both addresses
// 16 B aligned.
__device__ __forceinline__ void stage_issue(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  const uint32_t b = smem_addr(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(b)
      : "memory");
}

// Any thread, after the issuing thread's stage_issue is ordered before it
// (same thread, __syncwarp or __syncthreads).  False if the copy did not
// land in time (after one more bounded wait for it).
__device__ __forceinline__ bool stage_wait(uint64_t* bar) {
  const uint32_t b = smem_addr(bar);
  if (mbar_wait_bounded(b, 0)) return true;
  mbar_wait_bounded(b, 0);
  return false;
}

// Warp-cooperative: copies src[0 .. 32 w) int32 (global) to dst (shared).
// All 32 lanes call it.  False if the copy did not land in time.
__device__ __forceinline__ bool stage_chunk(int32_t* dst, const int32_t* src, int w, uint64_t* bar) {
  if (w <= 0) return true;
  if ((threadIdx.x & 31u) == 0) stage_issue(dst, src, (uint32_t)w * 128u, bar);
  __syncwarp();
  return stage_wait(bar);
}

// Index of slot k of lane `lane` in a staged int32 chunk.
struct SharedIdx {
  static constexpr bool kDense = false;
  const int32_t* base;
  int lane;
  __device__ __forceinline__ int operator()(int k) const { return base[k * 32 + lane]; }
};

// Halo position of slot k of lane `lane` in a staged 16-bit chunk; padding
// and broken slots hold the particle's own position (dense: never negative).
struct SharedHaloIdx {
  static constexpr bool kDense = true;
  const uint16_t* base;
  int lane;
  __device__ __forceinline__ int operator()(int k) const { return base[k * 32 + lane]; }
};

}  // namespace pd
