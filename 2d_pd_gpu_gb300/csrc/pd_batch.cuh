// Batched stepping of many independent plates (ragged sizes) in one launch.
//
// A batch is a device table of per-plate argument blocks (Fp64Args or
// MixedArgs: every plate keeps its own device arrays and parameters) and a
// work list of tiles {plate, first particle, count}.  Two launch modes:
//   persistent: one cooperative kernel for all nsteps; each phase (drift,
//     pass A, pass B) is a grid-stride loop over the tiles, separated by a
//     software grid barrier.  The barrier's waits are bounded: after
//     kBarrierSpinLimit polls (or the batch's own limit, BarrierLimits) a
//     block records a timeout in the error word and every block returns, so
//     the host gets PD_ERR_TIMEOUT and the context stays usable.
//     Co-residency of all blocks is guaranteed by the cooperative launch
//     (cudaLaunchAttributeCooperative).
//   phased: one ordinary kernel per phase (grid = tiles), captured in a CUDA
//     graph per step count.
// The per-particle work is the single-plate code, so every plate's results
// are identical to running it alone, in any mix and under any tuning.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pd {

struct BatchTile {
  int32_t plate;
  int32_t count;
  int64_t first;
};

struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;      // 1 = a wait gave up
  int pad;
};

constexpr unsigned long long kBarrierSpinLimit = 1ull << 26;  // x >= 64 ns sleeps: >= 4 s per barrier
constexpr unsigned kBarrierHoldMaxNs = 100000000u;              // 0.1 s

// Per-batch barrier controls (kernel arguments).  spins: polls before a wait
// gives up (0: kBarrierSpinLimit).  hold_ns: block 0 sleeps this long before
// it arrives at every barrier (0: never) -- a fault-injection control that
// lets a test make the other blocks' waits run out without any fault; at
// most kBarrierHoldMaxNs, so the hold itself is bounded.
struct BarrierLimits {
  unsigned long long spins = 0;
  unsigned hold_ns = 0;
};

// Returns false if this or another block gave up waiting (then return).
__device__ __forceinline__ bool grid_sync(GridBarrier* b, unsigned nblocks, const BarrierLimits& lim) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (lim.hold_ns && blockIdx.x == 0)
      for (unsigned t = 0; t < lim.hold_ns && t < kBarrierHoldMaxNs; t += 1000) __nanosleep(1000);
    const unsigned long long limit = lim.spins ? lim.spins : kBarrierSpinLimit;
    volatile unsigned int* vgen = &b->gen;
    volatile int* verr = &b->err;
    const unsigned g = *vgen;
    __threadfence();
    int ok = *verr == 0;
    if (ok) {
      const unsigned arrived = atomicAdd(&b->count, 1u);
      if (arrived == nblocks - 1) {
        atomicExch(&b->count, 0u);
        __threadfence();
        atomicAdd(&b->gen, 1u);
      } else {
        unsigned long long spins = 0;
        while (*vgen == g) {
          if (*verr) {
            ok = 0;
            break;
          }
          if (++spins > limit) {
            atomicExch(&b->err, 1);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

struct BatchLaunch {
  int block = 256;          // threads per block
  int blocks_per_sm = 2;    // persistent grid = SMs x this (<= occupancy)
  int persistent = 1;       // 1: cooperative persistent kernel, 0: phase kernels, 2: per-member graphs
  BarrierLimits limits;     // the persistent kernel's barrier controls
};

}  // namespace pd
