// Bond walk with memory-level parallelism.
//
// A particle's bonds are walked U slots at a time: the U neighbour indices
// are loaded first, then the U neighbour gathers are issued (slots that are
// padding or broken gather the particle itself, a valid address whose data
// is discarded), then the per-bond bodies run in slot order.  The gathers
// are the latency-bound part of every pass (dependent index -> data loads
// from L1/L2); U independent chains per thread keep U times more of them in
// flight.  The body order is the sequential slot order, so sums are
// bit-identical to the one-slot-at-a-time loop.
//
// idx(k) returns the neighbour index of the particle's slot k (from global
// memory or from a staged shared-memory copy); body(k, j, g) gets the slot
// number k, the index j >= 0 and the gathered data.  An index source with
// kDense = true never yields a negative index (padding and broken slots
// point at data that contributes exact zeros), so the bodies run unguarded.
#pragma once
#include <cstdint>

namespace pd {

// Programmatic dependent launch: a pass launched with programmatic stream
// serialization starts while the previous pass drains; grid_dep_sync() waits
// until that pass has completed and its writes are visible, then lets the next
// pass launch.  Without the launch attribute both instructions return at once.
__device__ __forceinline__ void grid_dep_sync() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int U, typename Idx, typename Gather, typename Body>
__device__ __forceinline__ void walk_bonds(int w, int64_t self, Idx idx, Gather gather, Body body) {
  using G = decltype(gather(0));
  int k = 0;
  for (; k + U <= w; k += U) {
    int j[U];
#pragma unroll
    for (int q = 0; q < U; ++q) j[q] = idx(k + q);
    G g[U];
    if constexpr (Idx::kDense) {
#pragma unroll
      for (int q = 0; q < U; ++q) g[q] = gather((int64_t)j[q]);
#pragma unroll
      for (int q = 0; q < U; ++q) body(k + q, j[q], g[q]);
    } else {
#pragma unroll
      for (int q = 0; q < U; ++q) g[q] = gather(j[q] < 0 ? self : (int64_t)j[q]);
#pragma unroll
      for (int q = 0; q < U; ++q)
        if (j[q] >= 0) body(k + q, j[q], g[q]);
    }
  }
  for (; k < w; ++k) {
    const int jj = idx(k);
    if (Idx::kDense || jj >= 0) body(k, jj, gather((int64_t)jj));
  }
}

// Streaming (evict-first) load of global slot s0 + 32 k of a SELL-32 row.
struct GlobalIdx {
  static constexpr bool kDense = false;
  const int32_t* nbr;
  int64_t s0;
  __device__ __forceinline__ int operator()(int k) const { return __ldcs(&nbr[s0 + (int64_t)k * 32]); }
};

}  // namespace pd
