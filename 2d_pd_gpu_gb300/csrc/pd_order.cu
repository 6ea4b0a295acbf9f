// Spatial SELL layout of the mixed form, built on the GPU.
//
// The reference positions are binned into square cells of side
// q = sqrt(bbox area / n) (about one particle per cell; a lattice's cells are
// its sites).  Cells are grouped in tiles of 32 cells x kTileRows rows
// (kTileRows = kHaloBlock / 32, one visiting block of the mixed passes):
//   SELL positions  tile by tile (tiles row-major, bands of kTileRows rows), cells
//                   row-major inside a tile, equal cells by particle id; every
//                   tile starts a new chunk, the tail of its last chunk is a
//                   hole (member -1).  A chunk (32 positions) is then a row
//                   segment with its lanes in x order, and a visiting block of
//                   the mixed passes (up to kHaloBlock / 32 chunks) is one
//                   tile, whose bonds reach few distinct particles.
//   spatial key rk  (row-major cell index << 31) | particle id: halos are
//                   sorted by it and every family is walked in ascending rk
//                   of its neighbours (for a row-major numbering that is the
//                   family order), so the 32 lanes of a row segment read the
//                   same neighbour offset at the same slot, from consecutive
//                   halo entries, and the step is bit-identical whatever the
//                   numbering.
// Work: one pass computing cells, tile counts (atomics), a scatter into tile
// buckets, one CTA per tile sorting its particles in shared memory (bitonic,
// up to kTileSortCap; larger tiles, which only strongly clustered point sets
// produce, are sorted on the host), and the inverse map.
#include <algorithm>
#include <cmath>

#include "pd_internal.h"

namespace pd {

namespace {

constexpr int kTileSortCap = 2048;
constexpr int64_t kTileRows = kHaloBlock / 32;
static_assert(kHaloBlock % 32 == 0 && kHaloBlock <= 1024, "a visiting block is whole warps");

struct CellGrid {
  double x0, y0, inv_q;
  int64_t gx, gy, tiles_x;
};

__host__ __device__ __forceinline__ int64_t cell_of(double v, double lo, double inv_q, int64_t g) {
  const double t = floor((v - lo) * inv_q);
  if (!(t > 0.0)) return 0;  // also NaN
  return t >= (double)(g - 1) ? g - 1 : (int64_t)t;
}

__global__ void k_spatial_keys(int64_t n, const double2* __restrict__ x, CellGrid G, int32_t* tile_of,
                               uint16_t* local, uint64_t* rk, int32_t* tile_cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 p = x[i];
  const int64_t cx = cell_of(p.x, G.x0, G.inv_q, G.gx), cy = cell_of(p.y, G.y0, G.inv_q, G.gy);
  const int64_t t = (cy / kTileRows) * G.tiles_x + (cx >> 5);
  tile_of[i] = (int32_t)t;
  local[i] = (uint16_t)((cy % kTileRows) * 32 + (cx & 31));
  rk[i] = ((uint64_t)(cy * G.gx + cx) << 31) | (uint64_t)i;
  atomicAdd(&tile_cnt[t], 1);
}

__global__ void k_tile_scatter(int64_t n, const int32_t* __restrict__ tile_of, const int64_t* __restrict__ tile_start,
                               int32_t* cursor, int32_t* bucket) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t t = tile_of[i];
  bucket[tile_start[t] + atomicAdd(&cursor[t], 1)] = (int32_t)i;
}

// One CTA per tile: its particles in (cell, id) order to member[first position ...).
__global__ void __launch_bounds__(256) k_tile_sort(const int32_t* __restrict__ tile_cnt,
                                                   const int64_t* __restrict__ tile_start,
                                                   const int64_t* __restrict__ tile_pos,
                                                   const int32_t* __restrict__ bucket,
                                                   const uint16_t* __restrict__ local, int32_t* member) {
  __shared__ uint64_t key[kTileSortCap];
  const int64_t t = blockIdx.x;
  const int cnt = tile_cnt[t];
  if (cnt <= 0 || cnt > kTileSortCap) return;  // block-uniform
  int P = 1;
  while (P < cnt) P <<= 1;
  const int32_t* b = bucket + tile_start[t];
  for (int r = threadIdx.x; r < P; r += blockDim.x) {
    if (r < cnt) {
      const int32_t i = b[r];
      key[r] = ((uint64_t)local[i] << 32) | (uint32_t)i;
    } else {
      key[r] = ~0ull;
    }
  }
  __syncthreads();
  for (int kk = 2; kk <= P; kk <<= 1)
    for (int jj = kk >> 1; jj > 0; jj >>= 1) {
      for (int r = threadIdx.x; r < P; r += blockDim.x) {
        const int o = r ^ jj;
        if (o > r) {
          const uint64_t a = key[r], c = key[o];
          if ((a > c) == ((r & kk) == 0)) {
            key[r] = c;
            key[o] = a;
          }
        }
      }
      __syncthreads();
    }
  int32_t* m = member + tile_pos[t];
  for (int r = threadIdx.x; r < cnt; r += blockDim.x) m[r] = (int32_t)(key[r] & 0xFFFFFFFFull);
}

__global__ void k_pos_from_member(int64_t npos, const int32_t* __restrict__ member, int32_t* pos_of) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npos) return;
  const int32_t i = member[p];
  if (i >= 0) pos_of[i] = (int32_t)p;
}

template <typename T>
cudaError_t alloc(T** p, size_t count, cudaStream_t s) {
  return cudaMallocAsync(reinterpret_cast<void**>(p), (count > 0 ? count : 1) * sizeof(T), s);
}

}  // namespace

int build_spatial_order(int64_t n, const double2* d_x, const double* h_x, cudaStream_t s, SellLayout* L,
                        int32_t** d_blocks, int64_t* nblocks, std::string* msg) {
  constexpr int kWarps = kHaloBlock / 32;
  *d_blocks = nullptr;
  *nblocks = 0;
  L->npos = 0;
  if (n <= 0) return PD_OK;
  // cell grid from the bounding box of the finite positions
  double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int64_t i = 0; i < n; ++i) {
    const double px = h_x[2 * i], py = h_x[2 * i + 1];
    if (!std::isfinite(px) || !std::isfinite(py)) continue;
    x0 = std::min(x0, px);
    x1 = std::max(x1, px);
    y0 = std::min(y0, py);
    y1 = std::max(y1, py);
  }
  CellGrid G{};
  const double ex = x1 - x0, ey = y1 - y0;
  double q = std::sqrt(ex * ey / (double)n);
  if (!(q > 0.0) || !std::isfinite(q)) q = std::max(ex, ey) / (double)n;
  G.x0 = std::isfinite(x0) ? x0 : 0.0;
  G.y0 = std::isfinite(y0) ? y0 : 0.0;
  G.inv_q = q > 0.0 && std::isfinite(q) ? 1.0 / q : 0.0;
  const int64_t cap = 2 * n + 2;  // cells per axis: at most about n + 1 by the choice of q
  G.gx = std::min<int64_t>(cap, cell_of(std::isfinite(x1) ? x1 : 0.0, G.x0, G.inv_q, cap) + 1);
  G.gy = std::min<int64_t>(cap, cell_of(std::isfinite(y1) ? y1 : 0.0, G.y0, G.inv_q, cap) + 1);
  G.tiles_x = (G.gx + 31) / 32;
  const int64_t ntiles = G.tiles_x * ((G.gy + kTileRows - 1) / kTileRows);
  int32_t *tile_of = nullptr, *tile_cnt = nullptr, *cursor = nullptr, *bucket = nullptr;
  uint16_t* local = nullptr;
  int64_t *tile_start = nullptr, *tile_pos = nullptr;
  cudaError_t e = alloc(&tile_of, (size_t)n, s);
  if (e == cudaSuccess) e = alloc(&local, (size_t)n, s);
  if (e == cudaSuccess) e = alloc(&tile_cnt, (size_t)ntiles, s);
  if (e == cudaSuccess) e = alloc(&cursor, (size_t)ntiles, s);
  if (e == cudaSuccess) e = alloc(&bucket, (size_t)n, s);
  if (e == cudaSuccess) e = alloc(&tile_start, (size_t)ntiles, s);
  if (e == cudaSuccess) e = alloc(&tile_pos, (size_t)ntiles, s);
  if (e == cudaSuccess) e = cudaMalloc(&L->rk, (size_t)n * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(tile_cnt, 0, (size_t)ntiles * sizeof(int32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, (size_t)ntiles * sizeof(int32_t), s);
  if (e == cudaSuccess)
    k_spatial_keys<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, d_x, G, tile_of, local, L->rk, tile_cnt);
  std::vector<int32_t> cnt((size_t)ntiles);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), tile_cnt, cnt.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  // tile buckets, first positions (a new chunk per tile) and visiting blocks
  std::vector<int64_t> start((size_t)ntiles), pos((size_t)ntiles);
  std::vector<int32_t> blocks;
  std::vector<int64_t> big;  // tiles sorted on the host
  int64_t acc = 0, chunks = 0;
  for (int64_t t = 0; t < ntiles && e == cudaSuccess; ++t) {
    const int64_t c = cnt[(size_t)t], nch = (c + 31) / 32;
    start[(size_t)t] = acc;
    pos[(size_t)t] = chunks * 32;
    for (int64_t k = 0; k < nch; k += kWarps)
      for (int w = 0; w < kWarps; ++w) blocks.push_back(k + w < nch ? (int32_t)(chunks + k + w) : -1);
    if (c > kTileSortCap) big.push_back(t);
    acc += c;
    chunks += nch;
  }
  L->npos = chunks * 32;
  *nblocks = (int64_t)blocks.size() / kWarps;
  if (e == cudaSuccess) e = cudaMemcpyAsync(tile_start, start.data(), start.size() * sizeof(int64_t),
                                            cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tile_pos, pos.data(), pos.size() * sizeof(int64_t),
                                            cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMalloc(&L->member, (size_t)L->npos * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&L->pos_of, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(d_blocks, blocks.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMemcpyAsync(*d_blocks, blocks.data(), blocks.size() * sizeof(int32_t),
                                            cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(L->member, 0xFF, (size_t)L->npos * sizeof(int32_t), s);
  if (e == cudaSuccess) {
    k_tile_scatter<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, tile_of, tile_start, cursor, bucket);
    k_tile_sort<<<(unsigned)ntiles, 256, 0, s>>>(tile_cnt, tile_start, tile_pos, bucket, local, L->member);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !big.empty()) {  // oversized tiles: (cell, id) order on the host
    std::vector<int32_t> hb((size_t)n);
    std::vector<uint16_t> hl((size_t)n);
    e = cudaMemcpyAsync(hb.data(), bucket, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hl.data(), local, (size_t)n * sizeof(uint16_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int64_t t : big) {
      if (e != cudaSuccess) break;
      int32_t* b = hb.data() + start[(size_t)t];
      const int64_t c = cnt[(size_t)t];
      std::sort(b, b + c, [&](int32_t a, int32_t d) { return hl[a] != hl[d] ? hl[a] < hl[d] : a < d; });
      e = cudaMemcpyAsync(L->member + pos[(size_t)t], b, (size_t)c * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host buffers go out of scope
  }
  if (e == cudaSuccess) {
    k_pos_from_member<<<(unsigned)blocks_for(L->npos), kBlock, 0, s>>>(L->npos, L->member, L->pos_of);
    e = cudaGetLastError();
  }
  cudaFreeAsync(tile_of, s);
  cudaFreeAsync(local, s);
  cudaFreeAsync(tile_cnt, s);
  cudaFreeAsync(cursor, s);
  cudaFreeAsync(bucket, s);
  cudaFreeAsync(tile_start, s);
  cudaFreeAsync(tile_pos, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("spatial layout: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  return PD_OK;
}

}  // namespace pd
