// Family (neighbour) build on the GPU and the SELL-32 bond layout.
//
// Replaces findNeighbor (src/SetupParticleSystem.cpp:100-121), an O(N^2)
// all-pairs loop, with a uniform cell list (cell >= cutoff, 3x3 stencil):
//   cell index + count -> scan -> scatter -> per-particle candidate test ->
//   count -> scan (row_ptr) -> fill with an in-register insertion sort so that
//   each family is in ascending neighbour id, the reference's order
//   (findNeighbor scans j upward).  The pair test is the reference's
//   `sqrt(d2) < 1.01*dx*horizon` with the caller's cutoff, evaluated in IEEE
//   binary64 with no contraction (this file is compiled with --fmad=false), so
//   it decides exactly as the oracle's restatement.  Bonds that properly
//   cross a crack segment are dropped (pre-crack; no reference counterpart).
#include <cmath>
#include <cstdio>

#include "pd_internal.h"

namespace pd {

namespace {

__device__ __forceinline__ double orient(double ax, double ay, double bx, double by, double px, double py) {
  const double d1 = (bx - ax) * (py - ay);
  const double d2 = (by - ay) * (px - ax);
  return d1 - d2;
}

__device__ __forceinline__ bool crosses(double px, double py, double qx, double qy, const double* c) {
  const double o1 = orient(c[0], c[1], c[2], c[3], px, py);
  const double o2 = orient(c[0], c[1], c[2], c[3], qx, qy);
  const double o3 = orient(px, py, qx, qy, c[0], c[1]);
  const double o4 = orient(px, py, qx, qy, c[2], c[3]);
  return ((o1 > 0.0 && o2 < 0.0) || (o1 < 0.0 && o2 > 0.0)) && ((o3 > 0.0 && o4 < 0.0) || (o3 < 0.0 && o4 > 0.0));
}

// The pre-crack segments of one family build, passed by value (a kernel
// parameter, read in place through __grid_constant__), so builds of several
// contexts can run at once.  box: each segment's bounding box in FP32,
// widened by a margin: a bond whose box misses a crack's box cannot properly
// cross it, so the exact FP64 test runs only near cracks.
struct CrackSet {
  int32_t n;
  double seg[PD_MAX_CRACKS * 4];
  float box[PD_MAX_CRACKS * 4];
};

struct Grid {
  double x0, y0, inv_cs;
  int64_t gx, gy;
  float c2_lo, c2_hi;  // cutoff^2 (1 -+ 4e-6): FP32 accept / reject bounds of the pair test
};

// The pair test sqrt(d2) < cutoff of the oracle, decided in FP32 when the
// FP32 squared distance is clearly inside or outside.  rx, ry are the exact
// FP64 differences; rounding them to FP32 and the FP32 squares and sum move
// d2 by < 2.5e-7 relative, far inside the 4e-6 band, so only pairs within the
// band (none on a jittered lattice) take the exact FP64 path.
__device__ __forceinline__ bool within_cutoff(double rx, double ry, double cutoff, const Grid& G) {
  const float fx = (float)rx, fy = (float)ry;
  const float q = fmaf(fx, fx, fy * fy);
  if (q < G.c2_lo) return true;
  if (q > G.c2_hi) return false;
  return sqrt(rx * rx + ry * ry) < cutoff;
}

__device__ __forceinline__ bool near_crack(float ax, float ay, float bx, float by, const float* box) {
  return fmaxf(ax, bx) >= box[0] && fminf(ax, bx) <= box[2] && fmaxf(ay, by) >= box[1] && fminf(ay, by) <= box[3];
}

__device__ __forceinline__ int64_t cell_coord(double v, double v0, double inv_cs, int64_t g) {
  int64_t c = (int64_t)floor((v - v0) * inv_cs);
  return c < 0 ? 0 : (c >= g ? g - 1 : c);
}

__global__ void k_cell_index(int64_t n, const double2* __restrict__ x, Grid G, int64_t* cell_of,
                             unsigned long long* cell_count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 p = x[i];
  const int64_t c = cell_coord(p.y, G.y0, G.inv_cs, G.gy) * G.gx + cell_coord(p.x, G.x0, G.inv_cs, G.gx);
  cell_of[i] = c;
  atomicAdd(cell_count + c, 1ull);
}

__global__ void k_cell_fill(int64_t n, const int64_t* cell_of, const int64_t* cell_start,
                            unsigned long long* cursor, int32_t* items) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t c = cell_of[i];
  const unsigned long long k = atomicAdd(cursor + c, 1ull);
  items[cell_start[c] + (int64_t)k] = (int32_t)i;
}

// Count (FILL = false) or write the family of each particle.
template <bool FILL>
__global__ void k_family(int64_t n, const double2* __restrict__ x, Grid G, const int64_t* __restrict__ cell_start,
                         const int32_t* __restrict__ items, double cutoff, const __grid_constant__ CrackSet cr,
                         int64_t* deg,
                         const int64_t* __restrict__ row_ptr, int32_t* col, unsigned long long* counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 pi = x[i];
  const int64_t cx = cell_coord(pi.x, G.x0, G.inv_cs, G.gx);
  const int64_t cy = cell_coord(pi.y, G.y0, G.inv_cs, G.gy);
  int32_t buf[FILL ? PD_MAX_FAMILY : 1];
  int cnt = 0;
  for (int64_t dy = -1; dy <= 1; ++dy) {
    const int64_t yy = cy + dy;
    if (yy < 0 || yy >= G.gy) continue;
    for (int64_t dx = -1; dx <= 1; ++dx) {
      const int64_t xx = cx + dx;
      if (xx < 0 || xx >= G.gx) continue;
      const int64_t c = yy * G.gx + xx;
      for (int64_t k = cell_start[c]; k < cell_start[c + 1]; ++k) {
        const int32_t j = items[k];
        if ((int64_t)j == i) continue;
        const double2 pj = x[j];
        if (!within_cutoff(pj.x - pi.x, pj.y - pi.y, cutoff, G)) continue;
        bool cut = false;
        for (int q = 0; q < cr.n && !cut; ++q)
          cut = near_crack((float)pi.x, (float)pi.y, (float)pj.x, (float)pj.y, cr.box + 4 * q) &&
                crosses(pi.x, pi.y, pj.x, pj.y, cr.seg + 4 * q);
        if (cut) continue;
        if (FILL) {
          if (cnt < PD_MAX_FAMILY) {
            int p = cnt;
            while (p > 0 && buf[p - 1] > j) {
              buf[p] = buf[p - 1];
              --p;
            }
            buf[p] = j;
          }
        }
        ++cnt;
      }
    }
  }
  if (!FILL) {
    if (cnt > PD_MAX_FAMILY) atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_FAMILY_OVERFLOW);
    deg[i] = cnt;
  } else {
    const int64_t o = row_ptr[i];
    const int m = cnt < PD_MAX_FAMILY ? cnt : PD_MAX_FAMILY;
    for (int k = 0; k < m; ++k) col[o + k] = buf[k];
  }
}

// ---- scan (3 phases: tile scan, single-block scan of tile sums, add)
constexpr int kScanItems = 4;
constexpr int kScanTile = kBlock * kScanItems;

__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[kBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < kBlock / 32 ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < kBlock / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const int64_t wpre = wid > 0 ? warp_sums[wid - 1] : 0;
  *total = warp_sums[kBlock / 32 - 1];
  __syncthreads();
  return wpre + incl - v;
}

__global__ void k_scan_tiles(const int64_t* in, int64_t* out, int64_t n, int64_t* tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems], s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int64_t total;
  int64_t pre = block_excl_scan(s, &total);
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int64_t* sums, int64_t nt, int64_t* out_total) {
  int64_t carry = 0;
  for (int64_t b = 0; b < nt; b += kBlock) {
    const int64_t idx = b + threadIdx.x;
    const int64_t v = idx < nt ? sums[idx] : 0;
    int64_t total;
    const int64_t pre = block_excl_scan(v, &total);
    if (idx < nt) sums[idx] = carry + pre;
    carry += total;
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* tile_off) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

// ---- SELL-32
__global__ void k_chunk_width(int64_t npos, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ member,
                              int64_t nchunks, int32_t* chunk_w, int64_t* chunk_slots) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  int64_t w = 0;
  for (int l = 0; l < kChunk; ++l) {
    const int64_t p = c * kChunk + l;
    if (p < npos) {
      const int64_t i = sell_member(member, p);
      if (i < 0) continue;  // a hole
      const int64_t d = row_ptr[i + 1] - row_ptr[i];
      w = d > w ? d : w;
    }
  }
  chunk_w[c] = (int32_t)w;
  chunk_slots[c] = w * kChunk;
}

// Slot (0 .. deg) of family entry k of a particle whose family is
// col[r0 .. r0 + deg): k itself (family order), or with a spatial key array
// the entry's place in ascending (rk of the neighbour, k) order; entries that
// are not valid neighbour ids sort last.
__device__ __forceinline__ int64_t family_slot(const int32_t* __restrict__ col, int64_t r0, int64_t deg, int64_t k,
                                               const uint64_t* __restrict__ rk, int64_t n) {
  if (!rk) return k;
  auto key = [&](int64_t q) {
    const int32_t j = col[r0 + q];
    return j >= 0 && (int64_t)j < n ? rk[j] : ~0ull;
  };
  const uint64_t kk = key(k);
  int64_t slot = 0;
  for (int64_t q = 0; q < deg; ++q) {
    const uint64_t kq = key(q);
    slot += kq < kk || (kq == kk && q < k);
  }
  return slot;
}

// nbr: every slot is padding (-1) before the fill.
__global__ void k_sell_fill(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                            const int64_t* __restrict__ chunk_base, const int32_t* __restrict__ pos_of,
                            const uint64_t* __restrict__ rk, int32_t* nbr, unsigned long long* counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = sell_slot0(chunk_base, sell_pos(pos_of, i));
  const int64_t r0 = row_ptr[i], deg = row_ptr[i + 1] - r0;
  for (int64_t k = 0; k < deg; ++k) {
    int32_t j = col[r0 + k];
    if (j < 0 || (int64_t)j >= n) {
      atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_BAD_NEIGHBOR);
      j = -1;
    } else if ((int64_t)j == i) {
      atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_SELF_BOND);
      j = -1;
    }
    nbr[s0 + family_slot(col, r0, deg, k, rk, n) * kChunk] = j;
  }
}

// Stretch limits of a bond: the exact FP64 one, and the FP32 certificate
// threshold (s_c |xi|)^2 (1 - 1e-5) rounded toward zero (never above the truth).
__device__ __forceinline__ void bond_limits(double ex, double ey, double s_c, double* lim, float* r2) {
  const double ee = fma(ex, ex, ey * ey);
  const double s2 = s_c > 0.0 ? s_c * (2.0 + s_c) : INFINITY;
  *lim = s2 * ee;
  *r2 = s_c > 0.0 ? __double2float_rz(((s_c * s_c) * ee) * (1.0 - 1e-5)) : 0.0f;
}

__global__ void k_bond_geometry(int64_t n, const double2* __restrict__ x, const double* __restrict__ vol,
                                const int64_t* __restrict__ chunk_base, const int32_t* __restrict__ chunk_w,
                                const int32_t* __restrict__ pos_of, const int32_t* __restrict__ nbr, double s_c,
                                double2* bxi, double2* bgeo, double* blim, float* br2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t p = sell_pos(pos_of, i);
  const int w = chunk_w[p >> 5];
  const int64_t s0 = sell_slot0(chunk_base, p);
  const double2 pi = x[i];
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    int32_t j = nbr[s];
    if (j < -1) j = -2 - j;  // broken bonds keep their geometry
    if (j < 0) {
      bxi[s] = make_double2(0.0, 0.0);
      bgeo[s] = make_double2(0.0, 0.0);
      blim[s] = 0.0;
      br2[s] = 0.0f;
      continue;
    }
    const double2 pj = x[j];
    const double ex = pj.x - pi.x, ey = pj.y - pi.y;
    const double vj = vol[j];
    bxi[s] = make_double2(ex, ey);
    bgeo[s] = make_double2(vj * ex, vj * ey);
    bond_limits(ex, ey, s_c, &blim[s], &br2[s]);
  }
}

__global__ void k_bond_limit(int64_t nslots, const double2* __restrict__ bxi, double s_c,
                             const int32_t* __restrict__ nbr, double* blim, float* br2) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const double2 e = bxi[s];
  if (nbr[s] == -1) {
    blim[s] = 0.0;
    br2[s] = 0.0f;
  } else {
    bond_limits(e.x, e.y, s_c, &blim[s], &br2[s]);
  }
}

__global__ void k_mask_out(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                           const int64_t* __restrict__ chunk_base, const int32_t* __restrict__ pos_of,
                           const uint64_t* __restrict__ rk, const int32_t* __restrict__ nbr, uint8_t* alive) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = sell_slot0(chunk_base, sell_pos(pos_of, i));
  const int64_t r0 = row_ptr[i], deg = row_ptr[i + 1] - r0;
  for (int64_t k = 0; k < deg; ++k)
    alive[r0 + k] = nbr[s0 + family_slot(col, r0, deg, k, rk, n) * kChunk] >= 0 ? 1 : 0;
}

// Restore every family bond to intact (pd_reset).
__global__ void k_sell_reset(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                             const int64_t* __restrict__ chunk_base, const int32_t* __restrict__ pos_of,
                             const uint64_t* __restrict__ rk, int32_t* nbr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = sell_slot0(chunk_base, sell_pos(pos_of, i));
  const int64_t r0 = row_ptr[i], deg = row_ptr[i + 1] - r0;
  for (int64_t k = 0; k < deg; ++k) {
    const int64_t s = s0 + family_slot(col, r0, deg, k, rk, n) * kChunk;
    if (nbr[s] < -1) nbr[s] = col[r0 + k];
  }
}

}  // namespace

void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  int64_t* sums = nullptr;
  cudaMallocAsync(&sums, (size_t)(nt > 0 ? nt : 1) * sizeof(int64_t), s);
  if (nt > 0) k_scan_tiles<<<(unsigned)nt, kBlock, 0, s>>>(in, out, n, sums);
  k_scan_sums<<<1, kBlock, 0, s>>>(sums, nt, out + n);
  if (n > 0) k_scan_add<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(out, n, sums);
  cudaFreeAsync(sums, s);
}

int build_families_gpu(int64_t n, const double2* d_x, const double* h_x, double cutoff, int n_cracks,
                       const double* h_cracks, cudaStream_t s, FamilyBuild* out, std::string* msg) {
  if (n_cracks < 0 || n_cracks > PD_MAX_CRACKS) {
    *msg = "n_cracks out of range";
    return PD_ERR_ARG;
  }
  if (!(cutoff > 0.0) || !std::isfinite(cutoff)) {
    *msg = "cutoff must be positive and finite";
    return PD_ERR_ARG;
  }
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (int64_t i = 0; i < n; ++i) {
    xmin = fmin(xmin, h_x[2 * i]);
    xmax = fmax(xmax, h_x[2 * i]);
    ymin = fmin(ymin, h_x[2 * i + 1]);
    ymax = fmax(ymax, h_x[2 * i + 1]);
  }
  if (n == 0) xmin = xmax = ymin = ymax = 0.0;
  double cs = cutoff * 1.0000001;
  Grid G;
  for (;;) {
    G.gx = (int64_t)floor((xmax - xmin) / cs) + 1;
    G.gy = (int64_t)floor((ymax - ymin) / cs) + 1;
    if ((double)G.gx * (double)G.gy <= 4.0 * (double)n + 4096.0) break;
    cs *= 2.0;  // sparse clouds: larger cells, still a superset of the cutoff disc
  }
  G.x0 = xmin;
  G.y0 = ymin;
  G.inv_cs = 1.0 / cs;
  const double c2 = cutoff * cutoff;
  if (c2 > 1e-30 && c2 < 1e30) {  // FP32 pre-filter only where FP32 holds c^2 with full precision
    G.c2_lo = (float)(c2 * (1.0 - 4e-6));
    G.c2_hi = (float)(c2 * (1.0 + 4e-6));
  } else {
    G.c2_lo = -1.0f;
    G.c2_hi = INFINITY;
  }
  const int64_t nc = G.gx * G.gy;
  CrackSet cr{};
  cr.n = n_cracks;
  if (n_cracks > 0) {
    for (int q = 0; q < 4 * n_cracks; ++q) cr.seg[q] = h_cracks[q];
    // crack boxes widened by far more than the FP32 rounding of any coordinate
    double big = fmax(fmax(fabs(xmin), fabs(xmax)), fmax(fabs(ymin), fabs(ymax)));
    for (int q = 0; q < 4 * n_cracks; ++q) big = fmax(big, fabs(h_cracks[q]));
    const double m = 1e-5 * big + 1e-300;
    for (int q = 0; q < n_cracks; ++q) {
      const double* c = h_cracks + 4 * q;
      cr.box[4 * q + 0] = (float)(fmin(c[0], c[2]) - m);
      cr.box[4 * q + 1] = (float)(fmin(c[1], c[3]) - m);
      cr.box[4 * q + 2] = (float)(fmax(c[0], c[2]) + m);
      cr.box[4 * q + 3] = (float)(fmax(c[1], c[3]) + m);
    }
  }

  int64_t *cell_of = nullptr, *cell_start = nullptr, *deg = nullptr;
  unsigned long long *cnt = nullptr, *counters = nullptr;
  int32_t* items = nullptr;
  const size_t nn = (size_t)(n > 0 ? n : 1);
  cudaMallocAsync(&cell_of, nn * sizeof(int64_t), s);
  cudaMallocAsync(&cell_start, (size_t)(nc + 1) * sizeof(int64_t), s);
  cudaMallocAsync(&cnt, (size_t)nc * sizeof(unsigned long long), s);
  cudaMallocAsync(&items, nn * sizeof(int32_t), s);
  cudaMallocAsync(&deg, nn * sizeof(int64_t), s);
  cudaMallocAsync(&counters, CNT_N * sizeof(unsigned long long), s);
  cudaMallocAsync(&out->row_ptr, (size_t)(n + 1) * sizeof(int64_t), s);
  cudaMemsetAsync(cnt, 0, (size_t)nc * sizeof(unsigned long long), s);
  cudaMemsetAsync(counters, 0, CNT_N * sizeof(unsigned long long), s);
  const unsigned nb = (unsigned)blocks_for(n > 0 ? n : 1);
  if (n > 0) k_cell_index<<<nb, kBlock, 0, s>>>(n, d_x, G, cell_of, cnt);
  scan_exclusive_i64(reinterpret_cast<const int64_t*>(cnt), cell_start, nc, s);
  cudaMemsetAsync(cnt, 0, (size_t)nc * sizeof(unsigned long long), s);
  if (n > 0) {
    k_cell_fill<<<nb, kBlock, 0, s>>>(n, cell_of, cell_start, cnt, items);
    k_family<false><<<nb, kBlock, 0, s>>>(n, d_x, G, cell_start, items, cutoff, cr, deg, nullptr, nullptr,
                                          counters);
  }
  scan_exclusive_i64(deg, out->row_ptr, n, s);
  unsigned long long h_cnt[CNT_N];
  cudaMemcpyAsync(&out->nnz, out->row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(h_cnt, counters, sizeof(h_cnt), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("family count: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  int rc = PD_OK;
  if (h_cnt[CNT_ERROR] & ERR_FAMILY_OVERFLOW) {
    *msg = "a family exceeds PD_MAX_FAMILY bonds (cutoff too large for the spacing)";
    rc = PD_ERR_CAPACITY;
  } else {
    cudaMallocAsync(&out->col, (size_t)(out->nnz > 0 ? out->nnz : 1) * sizeof(int32_t), s);
    if (n > 0)
      k_family<true><<<nb, kBlock, 0, s>>>(n, d_x, G, cell_start, items, cutoff, cr, nullptr, out->row_ptr,
                                           out->col, counters);
  }
  cudaFreeAsync(cell_of, s);
  cudaFreeAsync(cell_start, s);
  cudaFreeAsync(cnt, s);
  cudaFreeAsync(items, s);
  cudaFreeAsync(deg, s);
  cudaFreeAsync(counters, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("family fill: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  return rc;
}

int build_sell(int64_t n, const int64_t* d_row_ptr, const int32_t* d_col, cudaStream_t s, SellLayout* L,
               unsigned long long* d_counters, std::string* msg) {
  if (!L->member) L->npos = n;
  L->nchunks = (L->npos + kChunk - 1) / kChunk;
  int64_t* slots = nullptr;
  const size_t nch = (size_t)(L->nchunks > 0 ? L->nchunks : 1);
  cudaMallocAsync(&L->chunk_w, nch * sizeof(int32_t), s);
  cudaMallocAsync(&L->chunk_base, (nch + 1) * sizeof(int64_t), s);
  cudaMallocAsync(&slots, nch * sizeof(int64_t), s);
  if (L->nchunks > 0)
    k_chunk_width<<<(unsigned)blocks_for(L->nchunks), kBlock, 0, s>>>(L->npos, d_row_ptr, L->member, L->nchunks,
                                                                      L->chunk_w, slots);
  scan_exclusive_i64(slots, L->chunk_base, L->nchunks, s);
  cudaMemcpyAsync(&L->nslots, L->chunk_base + L->nchunks, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(slots, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("sell layout: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  if (cudaMalloc(&L->nbr, (size_t)(L->nslots > 0 ? L->nslots : 1) * sizeof(int32_t)) != cudaSuccess) {
    *msg = "out of device memory (bond slots)";
    return PD_ERR_CAPACITY;
  }
  // every slot starts as padding: the lanes past n of the last chunk own slots no particle fills
  if (L->nslots > 0) cudaMemsetAsync(L->nbr, 0xFF, (size_t)L->nslots * sizeof(int32_t), s);
  if (n > 0)
    k_sell_fill<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, d_row_ptr, d_col, L->chunk_base, L->pos_of, L->rk,
                                                          L->nbr, d_counters);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("sell fill: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  return PD_OK;
}

void launch_bond_geometry_fp64(int64_t n, const double2* x, const double* vol, const SellLayout& L,
                               const int64_t* /*row_ptr*/, double s_c, double2* bxi, double2* bgeo, double* blim,
                               float* br2, cudaStream_t s) {
  if (n > 0)
    k_bond_geometry<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, x, vol, L.chunk_base, L.chunk_w, L.pos_of, L.nbr,
                                                              s_c, bxi, bgeo, blim, br2);
}

void launch_bond_limit_fp64(int64_t nslots, const double2* bxi, double s_c, const int32_t* nbr, double* blim,
                            float* br2, cudaStream_t s) {
  if (nslots > 0) k_bond_limit<<<(unsigned)blocks_for(nslots), kBlock, 0, s>>>(nslots, bxi, s_c, nbr, blim, br2);
}

void launch_mask_out(int64_t n, const int64_t* row_ptr, const int32_t* col, const SellLayout& L, uint8_t* alive,
                     cudaStream_t s) {
  if (n > 0)
    k_mask_out<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, row_ptr, col, L.chunk_base, L.pos_of, L.rk, L.nbr,
                                                         alive);
}

void launch_sell_reset(int64_t n, const int64_t* row_ptr, const int32_t* col, const SellLayout& L, cudaStream_t s) {
  if (n > 0)
    k_sell_reset<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, row_ptr, col, L.chunk_base, L.pos_of, L.rk, L.nbr);
}

}  // namespace pd
