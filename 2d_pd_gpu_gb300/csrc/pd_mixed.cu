// Mixed-precision NOSB step (PD_MIXED): FP32 bond arithmetic, FP64 shape-
// tensor inversion + determinant guard, compensated FP32 force sums.
//
// Variables are scaled so that FP32 works on O(1e-4..1) numbers whatever the
// caller's units: lengths by Ls (the family cutoff), volumes by Vs (mean
// volume), stresses by Es (C11), and the Verlet update is written in
// per-step units:
//   x^ = x/Ls, u^ = u/Ls, V^ = V/Vs,  v^ = v dt/Ls,  a^ = a dt^2/Ls,
//   K^ = sum V^ xi^ (x) xi^,  D^ = sum V^ du^ (x) xi^,  G = D^ K^-1 = F - I,
//   sigma^ = (C/Es) eps,  W^ = V^ sigma^ K^-1,  f^ = W^_i m^_i + sum_j W^_j xi^_ij,
//   a^ = tau2 f^ with tau2 = Es dt^2 / (rho Ls^2).
// Reference positions, displacements, velocities and prescribed velocities
// are two-float pairs (hi + lo, ~48-bit significand): neighbour differences
// (hi_j - hi_i) + (lo_j - lo_i) keep full FP32 relative precision even when
// |u| >> |u_j - u_i|.  The FP64 K^-1 is rounded to FP32 for the per-step
// products.  Nothing here is bit-identical to the FP64 form; its error is
// measured against it (tests/test_gpu_mixed.py, bench.py).
#include "pd_internal.h"
#include "pd_stage.cuh"
#include "pd_walk.cuh"

namespace pd {

namespace {

__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = a + b;
  const float z = s - a;
  const float e = (a - (s - z)) + (b - z);
  return make_float2(s, e);
}

// (hi, lo) + d  -> renormalised pair
__device__ __forceinline__ void tf_add(float& hi, float& lo, float d) {
  const float2 s = two_sum(hi, d);
  const float l = s.y + lo;
  hi = s.x + l;
  lo = l - (hi - s.x);
}

// (hi, lo) + (dh, dl)
__device__ __forceinline__ void tf_add2(float& hi, float& lo, float dh, float dl) {
  const float2 s = two_sum(hi, dh);
  const float l = s.y + (lo + dl);
  hi = s.x + l;
  lo = l - (hi - s.x);
}

// Packed FP32x2 (Blackwell FFMA2 / FADD2 / FMUL2): the bond math is 2-vector
// (x, y) work, so one instruction does both components.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// (hi_j + lo_j) - (hi_i + lo_i) for two-float 2-vectors {hi.x, hi.y, lo.x, lo.y}
__device__ __forceinline__ float2 tf_diff2(float4 j, float2 nhi, float2 nlo) {
  return add2(add2(f2(j.x, j.y), nhi), add2(f2(j.z, j.w), nlo));
}

__device__ __forceinline__ int64_t slot0(const MixedArgs& a, int64_t i, int* w) {
  const int64_t c = i >> 5;
  *w = a.chunk_w[c];
  return a.chunk_base[c] + (i & 31);
}

// K^-1 (FP64 inversion + guard) and m^ from the FP64 reference positions.
__device__ void kinv_update_mixed(const MixedArgs& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  const double2 xi = a.x[i];
  double k11 = 0.0, k12 = 0.0, k22 = 0.0, mx = 0.0, my = 0.0;
  int nal = 0;
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = a.nbr[s];
    if (j < 0) continue;
    const double2 xj = a.x[j];
    const double ex = (xj.x - xi.x) * a.inv_ls, ey = (xj.y - xi.y) * a.inv_ls;
    const double vj = a.vol[j] * a.inv_vs;
    const double t0 = vj * ex, t1 = vj * ey;
    k11 = fma(t0, ex, k11);
    k12 = fma(t0, ey, k12);
    k22 = fma(t1, ey, k22);
    mx += t0;
    my += t1;
    ++nal;
  }
  const double det = fma(k11, k22, -(k12 * k12));
  const double vi = a.vol[i] * a.inv_vs;
  const int32_t fam = a.fam[i];
  const bool failed = fam > 0 && (double)a.broken[i] / (double)fam > a.damage_fail;
  if (nal == 0 || failed || !(det > a.det_guard * (k11 * k22))) {
    a.geo[i] = make_float4(0.f, 0.f, 0.f, (float)vi);
    a.mh[i] = make_float2(0.f, 0.f);
    a.singular[i] = 1;
    atomicAdd(a.counters + CNT_SINGULAR, 1ull);
    return;
  }
  const double r = 1.0 / det;
  a.geo[i] = make_float4((float)(k22 * r), (float)(-k12 * r), (float)(k11 * r), (float)vi);
  a.mh[i] = make_float2((float)(mx / vi), (float)(my / vi));
  a.singular[i] = 0;
}

__global__ void __launch_bounds__(kBlock) k_init_geometry_mixed(MixedArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) kinv_update_mixed(a, i);
}

// BC + drift of particle i in scaled per-step units; an = a^ of the new force.
__device__ __forceinline__ void drift_mixed(const MixedArgs& a, int64_t i, float4& v, float4& u, float anx,
                                            float any) {
  const int g = a.bc[i];
  const int kind = g ? a.gkind[g - 1] : PD_BC_NONE;
  if (kind == PD_BC_VELOCITY) v = a.gvel[g - 1];
  // u += v + a/2   (v two-float, a/2 FP32)
  tf_add2(u.x, u.z, v.x, v.z);
  tf_add2(u.y, u.w, v.y, v.w);
  tf_add(u.x, u.z, 0.5f * anx);
  tf_add(u.y, u.w, 0.5f * any);
  if (kind == PD_BC_FIXED) u = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void drift_particle_mixed(const MixedArgs& a, int64_t i) {
  float4 v = a.vs[i], u = a.us[i];
  const float2 f = a.fs[i];
  drift_mixed(a, i, v, u, a.tau2 * f.x, a.tau2 * f.y);
  a.vs[i] = v;
  a.us[i] = u;
}

__global__ void __launch_bounds__(kBlock) k_drift_mixed(MixedArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) drift_particle_mixed(a, i);
}

// Pass A of particle i: slots s0 + 32 k, k < w, indices read through idx.
template <bool BREAK, typename Idx>
__device__ __forceinline__ void pass_a_particle_mixed(const MixedArgs& a, int64_t i, int w, int64_t s0, Idx idx) {
  const float4 ui = a.us[i], xi = a.xs[i];
  float d11 = 0.f, d12 = 0.f, d21 = 0.f, d22 = 0.f, ax = 0.f, ay = 0.f;
  int newly = 0;
  struct Nb {
    float4 u, x;
    float v;
  };
  const float2 nxh = f2(-xi.x, -xi.y), nxl = f2(-xi.z, -xi.w), nuh = f2(-ui.x, -ui.y), nul = f2(-ui.z, -ui.w);
  float2 D1 = f2(0.f, 0.f), D2 = f2(0.f, 0.f), A = f2(0.f, 0.f);  // (d11, d12), (d21, d22), (ax, ay)
  walk_bonds<4>(
      w, i, idx, [&](int64_t j) { return Nb{a.us[j], a.xs[j], a.vh[j]}; },
      [&](int k, int j, const Nb& nb) {
        const float2 e = tf_diff2(nb.x, nxh, nxl);  // xi^
        const float2 d = tf_diff2(nb.u, nuh, nul);  // du^
        if (BREAK) {
          const float2 q = mul2(d, fma2(f2(2.f, 2.f), e, d));  // d . (2 xi + d)
          const float2 ee = mul2(e, e);
          if (q.x + q.y > a.s2 * (ee.x + ee.y)) {
            a.nbr[s0 + (int64_t)k * kChunk] = -2 - j;
            ++newly;
            return;
          }
        }
        const float2 vv = f2(nb.v, nb.v);
        const float2 t = mul2(vv, e);
        D1 = fma2(f2(d.x, d.x), t, D1);
        D2 = fma2(f2(d.y, d.y), t, D2);
        A = fma2(vv, d, A);
      });
  d11 = D1.x;
  d12 = D1.y;
  d21 = D2.x;
  d22 = D2.y;
  ax = A.x;
  ay = A.y;
  a.hgs[i] = make_float2(2.f * a.k_hg * ax, 2.f * a.k_hg * ay);
  if (BREAK && newly) {
    atomicAdd(a.counters + CNT_BROKEN, (unsigned long long)newly);
    const int32_t b = a.broken[i] + newly;
    a.broken[i] = b;
    a.damage[i] = (double)b / (double)a.fam[i];
    kinv_update_mixed(a, i);
  }
  if (a.singular[i]) {
    a.ws[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float4 g = a.geo[i];
  const float k11 = g.x, k12 = g.y, k22 = g.z, vi = g.w;
  const float g11 = fmaf(d11, k11, d12 * k12), g12 = fmaf(d11, k12, d12 * k22);
  const float g21 = fmaf(d21, k11, d22 * k12), g22 = fmaf(d21, k12, d22 * k22);
  const float e11 = g11, e22 = g22, e12 = 0.5f * (g12 + g21);
  const float s11 = fmaf(a.c11, e11, a.c12 * e22);
  const float s22 = fmaf(a.c12, e11, a.c11 * e22);
  const float s12 = a.c33 * e12;
  const float kh = -a.k_hg;  // W^ = V^ (sigma^ K^-1 - k^ G), stored by columns {W11, W21, W12, W22}
  a.ws[i] = make_float4(vi * fmaf(kh, g11, fmaf(s11, k11, s12 * k12)), vi * fmaf(kh, g21, fmaf(s12, k11, s22 * k12)),
                        vi * fmaf(kh, g12, fmaf(s11, k12, s12 * k22)), vi * fmaf(kh, g22, fmaf(s12, k12, s22 * k22)));
}

template <bool BREAK>
__device__ __forceinline__ void pass_a_particle_mixed(const MixedArgs& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  pass_a_particle_mixed<BREAK>(a, i, w, s0, GlobalIdx{a.nbr, s0});
}

// Picks the calling warp's chunk (visiting order: the 8 warps of a block run
// chunks that are neighbours in space, so their gathers share L1) and stages
// its indices in shared memory (pd_stage.cuh).  Returns the chunk width, or
// -1 when the warp has nothing to do or its copy timed out (error word set).
__device__ __forceinline__ int stage_warp(const MixedArgs& a, int32_t* stage, uint64_t* bars, int64_t* base,
                                          int64_t* chunk) {
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if ((gw << 5) >= a.n) return -1;  // warp-uniform
  const int64_t c = a.chunk_order[gw];
  *chunk = c;
  const int warp = threadIdx.x >> 5;
  const int w = a.chunk_w[c];
  *base = a.chunk_base[c];
  if (!stage_chunk(stage + (int64_t)warp * a.wmax * 32, a.nbr + *base, w, &bars[warp])) {
    if ((threadIdx.x & 31) == 0) atomicOr(a.counters + CNT_ERROR, (unsigned long long)ERR_STAGE_TIMEOUT);
    return -1;
  }
  return w;
}

template <bool BREAK>
__global__ void __launch_bounds__(kBlock) k_pass_a_mixed(MixedArgs a) {
  extern __shared__ __align__(128) int32_t stage[];
  __shared__ uint64_t bars[kBlock / 32];
  int64_t base, chunk;
  const int w = stage_warp(a, stage, bars, &base, &chunk);
  if (w < 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t i = chunk * 32 + lane;
  if (i >= a.n) return;
  pass_a_particle_mixed<BREAK>(a, i, w, base + lane, SharedIdx{stage + (threadIdx.x >> 5) * a.wmax * 32, lane});
}

// Pass B of particle i: slots s0 + 32 k, k < w, indices read through idx.
template <bool DRIFT, typename Idx>
__device__ __forceinline__ void pass_b_particle_mixed(const MixedArgs& a, int64_t i, int w, Idx idx) {
  const float4 wi = a.ws[i], xi = a.xs[i];
  const float2 m = a.mh[i], h = a.hgs[i];
  // W columns c1 = (W11, W21), c2 = (W12, W22): W v = c1 v.x + c2 v.y
  // compensated (TwoSum) sums S + C of both components at once
  float2 S = fma2(f2(wi.x, wi.y), f2(m.x, m.x), fma2(f2(wi.z, wi.w), f2(m.y, m.y), h)), C = f2(0.f, 0.f);
  const float2 nxh = f2(-xi.x, -xi.y), nxl = f2(-xi.z, -xi.w);
  struct Nb {
    float4 x, w;
  };
  walk_bonds<4>(
      w, i, idx, [&](int64_t j) { return Nb{a.xs[j], a.ws[j]}; },
      [&](int, int, const Nb& nb) {
        const float2 e = tf_diff2(nb.x, nxh, nxl);
        const float2 p = fma2(f2(nb.w.x, nb.w.y), f2(e.x, e.x), mul2(f2(nb.w.z, nb.w.w), f2(e.y, e.y)));
        const float2 s = add2(S, p);
        const float2 z = sub2(s, S);
        C = add2(C, add2(sub2(S, sub2(s, z)), sub2(p, z)));
        S = s;
      });
  const float fx = S.x + C.x, fy = S.y + C.y;
  const float2 fo = a.fs[i];
  const float aox = a.tau2 * fo.x, aoy = a.tau2 * fo.y;
  const float anx = a.tau2 * fx, any = a.tau2 * fy;
  float4 v = a.vs[i];
  tf_add(v.x, v.z, 0.5f * (aox + anx));
  tf_add(v.y, v.w, 0.5f * (aoy + any));
  a.fs[i] = make_float2(fx, fy);
  if (DRIFT) {
    float4 u = a.us[i];
    drift_mixed(a, i, v, u, anx, any);
    a.us[i] = u;
  }
  a.vs[i] = v;
}

template <bool DRIFT>
__device__ __forceinline__ void pass_b_particle_mixed(const MixedArgs& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  pass_b_particle_mixed<DRIFT>(a, i, w, GlobalIdx{a.nbr, s0});
}

template <bool DRIFT>
__global__ void __launch_bounds__(kBlock) k_pass_b_mixed(MixedArgs a) {
  extern __shared__ __align__(128) int32_t stage[];
  __shared__ uint64_t bars[kBlock / 32];
  int64_t base, chunk;
  const int w = stage_warp(a, stage, bars, &base, &chunk);
  if (w < 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t i = chunk * 32 + lane;
  if (i >= a.n) return;
  pass_b_particle_mixed<DRIFT>(a, i, w, SharedIdx{stage + (threadIdx.x >> 5) * a.wmax * 32, lane});
}

// Dynamic shared memory of the staged passes: one chunk of wmax slot rows per warp.
inline size_t stage_bytes(const MixedArgs& a) { return (size_t)(kBlock / 32) * (size_t)a.wmax * 128u; }

// ---- batched plates (see pd_batch.cuh): phase 0 drift, 1 pass A, 2 pass B + drift, 3 pass B
__device__ __forceinline__ void batch_particle_mixed(const MixedArgs& p, int64_t i, int phase) {
  if (phase == 0)
    drift_particle_mixed(p, i);
  else if (phase == 1)
    p.brk ? pass_a_particle_mixed<true>(p, i) : pass_a_particle_mixed<false>(p, i);
  else if (phase == 2)
    pass_b_particle_mixed<true>(p, i);
  else
    pass_b_particle_mixed<false>(p, i);
}

__device__ __forceinline__ void batch_phase_mixed(const MixedArgs* __restrict__ plates,
                                                  const BatchTile* __restrict__ tiles, int ntiles, int phase) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile T = tiles[t];
    const MixedArgs& p = plates[T.plate];
    for (int k = threadIdx.x; k < T.count; k += blockDim.x) batch_particle_mixed(p, T.first + k, phase);
  }
}

__global__ void __launch_bounds__(256) k_batch_persistent_mixed(const MixedArgs* __restrict__ plates,
                                                                const BatchTile* __restrict__ tiles, int ntiles,
                                                                int nsteps, GridBarrier* bar) {
  const unsigned nb = gridDim.x;
  batch_phase_mixed(plates, tiles, ntiles, 0);
  for (int s = 0; s < nsteps; ++s) {
    if (!grid_sync(bar, nb)) return;
    batch_phase_mixed(plates, tiles, ntiles, 1);
    if (!grid_sync(bar, nb)) return;
    batch_phase_mixed(plates, tiles, ntiles, s + 1 < nsteps ? 2 : 3);
  }
}

__global__ void __launch_bounds__(256) k_batch_phase_mixed(const MixedArgs* __restrict__ plates,
                                                           const BatchTile* __restrict__ tiles, int ntiles, int phase) {
  batch_phase_mixed(plates, tiles, ntiles, phase);
}

// FP64 <-> scaled two-float conversions (set/get state; not per step)
__device__ __forceinline__ void split2(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

__global__ void k_to_mixed(MixedArgs a, const double2* u, const double2* v, const double2* f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  float4 o;
  if (u) {
    const double2 q = u[i];
    split2(q.x * a.inv_ls, o.x, o.z);
    split2(q.y * a.inv_ls, o.y, o.w);
    a.us[i] = o;
  }
  if (v) {
    const double2 q = v[i];
    split2(q.x * a.v_scale, o.x, o.z);
    split2(q.y * a.v_scale, o.y, o.w);
    a.vs[i] = o;
  }
  if (f) {
    const double2 q = f[i];
    a.fs[i] = make_float2((float)(q.x * a.f_scale), (float)(q.y * a.f_scale));
  }
}

__global__ void k_from_mixed(MixedArgs a, double2* u, double2* v, double2* f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (u) {
    const float4 q = a.us[i];
    u[i] = make_double2(((double)q.x + (double)q.z) / a.inv_ls, ((double)q.y + (double)q.w) / a.inv_ls);
  }
  if (v) {
    const float4 q = a.vs[i];
    v[i] = make_double2(((double)q.x + (double)q.z) / a.v_scale, ((double)q.y + (double)q.w) / a.v_scale);
  }
  if (f) {
    const float2 q = a.fs[i];
    f[i] = make_double2((double)q.x / a.f_scale, (double)q.y / a.f_scale);
  }
}

__global__ void k_positions_mixed(MixedArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double2 q = a.x[i];
  float4 o;
  split2(q.x * a.inv_ls, o.x, o.z);
  split2(q.y * a.inv_ls, o.y, o.w);
  a.xs[i] = o;
  a.vh[i] = (float)(a.vol[i] * a.inv_vs);
}

}  // namespace

int batch_occupancy_mixed(const BatchLaunch& cfg) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_persistent_mixed, cfg.block, 0) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_batch_mixed(const MixedArgs* d_plates, const BatchTile* d_tiles, int ntiles, int nsteps,
                               const BatchLaunch& cfg, GridBarrier* d_bar, int nsm, cudaStream_t s) {
  if (ntiles <= 0 || nsteps <= 0) return cudaSuccess;
  if (!cfg.persistent) {
    const unsigned g = (unsigned)ntiles;
    k_batch_phase_mixed<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, 0);
    for (int k = 0; k < nsteps; ++k) {
      k_batch_phase_mixed<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, 1);
      k_batch_phase_mixed<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, k + 1 < nsteps ? 2 : 3);
    }
    return cudaGetLastError();
  }
  const int occ = batch_occupancy_mixed(cfg);
  const int bps = cfg.blocks_per_sm < occ ? cfg.blocks_per_sm : occ;
  if (bps < 1) return cudaErrorInvalidConfiguration;
  int grid = nsm * bps;
  if (grid > ntiles) grid = ntiles;
  cudaError_t e = cudaMemsetAsync(d_bar, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)grid);
  lc.blockDim = dim3((unsigned)cfg.block);
  lc.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  lc.attrs = at;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k_batch_persistent_mixed, d_plates, d_tiles, ntiles, nsteps, d_bar);
}

void launch_init_geometry_mixed(const MixedArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  // the staged passes may take up to 8 warps x PD_MAX_FAMILY rows x 128 B of dynamic shared memory
  const int mx = (kBlock / 32) * PD_MAX_FAMILY * 128;
  cudaFuncSetAttribute(k_pass_a_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_a_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_b_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_b_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  k_positions_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a);
  k_init_geometry_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a);
}

void launch_drift_mixed(const MixedArgs& a, cudaStream_t s) {
  if (a.n > 0) k_drift_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a);
}

void launch_pass_a_mixed(const MixedArgs& a, bool breaking, cudaStream_t s) {
  if (a.n <= 0) return;
  const size_t sm = stage_bytes(a);
  if (breaking)
    k_pass_a_mixed<true><<<(unsigned)blocks_for(a.n), kBlock, sm, s>>>(a);
  else
    k_pass_a_mixed<false><<<(unsigned)blocks_for(a.n), kBlock, sm, s>>>(a);
}

void launch_pass_b_mixed(const MixedArgs& a, bool drift, cudaStream_t s) {
  if (a.n <= 0) return;
  const size_t sm = stage_bytes(a);
  if (drift)
    k_pass_b_mixed<true><<<(unsigned)blocks_for(a.n), kBlock, sm, s>>>(a);
  else
    k_pass_b_mixed<false><<<(unsigned)blocks_for(a.n), kBlock, sm, s>>>(a);
}

void launch_to_mixed(const MixedArgs& a, const double2* u, const double2* v, const double2* f, cudaStream_t s) {
  if (a.n > 0) k_to_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, u, v, f);
}

void launch_from_mixed(const MixedArgs& a, double2* u, double2* v, double2* f, cudaStream_t s) {
  if (a.n > 0) k_from_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, u, v, f);
}

}  // namespace pd
