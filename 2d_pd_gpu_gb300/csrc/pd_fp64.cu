// FP64 explicit NOSB step (the plain form).  Compiled with --fmad=false: the
// only fused multiply-adds are the explicit fma() calls, written in the same
// places as the oracle's restatement, so results are bit-identical to it.
//
// One thread per particle, bonds walked in family order through the SELL-32
// layout (every slot load of a warp is one coalesced line).  Per-particle sums
// are sequential in family order, with no atomics, so results are
// deterministic and independent of the launch shape.
//
// Reference correspondence (src/main_seq.cpp):
//   k_drift / pass B tail : applyVelocityBC :28-36, updatePositions :386-393,
//                           applyFixedBC :38-46
//   k_pass_a              : computeShapeTensors :71-156 (n1=n2=0: one K per
//                           particle), computeStressTensor :204-268,
//                           S = sigma K^-1 of computeForceDensityStates :355
//   k_pass_b              : computeVelocity :396-470 in gather form
//                           f_i = sum_j V_j (S_i + S_j) xi_ij (= T_ij - T_ji)
// FP64 operations per bond: pass A 11 (d 2, stretch test 5, D 4) + 2 with the
// zero-energy-mode penalty (sum V_j d), pass B 4.  The stretch test runs in
// FP64 only for bonds an FP32 bound cannot prove intact (surely_intact), so
// pass A costs 8 FP64 operations for almost every bond.
#include "pd_internal.h"
#include "pd_walk.cuh"

namespace pd {

namespace {

__device__ __forceinline__ int64_t slot0(const Fp64Args& a, int64_t i, int* w) {
  const int64_t c = i >> 5;
  *w = a.chunk_w[c];
  return a.chunk_base[c] + (i & 31);
}

// K^-1 and m/V of particle i over its intact bonds (oracle: kinv_of).
__device__ void kinv_update(const Fp64Args& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  double k11 = 0.0, k12 = 0.0, k22 = 0.0, mx = 0.0, my = 0.0;
  int nal = 0;
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    if (a.nbr[s] < 0) continue;
    const double2 e = a.bxi[s];
    const double2 t = a.bgeo[s];
    k11 = fma(t.x, e.x, k11);
    k12 = fma(t.x, e.y, k12);
    k22 = fma(t.y, e.y, k22);
    mx = mx + t.x;
    my = my + t.y;
    ++nal;
  }
  const double det = fma(k11, k22, -(k12 * k12));
  const int32_t fam = a.fam[i];
  const bool failed = fam > 0 && (double)a.broken[i] / (double)fam > a.damage_fail;
  if (nal == 0 || failed || !(det > a.det_guard * (k11 * k22))) {
    a.kinv01[i] = make_double2(0.0, 0.0);
    a.kinv22[i] = 0.0;
    a.mt[i] = make_double2(0.0, 0.0);
    a.singular[i] = 1;
    atomicAdd(a.counters + CNT_SINGULAR, 1ull);
    return;
  }
  const double r = 1.0 / det;
  a.kinv01[i] = make_double2(k22 * r, -k12 * r);
  a.kinv22[i] = k11 * r;
  const double rv = 1.0 / a.vol[i];
  a.mt[i] = make_double2(mx * rv, my * rv);
  a.singular[i] = 0;
}

__global__ void __launch_bounds__(kBlock) k_init_geometry(Fp64Args a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  kinv_update(a, i);
}

// Velocity BC, drift, fixed BC of particle i; an = f_i / rho.
__device__ __forceinline__ void drift_one(const Fp64Args& a, int64_t i, double2& v, double2& u, double anx,
                                          double any) {
  const int g = a.bc[i];
  const int kind = g ? a.gkind[g - 1] : PD_BC_NONE;
  if (kind == PD_BC_VELOCITY) v = a.gval[g - 1];
  u.x = u.x + (v.x * a.dt + (0.5 * anx) * a.dt2);
  u.y = u.y + (v.y * a.dt + (0.5 * any) * a.dt2);
  if (kind == PD_BC_FIXED) u = make_double2(0.0, 0.0);
}

__device__ __forceinline__ void drift_particle(const Fp64Args& a, int64_t i) {
  double2 v = a.in_v ? a.in_v[i] : a.v[i], u = a.in_u ? a.in_u[i] : a.u[i];
  const double2 f = a.in_f ? a.in_f[i] : a.f[i];
  if (a.in_f) a.f[i] = f;
  drift_one(a, i, v, u, f.x * a.inv_rho, f.y * a.inv_rho);
  a.v[i] = v;
  a.u[i] = u;
  a.u32[i] = make_float2((float)u.x, (float)u.y);
}

__global__ void __launch_bounds__(kBlock) k_drift(Fp64Args a) {
  const int64_t i = a.i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) drift_particle(a, i);
}

// The FP32 shadow of u for particles i0 <= i < n; with in_u / in_v / in_a
// set (pd_compute_velocity on page-locked buffers), u, velocity and acce are
// first read from host memory into the device state.
__global__ void __launch_bounds__(kBlock) k_shadow(Fp64Args a) {
  const int64_t i = a.i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double2 u = a.in_u ? a.in_u[i] : a.u[i];
  if (a.in_u) a.u[i] = u;
  if (a.in_v) a.v[i] = a.in_v[i];
  if (a.in_a) a.acc[i] = a.in_a[i];
  a.u32[i] = make_float2((float)u.x, (float)u.y);
}

// FP32 certificate that a bond is intact: an upper bound B on the FP64
// |d| = |fl64(u_j - u_i)| from the FP32 shadows (|u - fl32(u)| <= 2^-24 |u|,
// FP32 rounding of the difference and of B itself covered by the 6e-8 and
// 1.000001 factors) with B^2 <= (s_c |xi|)^2 (1 - 1e-5).  Then
// d.(2 xi + d) <= 2|xi|B + B^2 < ((1 + s_c)^2 - 1)|xi|^2 by a relative
// margin >= 5e-6, far above the FP64 evaluation error of the exact test, so
// the FP64 test would say "intact": skipping it cannot change any result.
__device__ __forceinline__ bool surely_intact(float2 ui, float2 uj, float r2) {
  const float fx = uj.x - ui.x, fy = uj.y - ui.y;
  const float bx = fabsf(fx) + 6.0e-8f * (fabsf(uj.x) + fabsf(ui.x) + fabsf(fx));
  const float by = fabsf(fy) + 6.0e-8f * (fabsf(uj.y) + fabsf(ui.y) + fabsf(fy));
  return fmaf(bx, bx, by * by) * 1.000001f <= r2;
}

// Pass A of particle i (stretch tests, D, penalty sum, stress, W).
template <bool BREAK, bool HG>
__device__ __forceinline__ void pass_a_particle(const Fp64Args& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  const double2 ui = a.u[i];
  const float2 ui32 = a.u32[i];
  double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0, ax = 0.0, ay = 0.0;
  int newly = 0;
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = a.nbr[s];
    if (j < 0) continue;
    const double2 uj = a.u[j];
    const double dx = uj.x - ui.x, dy = uj.y - ui.y;
    if (BREAK && !surely_intact(ui32, a.u32[j], __ldcs(&a.br2[s]))) {
      const double2 e = __ldcs(&a.bxi[s]);
      const double q = fma(dx, fma(2.0, e.x, dx), dy * fma(2.0, e.y, dy));
      if (q > __ldcs(&a.blim[s])) {
        a.nbr[s] = -2 - j;
        ++newly;
        continue;
      }
    }
    const double2 t = __ldcs(&a.bgeo[s]);
    d11 = fma(dx, t.x, d11);
    d12 = fma(dx, t.y, d12);
    d21 = fma(dy, t.x, d21);
    d22 = fma(dy, t.y, d22);
    if (HG) {
      const double vj = a.vol[j];
      ax = fma(vj, dx, ax);
      ay = fma(vj, dy, ay);
    }
  }
  if (HG) {
    const double k2 = 2.0 * a.k_hg;
    a.hg[i] = make_double2(k2 * ax, k2 * ay);
  }
  if (BREAK && newly) {
    atomicAdd(a.counters + CNT_BROKEN, (unsigned long long)newly);
    const int32_t b = a.broken[i] + newly;
    a.broken[i] = b;
    a.damage[i] = (double)b / (double)a.fam[i];
    kinv_update(a, i);
  }
  if (a.singular[i]) {
    a.w01[i] = make_double2(0.0, 0.0);
    a.w23[i] = make_double2(0.0, 0.0);
    return;
  }
  const double2 k01 = a.kinv01[i];
  const double k11 = k01.x, k12 = k01.y, k22 = a.kinv22[i];
  // G = D K^-1 = F - I
  const double g11 = fma(d11, k11, d12 * k12), g12 = fma(d11, k12, d12 * k22);
  const double g21 = fma(d21, k11, d22 * k12), g22 = fma(d21, k12, d22 * k22);
  const double e11 = g11, e22 = g22, e12 = 0.5 * (g12 + g21);
  const double s11 = fma(a.c11, e11, a.c12 * e22);
  const double s22 = fma(a.c12, e11, a.c11 * e22);
  const double s12 = a.c33 * e12;
  const double vi = a.vol[i];
  if (HG) {  // W = V (sigma K^-1 - k G)
    const double kh = -a.k_hg;
    a.w01[i] = make_double2(vi * fma(kh, g11, fma(s11, k11, s12 * k12)), vi * fma(kh, g12, fma(s11, k12, s12 * k22)));
    a.w23[i] = make_double2(vi * fma(kh, g21, fma(s12, k11, s22 * k12)), vi * fma(kh, g22, fma(s12, k12, s22 * k22)));
  } else {
    a.w01[i] = make_double2(vi * fma(s11, k11, s12 * k12), vi * fma(s11, k12, s12 * k22));
    a.w23[i] = make_double2(vi * fma(s12, k11, s22 * k12), vi * fma(s12, k12, s22 * k22));
  }
}

template <bool BREAK, bool HG>
__global__ void __launch_bounds__(kBlock) k_pass_a(Fp64Args a) {
  const int64_t i = a.i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  grid_dep_sync();  // nothing is read before the previous pass has completed
  if (i < a.n) pass_a_particle<BREAK, HG>(a, i);
}

// Pass B of particle i (force gather, kick; MODE 1 adds the next drift,
// MODE 2 is the drop-in kick with acce in/out).
template <int MODE, bool HG>
__device__ __forceinline__ void pass_b_particle(const Fp64Args& a, int64_t i) {
  int w;
  const int64_t s0 = slot0(a, i, &w);
  const double2 wa = a.w01[i], wb = a.w23[i], m = a.mt[i];
  double fx, fy;
  if (HG) {
    const double2 h = a.hg[i];
    fx = fma(wa.x, m.x, fma(wa.y, m.y, h.x));
    fy = fma(wb.x, m.x, fma(wb.y, m.y, h.y));
  } else {
    fx = fma(wa.x, m.x, wa.y * m.y);
    fy = fma(wb.x, m.x, wb.y * m.y);
  }
  struct Nb {
    double2 a, b;
  };
  walk_bonds<4>(
      w, i, GlobalIdx{a.nbr, s0}, [&](int64_t j) { return Nb{a.w01[j], a.w23[j]}; },
      [&](int k, int, const Nb& nb) {
        const double2 e = __ldcs(&a.bxi[s0 + (int64_t)k * kChunk]);
        fx = fma(nb.a.x, e.x, fx);
        fx = fma(nb.a.y, e.y, fx);
        fy = fma(nb.b.x, e.x, fy);
        fy = fma(nb.b.y, e.y, fy);
      });
  double2 v = a.v[i];
  double aox, aoy;
  if (MODE == 2) {
    const double2 ao = a.acc[i];
    aox = ao.x;
    aoy = ao.y;
  } else {
    const double2 fo = a.f[i];
    aox = fo.x * a.inv_rho;
    aoy = fo.y * a.inv_rho;
  }
  const double anx = fx * a.inv_rho, any = fy * a.inv_rho;
  v.x = v.x + (0.5 * (aox + anx)) * a.dt;
  v.y = v.y + (0.5 * (aoy + any)) * a.dt;
  a.f[i] = make_double2(fx, fy);
  if (MODE == 2) a.acc[i] = make_double2(anx, any);
  if (MODE == 1) {
    double2 u = a.u[i];
    drift_one(a, i, v, u, anx, any);
    a.u[i] = u;
    a.u32[i] = make_float2((float)u.x, (float)u.y);
  }
  a.v[i] = v;
  if (a.out_v) {  // pd_step_host's last pass, or the drop-in call: the results straight to host memory
    if (MODE == 2)
      a.out_a[i] = make_double2(anx, any);
    else
      a.out_u[i] = a.u[i];
    a.out_v[i] = v;
    a.out_f[i] = make_double2(fx, fy);
  }
}

template <int MODE, bool HG>
// 6 blocks per SM (<= 40 registers, no spills): 262 -> 258 us on the 1M-particle plate
__global__ void __launch_bounds__(kBlock, 6) k_pass_b(Fp64Args a) {
  const int64_t i = a.i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  grid_dep_sync();
  if (i < a.n) pass_b_particle<MODE, HG>(a, i);
}

// ---- batched plates: phase 0 drift, 1 pass A, 2 pass B + next drift, 3 pass B
__device__ __forceinline__ void batch_particle(const Fp64Args& p, int64_t i, int phase) {
  const bool hg = p.k_hg != 0.0;
  if (phase == 0) {
    drift_particle(p, i);
  } else if (phase == 1) {
    if (p.brk)
      hg ? pass_a_particle<true, true>(p, i) : pass_a_particle<true, false>(p, i);
    else
      hg ? pass_a_particle<false, true>(p, i) : pass_a_particle<false, false>(p, i);
  } else if (phase == 2) {
    hg ? pass_b_particle<1, true>(p, i) : pass_b_particle<1, false>(p, i);
  } else {
    hg ? pass_b_particle<0, true>(p, i) : pass_b_particle<0, false>(p, i);
  }
}

__device__ __forceinline__ void batch_phase(const Fp64Args* __restrict__ plates, const BatchTile* __restrict__ tiles,
                                            int ntiles, int phase) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile T = tiles[t];
    const Fp64Args& p = plates[T.plate];
    for (int k = threadIdx.x; k < T.count; k += blockDim.x) batch_particle(p, T.first + k, phase);
  }
}

__global__ void __launch_bounds__(256) k_batch_persistent(const Fp64Args* __restrict__ plates,
                                                          const BatchTile* __restrict__ tiles, int ntiles, int nsteps,
                                                          GridBarrier* bar, const BarrierLimits lim) {
  const unsigned nb = gridDim.x;
  batch_phase(plates, tiles, ntiles, 0);
  for (int s = 0; s < nsteps; ++s) {
    if (!grid_sync(bar, nb, lim)) return;
    batch_phase(plates, tiles, ntiles, 1);
    if (!grid_sync(bar, nb, lim)) return;
    batch_phase(plates, tiles, ntiles, s + 1 < nsteps ? 2 : 3);
  }
}

__global__ void __launch_bounds__(256) k_batch_phase(const Fp64Args* __restrict__ plates,
                                                     const BatchTile* __restrict__ tiles, int ntiles, int phase) {
  batch_phase(plates, tiles, ntiles, phase);
}

}  // namespace

int batch_occupancy_fp64(const BatchLaunch& cfg) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_persistent, cfg.block, 0) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_batch_fp64(const Fp64Args* d_plates, const BatchTile* d_tiles, int ntiles, int nsteps,
                              const BatchLaunch& cfg, GridBarrier* d_bar, int nsm, cudaStream_t s) {
  if (ntiles <= 0 || nsteps <= 0) return cudaSuccess;
  if (!cfg.persistent) {
    const unsigned g = (unsigned)ntiles;
    k_batch_phase<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, 0);
    for (int k = 0; k < nsteps; ++k) {
      k_batch_phase<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, 1);
      k_batch_phase<<<g, cfg.block, 0, s>>>(d_plates, d_tiles, ntiles, k + 1 < nsteps ? 2 : 3);
    }
    return cudaGetLastError();
  }
  int occ = batch_occupancy_fp64(cfg);
  int bps = cfg.blocks_per_sm < occ ? cfg.blocks_per_sm : occ;
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
  return cudaLaunchKernelEx(&lc, k_batch_persistent, d_plates, d_tiles, ntiles, nsteps, d_bar, cfg.limits);
}

namespace {
}  // namespace

namespace {
// reach[k] / low[k] = the largest / smallest id among slab k's particles
// (k*slab .. k*slab + slab - 1) and their neighbours
__global__ void k_slab_reach(int64_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                             int64_t slab, int32_t* reach, int32_t* low) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t m = (int32_t)i, l = (int32_t)i;
  for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
    m = col[k] > m ? col[k] : m;
    l = col[k] < l ? col[k] : l;
  }
  atomicMax(&reach[i / slab], m);
  atomicMin(&low[i / slab], l);
}
}  // namespace

void launch_slab_reach(int64_t n, const int64_t* row_ptr, const int32_t* col, int64_t slab, int32_t* reach,
                       int32_t* low, cudaStream_t s) {
  if (n > 0) k_slab_reach<<<(unsigned)blocks_for(n), kBlock, 0, s>>>(n, row_ptr, col, slab, reach, low);
}

void launch_init_geometry_fp64(const Fp64Args& a, cudaStream_t s) {
  if (a.n > 0) k_init_geometry<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a);
}

void launch_drift_fp64(const Fp64Args& a, cudaStream_t s) {
  if (a.n > a.i0) k_drift<<<(unsigned)blocks_for(a.n - a.i0), kBlock, 0, s>>>(a);
}

void launch_shadow_fp64(const Fp64Args& a, cudaStream_t s) {
  if (a.n > a.i0) k_shadow<<<(unsigned)blocks_for(a.n - a.i0), kBlock, 0, s>>>(a);
}

// pdl: launched with programmatic stream serialization (the blocks start
// while the previous kernel on the stream drains, and wait for it first).
static void launch_pass(void (*kernel)(Fp64Args), const Fp64Args& a, bool pdl, cudaStream_t s) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)blocks_for(a.n - a.i0));
  lc.blockDim = dim3(kBlock);
  lc.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  lc.attrs = at;
  lc.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&lc, kernel, a);
}

void launch_pass_a_fp64(const Fp64Args& a, bool breaking, cudaStream_t s, bool pdl) {
  if (a.n <= a.i0) return;
  const bool hg = a.k_hg != 0.0;
  if (breaking)
    launch_pass(hg ? k_pass_a<true, true> : k_pass_a<true, false>, a, pdl, s);
  else
    launch_pass(hg ? k_pass_a<false, true> : k_pass_a<false, false>, a, pdl, s);
}

void launch_pass_b_fp64(const Fp64Args& a, int mode, cudaStream_t s, bool pdl) {
  if (a.n <= a.i0) return;
  const bool hg = a.k_hg != 0.0;
  if (mode == 0)
    launch_pass(hg ? k_pass_b<0, true> : k_pass_b<0, false>, a, pdl, s);
  else if (mode == 1)
    launch_pass(hg ? k_pass_b<1, true> : k_pass_b<1, false>, a, pdl, s);
  else
    launch_pass(hg ? k_pass_b<2, true> : k_pass_b<2, false>, a, pdl, s);
}

}  // namespace pd
