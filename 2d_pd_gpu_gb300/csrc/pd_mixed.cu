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
#include <climits>
#include <vector>

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
// a - b as one FFMA2: b * -1 is exact, so the single rounding is that of a - b
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// (hi_j + lo_j) - (hi_i + lo_i) for two-float 2-vectors {hi.x, hi.y, lo.x, lo.y}
__device__ __forceinline__ float2 tf_diff2(float4 j, float2 nhi, float2 nlo) {
  return add2(add2(f2(j.x, j.y), nhi), add2(f2(j.z, j.w), nlo));
}

// A SELL slot's neighbour: its particle id, broken bonds included (-1: padding).
__device__ __forceinline__ int decode_nbr(int v) { return v >= 0 ? v : (v <= -2 ? -2 - v : -1); }

// FP64 -> two-float (hi + lo) for the scaled state.
__device__ __forceinline__ void split2(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// K^-1 (FP64 inversion + guard) and m^ from the FP64 reference positions of
// particle i at SELL position p, whose slots are s0 + 32 k, k < w.
__device__ void kinv_update_mixed(const MixedArgs& a, int64_t i, int64_t p, int64_t s0, int w) {
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
    a.geo[p] = make_float4(0.f, 0.f, 0.f, (float)vi);
    a.mh[p] = make_float2(0.f, 0.f);
    a.singular[p] = 1;
    atomicAdd(a.counters + CNT_SINGULAR, 1ull);
    return;
  }
  const double r = 1.0 / det;
  a.geo[p] = make_float4((float)(k22 * r), (float)(-k12 * r), (float)(k11 * r), (float)vi);
  a.mh[p] = make_float2((float)(mx / vi), (float)(my / vi));
  a.singular[p] = 0;
}

__global__ void __launch_bounds__(kBlock) k_init_geometry_mixed(MixedArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t p = sell_pos(a.pos_of, i);
  kinv_update_mixed(a, i, p, sell_slot0(a.chunk_base, p), a.chunk_w[p >> 5]);
}

// BC + drift of particle i in scaled per-step units; an = a^ of the new force.
// BC group of a particle, resolved (kind, prescribed v^).
struct BcOf {
  int kind;
  float4 gv;
};

__device__ __forceinline__ BcOf resolve_bc(const MixedArgs& a, int g) {
  BcOf b{PD_BC_NONE, make_float4(0.f, 0.f, 0.f, 0.f)};
  if (g) {
    b.kind = a.gkind[g - 1];
    if (b.kind == PD_BC_VELOCITY) b.gv = a.gvel[g - 1];
  }
  return b;
}

__device__ __forceinline__ void drift_bc(const BcOf& b, float4& v, float4& u, float anx, float any) {
  if (b.kind == PD_BC_VELOCITY) v = b.gv;
  // u += v + a/2   (v two-float, a/2 FP32)
  tf_add2(u.x, u.z, v.x, v.z);
  tf_add2(u.y, u.w, v.y, v.w);
  tf_add(u.x, u.z, 0.5f * anx);
  tf_add(u.y, u.w, 0.5f * any);
  if (b.kind == PD_BC_FIXED) u = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void drift_mixed(const MixedArgs& a, int64_t p, float4& v, float4& u, float anx,
                                            float any) {
  const int g = a.bc[p];
  const int kind = g ? a.gkind[g - 1] : PD_BC_NONE;
  if (kind == PD_BC_VELOCITY) v = a.gvel[g - 1];
  // u += v + a/2   (v two-float, a/2 FP32)
  tf_add2(u.x, u.z, v.x, v.z);
  tf_add2(u.y, u.w, v.y, v.w);
  tf_add(u.x, u.z, 0.5f * anx);
  tf_add(u.y, u.w, 0.5f * any);
  if (kind == PD_BC_FIXED) u = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Drift of SELL position p (a hole holds zeros and stays zero).
__device__ __forceinline__ void drift_particle_mixed(const MixedArgs& a, int64_t p) {
  float4 v = a.vs[p], u = a.us[p];
  const float2 f = a.fs[p];
  drift_mixed(a, p, v, u, a.tau2 * f.x, a.tau2 * f.y);
  a.vs[p] = v;
  a.us[p] = u;
}

__global__ void __launch_bounds__(kBlock) k_drift_mixed(MixedArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < a.npos) drift_particle_mixed(a, p);
}

// Neighbour data gathered by the two passes.
struct NbA {
  float4 u, x;
  float v;
};
struct NbB {
  float4 x, w;
};

// Per-particle inputs of pass A, loaded ahead of the bond walk.
struct PreA {
  float4 ui, xi, geo;
  int singular;
  int self_l;  // own halo position (staged blocks)
};

__device__ __forceinline__ PreA load_a(const MixedArgs& a, int64_t p) {
  return PreA{a.us[p], a.xs[p], a.geo[p], a.singular[p], a.self_loc ? (int)a.self_loc[p] : 0};
}

// Pass A of the particle at SELL position p: slots s0 + 32 k, k < w; idx(k)
// gives a slot's neighbour (a particle id, -1 for padding or broken; or, when
// the data is staged, a halo entry, the particle's own for padding or
// broken) and gather(j) its data.
// UV: every particle's V^ is 1 (uniform volumes; the host checks that
// (float)(V_i / Vs) == 1 for all i): the V^ gathers and products are left
// out, which changes no result -- x * 1 and fma(1, x, y) are exact.
template <bool BREAK, bool UV, typename Idx, typename Gather>
__device__ __forceinline__ void pass_a_core(const MixedArgs& a, int64_t p, const PreA& pre, int w, int64_t s0, Idx idx,
                                            Gather gather) {
  const float4 ui = pre.ui, xi = pre.xi;
  int newly = 0;
  const float2 nxh = f2(-xi.x, -xi.y), nxl = f2(-xi.z, -xi.w), nuh = f2(-ui.x, -ui.y), nul = f2(-ui.z, -ui.w);
  const float2 ns2 = f2(-a.s2, -a.s2);
  float2 D1 = f2(0.f, 0.f), D2 = f2(0.f, 0.f), A = f2(0.f, 0.f);  // (d11, d12), (d21, d22), (ax, ay)
  // 2 slots at a time: the halo walk reads shared memory, whose short latency needs less
  // memory-level parallelism than global gathers did, and at 64 registers 4 blocks fit an
  // SM (4-wide, 80 registers, 3 blocks: 61.4 us against 55.3 us on the 1M-particle plate)
  walk_bonds<2>(w, 0, idx, gather, [&](int k, int j, const NbA& nb) {
    const float2 e = tf_diff2(nb.x, nxh, nxl);  // xi^
    const float2 d = tf_diff2(nb.u, nuh, nul);  // du^
    if (BREAK) {  // d . (2 xi + d) - s2 xi . xi > 0, per component with one rounding
      const float2 r = fma2(ns2, mul2(e, e), mul2(d, fma2(f2(2.f, 2.f), e, d)));
      if (r.x + r.y > 0.f) {
        const int64_t s = s0 + (int64_t)k * kChunk;
        a.nbr[s] = -2 - a.nbr[s];  // the particle id of slot s (j may be a halo position)
        if (a.loc) a.loc[s] = (uint16_t)pre.self_l;  // the slot now adds exact zeros
        ++newly;
        return;
      }
    }
    if (UV) {
      D1 = fma2(f2(d.x, d.x), e, D1);
      D2 = fma2(f2(d.y, d.y), e, D2);
      A = add2(A, d);
    } else {
      const float2 vv = f2(nb.v, nb.v);
      const float2 t = mul2(vv, e);
      D1 = fma2(f2(d.x, d.x), t, D1);
      D2 = fma2(f2(d.y, d.y), t, D2);
      A = fma2(vv, d, A);
    }
  });
  const float d11 = D1.x, d12 = D1.y, d21 = D2.x, d22 = D2.y;
  a.hgs[p] = make_float2(2.f * a.k_hg * A.x, 2.f * a.k_hg * A.y);
  float4 g = pre.geo;
  int singular = pre.singular;
  if (BREAK && newly) {
    atomicAdd(a.counters + CNT_BROKEN, (unsigned long long)newly);
    const int64_t i = a.member[p];
    const int32_t b = a.broken[i] + newly;
    a.broken[i] = b;
    a.damage[i] = (double)b / (double)a.fam[i];
    kinv_update_mixed(a, i, p, s0, w);
    g = a.geo[p];
    singular = a.singular[p];
  }
  if (singular) {
    a.ws[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float k11 = g.x, k12 = g.y, k22 = g.z, vi = g.w;
  const float g11 = fmaf(d11, k11, d12 * k12), g12 = fmaf(d11, k12, d12 * k22);
  const float g21 = fmaf(d21, k11, d22 * k12), g22 = fmaf(d21, k12, d22 * k22);
  const float e11 = g11, e22 = g22, e12 = 0.5f * (g12 + g21);
  const float s11 = fmaf(a.c11, e11, a.c12 * e22);
  const float s22 = fmaf(a.c12, e11, a.c11 * e22);
  const float s12 = a.c33 * e12;
  const float kh = -a.k_hg;  // W^ = V^ (sigma^ K^-1 - k^ G), stored by columns {W11, W21, W12, W22}
  a.ws[p] = make_float4(vi * fmaf(kh, g11, fmaf(s11, k11, s12 * k12)), vi * fmaf(kh, g21, fmaf(s12, k11, s22 * k12)),
                        vi * fmaf(kh, g12, fmaf(s11, k12, s12 * k22)), vi * fmaf(kh, g22, fmaf(s12, k12, s22 * k22)));
}

struct GatherA {  // neighbour data of particle j (unstaged blocks)
  const MixedArgs* a;
  __device__ __forceinline__ NbA operator()(int64_t j) const {
    const int64_t q = a->pos_of[j];
    return NbA{a->us[q], a->xs[q], a->vh[q]};
  }
};

// Per-particle inputs of pass B, loaded ahead of the bond walk (the BC
// group is resolved separately: resolve_bc).
struct PreB {
  float4 wi, xi, v, u;
  float2 m, h, fo;
  int g;
};

template <bool DRIFT, bool EXPORT = false>
__device__ __forceinline__ PreB load_b(const MixedArgs& a, int64_t q) {
  PreB p;
  p.wi = a.ws[q];
  p.xi = a.xs[q];
  p.m = a.mh[q];
  p.h = a.hgs[q];
  p.fo = a.fs[q];
  p.v = a.vs[q];
  if (DRIFT || EXPORT) p.u = a.us[q];
  if (DRIFT) p.g = a.bc[q];
  return p;
}

// The FP64 state of SELL position p written by particle id to the export
// buffers (pd_step_host): the same conversions as pd_get_state (k_from_mixed).
__device__ __forceinline__ void export_state(const MixedArgs& a, int64_t p, const float4& u, const float4& v, float fx,
                                             float fy) {
  const int64_t i = a.member[p];
  if (i < 0) return;
  a.out_u[i] = make_double2(((double)u.x + (double)u.z) * a.ls, ((double)u.y + (double)u.w) * a.ls);
  a.out_v[i] = make_double2(((double)v.x + (double)v.z) * a.v_unscale, ((double)v.y + (double)v.w) * a.v_unscale);
  a.out_f[i] = make_double2((double)fx * a.f_unscale, (double)fy * a.f_unscale);
}

// Pass B of the particle at SELL position p (force gather, kick, optional
// next drift, or -- EXPORT -- the new state written to host buffers).
template <bool DRIFT, bool EXPORT = false, typename Idx, typename Gather>
__device__ __forceinline__ void pass_b_core(const MixedArgs& a, int64_t p, const PreB& pre, const BcOf& bc, int w,
                                            Idx idx, Gather gather) {
  const float4 wi = pre.wi, xi = pre.xi;
  const float2 m = pre.m, h = pre.h;
  // W columns c1 = (W11, W21), c2 = (W12, W22): W v = c1 v.x + c2 v.y
  // compensated (Kahan) sums S - C of both components at once: C carries
  // the rounding error of every addition into the next term
  float2 S = fma2(f2(wi.x, wi.y), f2(m.x, m.x), fma2(f2(wi.z, wi.w), f2(m.y, m.y), h)), C = f2(0.f, 0.f);
  const float2 nxh = f2(-xi.x, -xi.y), nxl = f2(-xi.z, -xi.w);
  walk_bonds<4>(w, 0, idx, gather, [&](int, int, const NbB& nb) {
    const float2 e = tf_diff2(nb.x, nxh, nxl);
    const float2 p = fma2(f2(nb.w.x, nb.w.y), f2(e.x, e.x), mul2(f2(nb.w.z, nb.w.w), f2(e.y, e.y)));
    const float2 y = sub2(p, C);
    const float2 t = add2(S, y);
    C = sub2(sub2(t, S), y);
    S = t;
  });
  const float fx = S.x - C.x, fy = S.y - C.y;
  const float2 fo = pre.fo;
  const float aox = a.tau2 * fo.x, aoy = a.tau2 * fo.y;
  const float anx = a.tau2 * fx, any = a.tau2 * fy;
  float4 v = pre.v;
  tf_add(v.x, v.z, 0.5f * (aox + anx));
  tf_add(v.y, v.w, 0.5f * (aoy + any));
  a.fs[p] = make_float2(fx, fy);
  if (DRIFT) {
    float4 u = pre.u;
    drift_bc(bc, v, u, anx, any);
    a.us[p] = u;
  }
  a.vs[p] = v;
  if (EXPORT) export_state(a, p, pre.u, v, fx, fy);
}

struct GatherB {  // neighbour data of particle j (unstaged blocks)
  const MixedArgs* a;
  __device__ __forceinline__ NbB operator()(int64_t j) const {
    const int64_t q = a->pos_of[j];
    return NbB{a->xs[q], a->ws[q]};
  }
};


// ---- single-plate and batched passes.  Visiting block b runs the chunks
// visit[8b .. 8b+8): SELL positions 256 b .. 256 b + 256, one 32 x 8 tile
// of the reference positions (8 row segments of 32).
// Blocks whose halo -- the distinct particles their bonds reach -- was
// staged at setup (halo_n[b] >= 0) gather the halo's data into shared memory
// (cp.async) and walk their bonds entirely out of shared memory (16-bit halo
// indices, TMA-staged per warp); other blocks stage their int32 indices and
// gather neighbour data from L1/L2.

struct HaloSmem {  // dynamic shared memory carve-up of a halo block
  float4* q0;      // pass A: u^, pass B: x^
  float4* q1;      // pass A: x^, pass B: W^
  uint16_t* li;    // kHaloBlock / 32 warps x wmax x 32 halo indices
  float* vh;       // pass A: V^
};

__device__ __forceinline__ HaloSmem halo_smem(const MixedArgs& a, unsigned char* sm) {
  HaloSmem h;
  const int hm = a.halo_max;
  h.q0 = reinterpret_cast<float4*>(sm);
  h.q1 = h.q0 + hm;
  h.li = reinterpret_cast<uint16_t*>(h.q1 + hm);
  h.vh = reinterpret_cast<float*>(h.li + (kHaloBlock / 32) * a.wmax * 32);
  return h;
}

// Halo loads: each thread fetches kHaloBatch halo ids, then issues
// asynchronous global -> shared copies (cp.async; no registers held while
// they are in flight) for all of them, so a block's whole halo is requested
// after one id round trip and lands after one gather round trip.
constexpr int kHaloBatch = 4;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// The calling warp's chunk (one 16 B visit record): false if the warp has
// none; *live = its lanes that hold a particle (the first ones).
__device__ __forceinline__ bool warp_chunk(const MixedArgs& a, int64_t blk, int64_t* chunk, int* w, int64_t* base,
                                           int* live) {
  const VisitRec r = a.visit[blk * (kHaloBlock / 32) + (threadIdx.x >> 5)];
  if (r.chunk < 0) return false;  // warp-uniform
  *chunk = r.chunk;
  *w = r.w;
  *live = r.live;
  *base = r.base;
  return true;
}

__device__ __forceinline__ void stage_timeout(const MixedArgs& a) {
  if ((threadIdx.x & 31) == 0) atomicOr(a.counters + CNT_ERROR, (unsigned long long)ERR_STAGE_TIMEOUT);
}

// Halo blocks: lane 0 of each warp issues the TMA copy of its 16-bit index
// chunk (waited on after the halo gather).
__device__ __forceinline__ void halo_begin(const MixedArgs& a, const HaloSmem& h, uint64_t* bars, bool has, int w,
                                           int64_t base) {
  const int warp = threadIdx.x >> 5;
  if (has && w > 0 && (threadIdx.x & 31) == 0)
    stage_issue(h.li + warp * a.wmax * 32, a.loc + base, (uint32_t)w * 64u, &bars[warp]);
}

// Invalidates a completed stage barrier so the next tile can arm it again.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Waits for the warp's staged chunk; on success the barrier is invalidated
// (reusable).  All 32 lanes call it.  False: the copy timed out (recorded).
__device__ __forceinline__ bool warp_stage_done(const MixedArgs& a, uint64_t* bar, int w) {
  if (w <= 0) return true;
  const bool ok = __all_sync(~0u, stage_wait(bar));
  if (!ok) {
    stage_timeout(a);
    return false;
  }
  if ((threadIdx.x & 31) == 0) mbar_inval(bar);
  __syncwarp();
  return true;
}

// The halo ids H[k0 + q kHaloBlock + t], q < kHaloBatch, that thread t
// fetches (-1 past hn), and the calls f(k, id) for them: every thread loads
// kHaloBatch ids before it issues their copies, so the id loads overlap.
__device__ __forceinline__ void halo_ids(const int32_t* H, int hn, int k0, int (&g)[kHaloBatch]) {
#pragma unroll
  for (int q = 0; q < kHaloBatch; ++q) {
    const int k = k0 + q * kHaloBlock + threadIdx.x;
    g[q] = k < hn ? H[k] : -1;
  }
}

template <typename F>
__device__ __forceinline__ void for_halo(const int32_t* H, int hn, int (&g)[kHaloBatch], F f) {
  for (int k0 = 0;;) {  // g holds the ids of the first batch
#pragma unroll
    for (int q = 0; q < kHaloBatch; ++q)
      if (g[q] >= 0) f(k0 + q * kHaloBlock + threadIdx.x, g[q]);
    k0 += kHaloBatch * kHaloBlock;
    if (k0 >= hn) break;
    halo_ids(H, hn, k0, g);
  }
}

// Pass A of visiting block blk (kHaloBlock / 32 chunks) of plate a.  Every
// thread of the kHaloBlock-thread block calls it; sm = the pass's dynamic
// shared memory.  False if a staged copy timed out.  PDL: the pass may start
// before the previous one has finished; until grid_dep_sync() it reads only
// the visit record and the first halo ids, which no step writes.
template <bool BREAK, bool PDL = false, bool UV = false>
__device__ __forceinline__ bool pass_a_block(const MixedArgs& a, int64_t blk, unsigned char* sm, uint64_t* bars) {
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  const bool has = warp_chunk(a, blk, &chunk, &w, &base, &nlive);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int hn = a.halo_n ? a.halo_n[blk] : -1;
  const int64_t p = chunk * 32 + lane;  // SELL position
  const bool live = has && lane < nlive;
  int g[kHaloBatch];
  if (PDL) {
    if (hn >= 0) halo_ids(a.halo + blk * a.halo_cap, hn, 0, g);
    grid_dep_sync();
  }
  PreA pre{};
  if (live) pre = load_a(a, p);  // in flight during the staging below
  if (hn < 0) {  // int32 indices staged per warp, neighbour data from L1/L2
    if (!has) return true;
    int32_t* mine = reinterpret_cast<int32_t*>(sm) + warp * a.wmax * 32;
    if (w > 0 && lane == 0) stage_issue(mine, a.nbr + base, (uint32_t)w * 128u, &bars[warp]);
    __syncwarp();
    if (!warp_stage_done(a, &bars[warp], w)) return false;
    if (live) pass_a_core<BREAK, UV>(a, p, pre, w, base + lane, SharedIdx{mine, lane}, GatherA{&a});
    return true;
  }
  const HaloSmem h = halo_smem(a, sm);
  halo_begin(a, h, bars, has, w, base);
  const int32_t* H = a.halo + blk * a.halo_cap;
  if (!PDL) halo_ids(H, hn, 0, g);
  for_halo(H, hn, g, [&](int k, int j) {
    cp_async16(&h.q0[k], &a.us[j]);
    cp_async16(&h.q1[k], &a.xs[j]);
    if (!UV) cp_async4(&h.vh[k], &a.vh[j]);
  });
  cp_async_wait_all();
  __syncthreads();
  if (!has) return true;
  if (!warp_stage_done(a, &bars[warp], w)) return false;
  if (!live) return true;
  const float4* q0 = h.q0;
  const float4* q1 = h.q1;
  const float* vh = h.vh;
  pass_a_core<BREAK, UV>(a, p, pre, w, base + lane, SharedHaloIdx{h.li + warp * a.wmax * 32, lane},
                     [=](int64_t l) { return NbA{q0[l], q1[l], vh[l]}; });
  return true;
}

// Pass B (+ the next drift when DRIFT, or the export when EXPORT) of
// visiting block blk of plate a.  PDL: as for pass A.
template <bool DRIFT, bool PDL = false, bool EXPORT = false>
__device__ __forceinline__ bool pass_b_block(const MixedArgs& a, int64_t blk, unsigned char* sm, uint64_t* bars) {
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  const bool has = warp_chunk(a, blk, &chunk, &w, &base, &nlive);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int hn = a.halo_n ? a.halo_n[blk] : -1;
  const int64_t p = chunk * 32 + lane;  // SELL position
  const bool live = has && lane < nlive;
  int g[kHaloBatch];
  if (PDL) {
    if (hn >= 0) halo_ids(a.halo + blk * a.halo_cap, hn, 0, g);
    grid_dep_sync();
  }
  PreB pre{};
  if (live) pre = load_b<DRIFT, EXPORT>(a, p);  // in flight during the staging below
  if (hn < 0) {
    if (!has) return true;
    int32_t* mine = reinterpret_cast<int32_t*>(sm) + warp * a.wmax * 32;
    if (w > 0 && lane == 0) stage_issue(mine, a.nbr + base, (uint32_t)w * 128u, &bars[warp]);
    __syncwarp();
    if (!warp_stage_done(a, &bars[warp], w)) return false;
    if (live)
      pass_b_core<DRIFT, EXPORT>(a, p, pre, DRIFT ? resolve_bc(a, pre.g) : BcOf{}, w, SharedIdx{mine, lane},
                                 GatherB{&a});
    return true;
  }
  const HaloSmem h = halo_smem(a, sm);
  halo_begin(a, h, bars, has, w, base);
  const int32_t* H = a.halo + blk * a.halo_cap;
  if (!PDL) halo_ids(H, hn, 0, g);
  for_halo(H, hn, g, [&](int k, int j) {
    cp_async16(&h.q0[k], &a.xs[j]);
    cp_async16(&h.q1[k], &a.ws[j]);
  });
  BcOf bc{};
  if (DRIFT && live) bc = resolve_bc(a, pre.g);
  cp_async_wait_all();
  __syncthreads();
  if (!has) return true;
  if (!warp_stage_done(a, &bars[warp], w)) return false;
  if (!live) return true;
  const float4* q0 = h.q0;
  const float4* q1 = h.q1;
  pass_b_core<DRIFT, EXPORT>(a, p, pre, bc, w, SharedHaloIdx{h.li + warp * a.wmax * 32, lane},
                             [=](int64_t l) { return NbB{q0[l], q1[l]}; });
  return true;
}

// Drift of visiting block blk of plate a (the first drift of a batched call).
__device__ __forceinline__ void drift_block(const MixedArgs& a, int64_t blk) {
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  if (!warp_chunk(a, blk, &chunk, &w, &base, &nlive)) return;
  const int lane = threadIdx.x & 31;
  if (lane < nlive) drift_particle_mixed(a, chunk * 32 + lane);
}

template <bool BREAK, bool UV>
__global__ void __launch_bounds__(kHaloBlock, 1024 / kHaloBlock) k_pass_a_mixed(MixedArgs a) {  // <= 64 registers
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bars[kHaloBlock / 32];
  pass_a_block<BREAK, true, UV>(a, a.blk0 + blockIdx.x, sm, bars);
}

template <bool DRIFT>
__global__ void __launch_bounds__(kHaloBlock, 1024 / kHaloBlock) k_pass_b_mixed(MixedArgs a) {  // <= 64 registers
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bars[kHaloBlock / 32];
  pass_b_block<DRIFT, true>(a, a.blk0 + blockIdx.x, sm, bars);
}

// The last pass B of pd_step_host: no drift, the new state written by
// particle id to the host buffers a.out_u / out_v / out_f.
__global__ void __launch_bounds__(kHaloBlock, 1024 / kHaloBlock) k_pass_b_mixed_export(MixedArgs a) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bars[kHaloBlock / 32];
  pass_b_block<false, true, true>(a, a.blk0 + blockIdx.x, sm, bars);
}

// pd_step_host's import: the positions of visiting blocks blk0 .. blk1 - 1
// take the FP64 state of their particles from u, v, f (by particle id; the
// same conversions as pd_set_state, k_to_mixed) and drift, as pd_set_state
// followed by a step's first drift (k_drift_mixed).  One thread per lane of
// each block's warps, as in the passes; holes keep their zeros.
__global__ void __launch_bounds__(kHaloBlock) k_import_drift_mixed(MixedArgs a, int64_t blk0,
                                                                 const double2* __restrict__ u,
                                                                 const double2* __restrict__ v,
                                                                 const double2* __restrict__ f) {
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  const int lane = threadIdx.x & 31;
  if (!warp_chunk(a, blk0 + blockIdx.x, &chunk, &w, &base, &nlive) || lane >= nlive) return;
  const int64_t p = chunk * 32 + lane;
  const int64_t i = a.member[p];
  if (i < 0) return;
  const double2 qu = u[i], qv = v[i], qf = f[i];
  float4 uu, vv;
  split2(qu.x * a.inv_ls, uu.x, uu.z);
  split2(qu.y * a.inv_ls, uu.y, uu.w);
  split2(qv.x * a.v_scale, vv.x, vv.z);
  split2(qv.y * a.v_scale, vv.y, vv.w);
  const float2 ff = make_float2((float)(qf.x * a.f_scale), (float)(qf.y * a.f_scale));
  a.fs[p] = ff;
  drift_mixed(a, p, vv, uu, a.tau2 * ff.x, a.tau2 * ff.y);
  a.vs[p] = vv;
  a.us[p] = uu;
}

// Per visiting block: the lowest and highest SELL position its bonds reach
// (its own positions included), the lowest and highest particle id it holds,
// and its first chunk (-1: none), for pd_step_host's slab plan.  A block's
// positions are those of its warps' chunks (visit records), not a fixed
// range: a tile's last block may hold fewer than kHaloBlock / 32 chunks.
// Staged blocks read their halo list (which holds their own positions); the
// others their slots.
__global__ void __launch_bounds__(kHaloBlock) k_block_reach_mixed(MixedArgs a, int64_t* lo, int64_t* hi,
                                                                 int64_t* idlo, int64_t* idhi, int64_t* cfirst) {
  __shared__ unsigned long long s_lo, s_hi, s_idlo, s_idhi, s_c;
  const int64_t blk = blockIdx.x;
  if (threadIdx.x == 0) {
    s_lo = ~0ull;
    s_hi = 0ull;
    s_idlo = ~0ull;
    s_idhi = 0ull;
    s_c = ~0ull;
  }
  __syncthreads();
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  const int lane = threadIdx.x & 31;
  const bool has = warp_chunk(a, blk, &chunk, &w, &base, &nlive);
  unsigned long long mn = ~0ull, mx = 0ull;
  if (has) {
    if (lane == 0) atomicMin(&s_c, (unsigned long long)chunk);
    if (lane < nlive) {
      const int64_t p = chunk * 32 + lane;
      const int64_t i = a.member[p];
      if (i >= 0) {
        atomicMin(&s_idlo, (unsigned long long)i);
        atomicMax(&s_idhi, (unsigned long long)i);
      }
      mn = (unsigned long long)p;
      mx = (unsigned long long)p;
    }
  }
  const int hn = a.halo_n ? a.halo_n[blk] : -1;
  if (hn >= 0) {
    for (int k = threadIdx.x; k < hn; k += blockDim.x) {
      const unsigned long long q = (unsigned long long)a.halo[blk * a.halo_cap + k];
      mn = q < mn ? q : mn;
      mx = q > mx ? q : mx;
    }
  } else if (has && lane < nlive) {
    for (int k = 0; k < w; ++k) {
      const int j = decode_nbr(a.nbr[base + lane + (int64_t)k * kChunk]);
      if (j < 0) continue;
      const unsigned long long q = (unsigned long long)a.pos_of[j];
      mn = q < mn ? q : mn;
      mx = q > mx ? q : mx;
    }
  }
  if (mn != ~0ull) atomicMin(&s_lo, mn);
  if (mn != ~0ull) atomicMax(&s_hi, mx);
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool none = s_lo == ~0ull;  // a block without positions reaches nothing
    lo[blk] = none ? -1 : (int64_t)s_lo;
    hi[blk] = none ? -1 : (int64_t)s_hi;
    idlo[blk] = s_idlo == ~0ull ? -1 : (int64_t)s_idlo;  // -1: no particle (holes only)
    idhi[blk] = s_idlo == ~0ull ? -1 : (int64_t)s_idhi;
    cfirst[blk] = s_c == ~0ull ? -1 : (int64_t)s_c;
  }
}

// Dynamic shared memory of the single-plate passes: the larger of the int32
// index staging (one wmax x 128 B chunk per warp) and the halo carve-up.
inline size_t pass_smem_bytes(const MixedArgs& a, bool pass_a) {
  const size_t idx32 = (size_t)(kHaloBlock / 32) * (size_t)a.wmax * 128u;
  if (!a.halo_n) return idx32;
  const size_t hm = (size_t)a.halo_max;
  const size_t halo = hm * 32u + (size_t)(kHaloBlock / 32) * (size_t)a.wmax * 64u + (pass_a ? hm * 4u : 0u);
  return halo > idx32 ? halo : idx32;
}

// ---- halo build (setup): per block, the distinct particles its chunks'
// bonds reach (own particles included) in ascending spatial key rk, and
// every slot's position in that list.  The ids are collected in a
// shared-memory hash set (open addressing, linear probing), their keys
// compacted, sorted (bitonic) and looked up by binary search; a block with
// more than kHaloCap distinct particles is not staged.

constexpr int kHaloHashBits = 12;
constexpr int kHaloHash = 1 << kHaloHashBits;
static_assert(kHaloHash >= 2 * kHaloCap && kHaloHash > kHaloCap + kHaloBlock, "halo hash table too small");
static_assert((kHaloCap & (kHaloCap - 1)) == 0, "kHaloCap is a power of two (bitonic sort)");

__global__ void __launch_bounds__(kHaloBlock) k_halo_build(MixedArgs a, const uint64_t* __restrict__ rk, int32_t* halo,
                                                       int32_t* halo_n, uint16_t* loc, uint16_t* loc0,
                                                       uint16_t* self_loc) {
  __shared__ int32_t tab[kHaloHash];
  __shared__ uint64_t list[kHaloCap];
  __shared__ int32_t s_cnt, s_put;
  const int tid = threadIdx.x, lane = tid & 31;
  int64_t chunk = 0, base = 0;
  int w = 0, nlive = 0;
  const bool has = warp_chunk(a, blockIdx.x, &chunk, &w, &base, &nlive);
  if (!has) w = 0;
  const int64_t s0 = base + lane;
  const int64_t p = chunk * 32 + lane;  // SELL position
  const int64_t i = has && lane < nlive ? (int64_t)a.member[p] : -1;
  for (int k = tid; k < kHaloHash; k += kHaloBlock) tab[k] = -1;
  if (tid == 0) {
    s_cnt = 0;
    s_put = 0;
  }
  __syncthreads();
  // A thread inserts only while the count is <= kHaloCap, so at most
  // kHaloCap + kHaloBlock ids enter the table: it never fills, and every
  // probe sequence ends at a free or matching entry within kHaloHash steps.
  auto insert = [&](int j) {
    if (*reinterpret_cast<volatile int32_t*>(&s_cnt) > kHaloCap) return;
    uint32_t h = ((uint32_t)j * 2654435761u) >> (32 - kHaloHashBits);
    for (int probe = 0; probe < kHaloHash; ++probe) {
      const int prev = atomicCAS(&tab[h], -1, j);
      if (prev == -1) {
        atomicAdd(&s_cnt, 1);
        return;
      }
      if (prev == j) return;
      h = (h + 1u) & (uint32_t)(kHaloHash - 1);
    }
  };
  const int wl = i >= 0 ? w : 0;  // lanes past n own padding slots only
  if (i >= 0) insert((int)i);
  for (int k = 0; k < wl; ++k) {
    const int j = decode_nbr(a.nbr[s0 + (int64_t)k * kChunk]);
    if (j >= 0) insert(j);
  }
  __syncthreads();
  const int tot = s_cnt;  // block-uniform
  if (tot <= kHaloCap) {
    int P = 1;
    while (P < tot) P <<= 1;
    for (int k = tid; k < kHaloHash; k += kHaloBlock) {
      const int v = tab[k];
      if (v >= 0) list[atomicAdd(&s_put, 1)] = rk[v];
    }
    for (int k = tot + tid; k < P; k += kHaloBlock) list[k] = ~0ull;
    __syncthreads();
    for (int kk = 2; kk <= P; kk <<= 1)
      for (int jj = kk >> 1; jj > 0; jj >>= 1) {
        for (int t = tid; t < P; t += kHaloBlock) {
          const int o = t ^ jj;
          if (o > t) {
            const uint64_t x = list[t], y = list[o];
            if ((x > y) == ((t & kk) == 0)) {
              list[t] = y;
              list[o] = x;
            }
          }
        }
        __syncthreads();
      }
    if (tid == 0) halo_n[blockIdx.x] = tot;
    int32_t* H = halo + (int64_t)blockIdx.x * kHaloCap;
    for (int k = tid; k < tot; k += kHaloBlock) H[k] = a.pos_of[list[k] & 0x7FFFFFFFull];  // rk's low bits: the id
    auto pos = [&](int j) {  // the entry of particle j (its key is in the list)
      const uint64_t r = rk[j];
      int lo = 0, hi = tot;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (list[mid] < r)
          lo = mid + 1;
        else
          hi = mid;
      }
      return (uint16_t)lo;
    };
    const uint16_t self = i >= 0 ? pos((int)i) : (uint16_t)0;
    if (i >= 0) self_loc[p] = self;
    for (int k = 0; k < w; ++k) {
      const int64_t s = s0 + (int64_t)k * kChunk;
      const int v = k < wl ? a.nbr[s] : -1;
      const int j = decode_nbr(v);
      const uint16_t l = j >= 0 ? pos(j) : self;  // padding: the particle itself (adds exact zeros)
      loc0[s] = l;
      loc[s] = v >= 0 ? l : self;
    }
    return;
  }
  // too many: the block reads neighbour data from HBM (loc unused)
  if (tid == 0) halo_n[blockIdx.x] = -1;
  if (i >= 0) self_loc[p] = 0;
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    loc0[s] = 0xFFFF;
    loc[s] = 0xFFFF;
  }
}

// visit record of every warp of every visiting block: {chunk, width, live
// lanes, first slot} (a chunk's holes are its last lanes)
__global__ void k_visit_build(int64_t nwarps, const int32_t* __restrict__ block_chunks,
                              const int32_t* __restrict__ chunk_w, const int64_t* __restrict__ chunk_base,
                              const int32_t* __restrict__ member, VisitRec* visit) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nwarps) return;
  const int32_t c = block_chunks[k];
  VisitRec r{-1, 0, 0, 0};
  if (c >= 0) {
    int live = 0;
    for (int l = 0; l < 32; ++l) live += member[(int64_t)c * 32 + l] >= 0;
    r = VisitRec{c, (int16_t)chunk_w[c], (int16_t)live, chunk_base[c]};
  }
  visit[k] = r;
}

// live 16-bit indices from the pristine ones and the int32 mask (after a
// reset or a restore): broken slots point at the particle itself
__global__ void k_halo_relink(MixedArgs a, const uint16_t* __restrict__ loc0, const uint16_t* __restrict__ self_loc,
                              uint16_t* loc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t p = sell_pos(a.pos_of, i);
  const int w = a.chunk_w[p >> 5];
  const int64_t s0 = sell_slot0(a.chunk_base, p);
  const uint16_t self = self_loc[p];
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    loc[s] = a.nbr[s] >= 0 ? loc0[s] : self;
  }
}

// ---- batched plates (see pd_batch.cuh): phase 0 drift, 1 pass A, 2 pass B +
// drift, 3 pass B.  A mixed tile is one visiting block of one plate (tile.first
// = the block index, tile.count = 256 particles at most), run by the same
// block code as the single-plate passes, so every plate's result is the one it
// gets alone.  False if a staged copy timed out.  The phase kernels of the
// passes (PHASE > 0) are launched with programmatic stream serialization: the
// tile records and plate arguments they read first are written before the
// step's launches.
template <int PHASE>  // PHASE < 0: the phase is the runtime argument
__device__ __forceinline__ bool batch_phase_mixed(const MixedArgs* __restrict__ plates,
                                                  const BatchTile* __restrict__ tiles, int ntiles, int phase_rt,
                                                  unsigned char* sm, uint64_t* bars) {
  const int phase = PHASE < 0 ? phase_rt : PHASE;
  bool ok = true;
  // the tile's plate arguments, copied to shared memory once per tile (the block code
  // reads them field by field; 2 % on the 256-plate batch)
  __shared__ __align__(16) MixedArgs sp;
  static_assert(sizeof(MixedArgs) % 8 == 0, "MixedArgs copies as int2");
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const BatchTile T = tiles[t];
    __syncthreads();  // the previous tile's shared memory is no longer read
    {
      const int2* src = reinterpret_cast<const int2*>(plates + T.plate);
      int2* dst = reinterpret_cast<int2*>(&sp);
      for (int q = threadIdx.x; q < (int)(sizeof(MixedArgs) / 8); q += blockDim.x) dst[q] = src[q];
    }
    __syncthreads();
    const MixedArgs& p = sp;
    if (phase == 0)
      drift_block(p, T.first);
    else if (phase == 1)  // the breaking pass also serves plates without breaking (their s2 is +inf)
      ok = pass_a_block<true, (PHASE > 0)>(p, T.first, sm, bars);
    else if (phase == 2)
      ok = pass_b_block<true, (PHASE > 0)>(p, T.first, sm, bars);
    else
      ok = pass_b_block<false, (PHASE > 0)>(p, T.first, sm, bars);
    ok = __syncthreads_and(ok);
  }
  return ok;
}

__global__ void __launch_bounds__(kHaloBlock) k_batch_persistent_mixed(const MixedArgs* __restrict__ plates,
                                                                   const BatchTile* __restrict__ tiles, int ntiles,
                                                                   int nsteps, GridBarrier* bar,
                                                                   const BarrierLimits lim) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bars[kHaloBlock / 32];
  const unsigned nb = gridDim.x;
  bool ok = batch_phase_mixed<-1>(plates, tiles, ntiles, 0, sm, bars);
  for (int s = 0; s < nsteps && ok; ++s) {
    if (!grid_sync(bar, nb, lim)) return;
    ok = batch_phase_mixed<-1>(plates, tiles, ntiles, 1, sm, bars);
    if (!ok) break;
    if (!grid_sync(bar, nb, lim)) return;
    ok = batch_phase_mixed<-1>(plates, tiles, ntiles, s + 1 < nsteps ? 2 : 3, sm, bars);
  }
  if (!ok && threadIdx.x == 0) atomicExch(&bar->err, 1);  // releases the other blocks' barrier waits
}

// registers as the single-plate passes: pass A 80 (3 blocks / SM), pass B 64 (4)
template <int PHASE>
__global__ void __launch_bounds__(kHaloBlock, 1024 / kHaloBlock)
    k_batch_phase_mixed(const MixedArgs* __restrict__ plates,
                                                              const BatchTile* __restrict__ tiles, int ntiles) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t bars[kHaloBlock / 32];
  batch_phase_mixed<PHASE>(plates, tiles, ntiles, PHASE, sm, bars);
}

// FP64 <-> scaled two-float conversions (set/get state; not per step): split2 above

// (per particle i; the scaled state of i sits at SELL position pos_of[i])
__global__ void k_to_mixed(MixedArgs a, const double2* u, const double2* v, const double2* f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t p = a.pos_of[i];
  float4 o;
  if (u) {
    const double2 q = u[i];
    split2(q.x * a.inv_ls, o.x, o.z);
    split2(q.y * a.inv_ls, o.y, o.w);
    a.us[p] = o;
  }
  if (v) {
    const double2 q = v[i];
    split2(q.x * a.v_scale, o.x, o.z);
    split2(q.y * a.v_scale, o.y, o.w);
    a.vs[p] = o;
  }
  if (f) {
    const double2 q = f[i];
    a.fs[p] = make_float2((float)(q.x * a.f_scale), (float)(q.y * a.f_scale));
  }
}

__global__ void k_from_mixed(MixedArgs a, double2* u, double2* v, double2* f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t p = a.pos_of[i];
  if (u) {
    const float4 q = a.us[p];
    u[i] = make_double2(((double)q.x + (double)q.z) * a.ls, ((double)q.y + (double)q.w) * a.ls);
  }
  if (v) {
    const float4 q = a.vs[p];
    v[i] = make_double2(((double)q.x + (double)q.z) * a.v_unscale, ((double)q.y + (double)q.w) * a.v_unscale);
  }
  if (f) {
    const float2 q = a.fs[p];
    f[i] = make_double2((double)q.x * a.f_unscale, (double)q.y * a.f_unscale);
  }
}

// x^, V^ by SELL position (holes: zeros)
__global__ void k_positions_mixed(MixedArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npos) return;
  const int64_t i = a.member[p];
  if (i < 0) {
    a.xs[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    a.vh[p] = 0.f;
    return;
  }
  const double2 q = a.x[i];
  float4 o;
  split2(q.x * a.inv_ls, o.x, o.z);
  split2(q.y * a.inv_ls, o.y, o.w);
  a.xs[p] = o;
  a.vh[p] = (float)(a.vol[i] * a.inv_vs);
}

// BC group by SELL position (holes: none)
__global__ void k_bc_by_position(int64_t npos, const int32_t* __restrict__ member, const uint8_t* __restrict__ bc,
                                 uint8_t* bcp) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npos) return;
  const int32_t i = member[p];
  bcp[p] = i >= 0 ? bc[i] : 0;
}

}  // namespace

size_t mixed_pass_smem(const MixedArgs& a, bool pass_a) { return pass_smem_bytes(a, pass_a); }

int batch_occupancy_mixed(const BatchLaunch& cfg, size_t smem) {
  (void)cfg;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_persistent_mixed, kHaloBlock, smem) != cudaSuccess)
    return 0;
  return nb;
}

// Mixed batches run kHaloBlock-thread blocks over visiting-block tiles; cfg.block is
// not used.
cudaError_t launch_batch_mixed(const MixedArgs* d_plates, const BatchTile* d_tiles, int ntiles, int nsteps,
                               const BatchLaunch& cfg, size_t smem_a, size_t smem_b, GridBarrier* d_bar, int nsm,
                               cudaStream_t s) {
  if (ntiles <= 0 || nsteps <= 0) return cudaSuccess;
  const size_t smem = smem_a > smem_b ? smem_a : smem_b;
  if (!cfg.persistent) {
    const unsigned g = (unsigned)ntiles;
    k_batch_phase_mixed<0><<<g, kHaloBlock, 0, s>>>(d_plates, d_tiles, ntiles);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(g);
    lc.blockDim = dim3(kHaloBlock);
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    for (int k = 0; k < nsteps; ++k) {
      lc.dynamicSmemBytes = smem_a;
      cudaLaunchKernelEx(&lc, k_batch_phase_mixed<1>, d_plates, d_tiles, ntiles);
      lc.dynamicSmemBytes = smem_b;
      cudaLaunchKernelEx(&lc, k + 1 < nsteps ? k_batch_phase_mixed<2> : k_batch_phase_mixed<3>, d_plates, d_tiles,
                         ntiles);
    }
    return cudaGetLastError();
  }
  const int occ = batch_occupancy_mixed(cfg, smem);
  const int bps = cfg.blocks_per_sm < occ ? cfg.blocks_per_sm : occ;
  if (bps < 1) return cudaErrorInvalidConfiguration;
  int grid = nsm * bps;
  if (grid > ntiles) grid = ntiles;
  cudaError_t e = cudaMemsetAsync(d_bar, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)grid);
  lc.blockDim = dim3((unsigned)kHaloBlock);
  lc.dynamicSmemBytes = smem;
  lc.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  lc.attrs = at;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k_batch_persistent_mixed, d_plates, d_tiles, ntiles, nsteps, d_bar, cfg.limits);
}

void launch_init_geometry_mixed(const MixedArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  // the passes may take up to kHaloCap x 36 B + one PD_MAX_FAMILY x 64 B index chunk per warp of shared memory
  const int mx = kHaloCap * 36 + (kHaloBlock / 32) * PD_MAX_FAMILY * 64;
  cudaFuncSetAttribute(k_pass_a_mixed<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_a_mixed<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_a_mixed<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_a_mixed<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_b_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_b_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_pass_b_mixed_export, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_batch_persistent_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_batch_phase_mixed<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_batch_phase_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_batch_phase_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  cudaFuncSetAttribute(k_batch_phase_mixed<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  k_positions_mixed<<<(unsigned)blocks_for(a.npos), kBlock, 0, s>>>(a);
  k_init_geometry_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a);
}

void launch_drift_mixed(const MixedArgs& a, cudaStream_t s) {
  if (a.n > 0) k_drift_mixed<<<(unsigned)blocks_for(a.npos), kBlock, 0, s>>>(a);
}

// The single-plate passes are launched with programmatic stream
// serialization: a pass's blocks may start (and fetch what no step writes)
// while the previous kernel on the stream drains.
static void (*pass_a_kernel(const MixedArgs& a, bool breaking))(MixedArgs) {
  if (a.uniform_v) return breaking ? k_pass_a_mixed<true, true> : k_pass_a_mixed<false, true>;
  return breaking ? k_pass_a_mixed<true, false> : k_pass_a_mixed<false, false>;
}

static void launch_pass_pdl(void (*kernel)(MixedArgs), const MixedArgs& a, size_t sm, cudaStream_t s,
                            bool pdl = true) {
  if (a.nblocks <= a.blk0) return;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)(a.nblocks - a.blk0));
  lc.blockDim = dim3(kHaloBlock);
  lc.dynamicSmemBytes = sm;
  lc.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  lc.attrs = at;
  lc.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&lc, kernel, a);
}

void launch_pass_a_mixed(const MixedArgs& a, bool breaking, cudaStream_t s) {
  if (a.n <= 0) return;
  launch_pass_pdl(pass_a_kernel(a, breaking), a, pass_smem_bytes(a, true), s);
}

void launch_pass_b_mixed(const MixedArgs& a, bool drift, cudaStream_t s) {
  if (a.n <= 0) return;
  launch_pass_pdl(drift ? k_pass_b_mixed<true> : k_pass_b_mixed<false>, a, pass_smem_bytes(a, false), s);
}

// pd_step_host's slabbed launches: plain stream order (each waits on events of
// other streams), visiting blocks a.blk0 .. a.nblocks - 1.
void launch_slab_pass_a_mixed(const MixedArgs& a, bool breaking, cudaStream_t s) {
  if (a.n <= 0) return;
  launch_pass_pdl(pass_a_kernel(a, breaking), a, pass_smem_bytes(a, true), s, false);
}

void launch_slab_pass_b_mixed(const MixedArgs& a, bool exporting, cudaStream_t s) {
  if (a.n <= 0) return;
  launch_pass_pdl(exporting ? k_pass_b_mixed_export : k_pass_b_mixed<true>, a, pass_smem_bytes(a, false), s,
                  false);
}

void launch_import_drift_mixed(const MixedArgs& a, int64_t blk0, int64_t blk1, const double2* u, const double2* v,
                               const double2* f, cudaStream_t s) {
  if (blk1 > blk0) k_import_drift_mixed<<<(unsigned)(blk1 - blk0), kHaloBlock, 0, s>>>(a, blk0, u, v, f);
}

void launch_block_reach_mixed(const MixedArgs& a, int64_t* lo, int64_t* hi, int64_t* idlo, int64_t* idhi,
                              int64_t* cfirst, cudaStream_t s) {
  if (a.nblocks > 0) k_block_reach_mixed<<<(unsigned)a.nblocks, kHaloBlock, 0, s>>>(a, lo, hi, idlo, idhi, cfirst);
}

void launch_to_mixed(const MixedArgs& a, const double2* u, const double2* v, const double2* f, cudaStream_t s) {
  if (a.n > 0) k_to_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, u, v, f);
}

void launch_from_mixed(const MixedArgs& a, double2* u, double2* v, double2* f, cudaStream_t s) {
  if (a.n > 0) k_from_mixed<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, u, v, f);
}

int build_halo_mixed(const MixedArgs& a0, int64_t nslots, int64_t nblocks, const int32_t* block_chunks,
                     const uint64_t* rk, cudaStream_t s, HaloLayout* h, std::string* msg) {
  const int64_t nb = nblocks;
  h->nblocks = nb;
  h->staged = 0;
  h->halo_max = 0;
  if (a0.n <= 0 || nb <= 0) return PD_OK;
  const size_t ns = (size_t)(nslots > 0 ? nslots : 1);
  const int64_t nw = nb * (kHaloBlock / 32);
  MixedArgs a = a0;
  if (cudaMalloc(&h->visit, (size_t)nw * sizeof(VisitRec)) != cudaSuccess ||
      cudaMalloc(&h->loc, ns * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&h->loc0, ns * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&h->self_loc, (size_t)a.npos * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&h->halo, (size_t)nb * kHaloCap * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&h->halo_n, (size_t)nb * sizeof(int32_t)) != cudaSuccess) {
    *msg = "halo staging: out of device memory";
    return PD_ERR_CUDA;
  }
  k_visit_build<<<(unsigned)blocks_for(nw), kBlock, 0, s>>>(nw, block_chunks, a.chunk_w, a.chunk_base, a.member,
                                                            h->visit);
  a.visit = h->visit;
  a.nblocks = nb;
  k_halo_build<<<(unsigned)nb, kHaloBlock, 0, s>>>(a, rk, h->halo, h->halo_n, h->loc, h->loc0, h->self_loc);
  std::vector<int32_t> cnt((size_t)nb);
  cudaError_t e = cudaMemcpyAsync(cnt.data(), h->halo_n, (size_t)nb * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("halo staging: ") + cudaGetErrorString(e);
    return PD_ERR_CUDA;
  }
  int32_t mx = 0;
  for (int32_t v : cnt)
    if (v >= 0) {
      ++h->staged;
      mx = v > mx ? v : mx;
    }
  h->halo_max = (mx + 7) & ~7;
  return PD_OK;
}

void launch_bc_by_position(int64_t npos, const int32_t* member, const uint8_t* bc, uint8_t* bcp, cudaStream_t s) {
  if (npos > 0) k_bc_by_position<<<(unsigned)blocks_for(npos), kBlock, 0, s>>>(npos, member, bc, bcp);
}

void launch_halo_relink(const MixedArgs& a, const HaloLayout& h, cudaStream_t s) {
  if (a.n > 0 && h.loc) k_halo_relink<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, h.loc0, h.self_loc, h.loc);
}

}  // namespace pd
