// C ABI of the GB300 NOSB step (include/pd_gb300.h): context, device-resident
// state, family/bond set-up, step launches captured in CUDA graphs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "pd_internal.h"

using pd::Fp64Args;

struct pd_ctx {
  pd_params p{};
  bool c_override = false;
  double c11 = 0.0, c12 = 0.0, c33 = 0.0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t n = 0;
  bool has_particles = false, has_families = false;
  std::vector<double> h_x;    // host copy of the reference positions (cell-list bbox, scales)
  std::vector<double> h_vol;  // host copy of the volumes
  double cutoff = 0.0;        // family cutoff (0 if families came from the host)
  // mixed-form scales: lengths / Ls, volumes / Vs, stresses / Es
  double ls = 1.0, vs_scale = 1.0;
  bool uniform_v = false;  // mixed form: every (float)(V_i / Vs) is exactly 1

  // per particle
  double2 *x = nullptr, *u = nullptr, *v = nullptr, *f = nullptr, *acc = nullptr;
  double *vol = nullptr, *kinv22 = nullptr, *damage = nullptr;
  double2 *w01 = nullptr, *w23 = nullptr, *kinv01 = nullptr, *mt = nullptr, *hg = nullptr;
  uint8_t *bc = nullptr, *singular = nullptr;
  int32_t *broken = nullptr, *fam = nullptr;
  // mixed form (PD_MIXED): by SELL position (sell.npos entries), with the families
  float4 *xs = nullptr, *us = nullptr, *vsm = nullptr, *ws = nullptr, *geo = nullptr;
  float2 *fs = nullptr, *mh = nullptr, *hgs = nullptr;
  float* vh = nullptr;
  uint8_t *bcp = nullptr, *sgp = nullptr;  // BC group, singular flag
  // BC groups
  int32_t* gkind = nullptr;
  double2* gval = nullptr;
  float4* gvel = nullptr;  // mixed: scaled two-float prescribed velocities
  std::vector<double> h_gval = std::vector<double>(2 * PD_MAX_BC_GROUPS, 0.0);
  // families
  int64_t nnz = 0;
  int64_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  pd::SellLayout sell;
  pd::HaloLayout halo;  // mixed form
  double2 *bxi = nullptr, *bgeo = nullptr;
  double* blim = nullptr;
  float* br2 = nullptr;
  float2* u32 = nullptr;
  // bond-associated mode
  double2* tb = nullptr;
  int64_t* rslot = nullptr;
  double2* ba_lr = nullptr;  // bond-associated mode, per slot: |xi|, 1/|xi|
  double2* ba_ex = nullptr;  // exp(+-n1 |xi| / l)
  double2* ba_kq0 = nullptr;  // K_b^-1 with its det-guard flag
  double2* ba_kq1 = nullptr;
  double* ba_wtri = nullptr;  // and, per particle, its weight matrix's lower triangle
  int32_t max_family = 0;
  // pd_step_host's copy / compute pipeline (streams and events, see plan_slabs)
  cudaStream_t io[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaStream_t> ps;  // pd_step_host: one stream per slab's pass A, then one per slab's pass B
  std::vector<cudaEvent_t> slab_ev;
  std::vector<int64_t> slab_bnd;    // slab k = particles slab_bnd[k] .. slab_bnd[k+1]; empty: not planned
  std::vector<int32_t> slab_need;   // slab k's pass A needs slabs 0 .. slab_need[k] imported
  std::vector<int32_t> slab_low;    // the first slab holding a neighbour of slab k (its pass B waits on
                                    // pass A of slabs slab_low[k] .. slab_need[k])
  // the mixed form's: slab k = visiting blocks mslab_blk[k] .. mslab_blk[k+1], whose bonds
  // reach slabs mslab_lo[k] .. mslab_hi[k]; id slab k = particles mslab_id[k] ..
  // mslab_id[k+1], which slab k's import needs at the latest
  std::vector<int64_t> mslab_blk, mslab_id;
  std::vector<int32_t> mslab_lo, mslab_hi;
  // Mazars damage history (pd_mazars_*)
  double *mz_thr = nullptr, *mz_bd = nullptr, *mz_status = nullptr;
  pd_mazars_params mz{};
  // counters (device) + host mirror of steps
  unsigned long long* counters = nullptr;
  int64_t steps = 0;
  // graphs per step count
  std::map<int32_t, cudaGraphExec_t> graphs;
  // drop-in staging (pinned)
  std::vector<void*> scratch;
  // batch membership (pd_batch_add)
  pd_batch* batch = nullptr;
};

struct pd_batch {
  int32_t device = 0, precision = PD_FP64;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;  // around the last pd_batch_step's GPU work
  cudaEvent_t join = nullptr;               // persistent == 2: a member's step graph ends
  std::string err;
  std::vector<pd_ctx*> members;
  pd::BatchLaunch cfg;
  int tile = 1024;
  int nsm = 0;
  bool dirty = true;
  void* d_plates = nullptr;
  size_t plates_bytes = 0;
  pd::BatchTile* d_tiles = nullptr;
  size_t tiles_cap = 0;
  int ntiles = 0;
  pd::GridBarrier* d_bar = nullptr;
  int64_t particles = 0, bonds = 0;
  std::map<int32_t, cudaGraphExec_t> graphs;
  bool direct = false;  // persistent kernel launched directly (its capture was refused)
  size_t smem_a = 0, smem_b = 0;  // mixed: dynamic shared memory of the batched passes A and B
};

namespace {

thread_local std::string g_create_err;

int fail(pd_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(pd_ctx* c, cudaError_t e, const char* where) {
  return fail(c, PD_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define PD_CK(ctx, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

void clear_batch_graphs(pd_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

// Captured kernel arguments are stale: drop the graphs (and the batch tables).
void clear_graphs(pd_ctx* c) {
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
  if (c->batch) {
    c->batch->dirty = true;
    clear_batch_graphs(c->batch);
  }
}

// A copy ordered on stream s (the contexts' and batches' streams are
// non-blocking, so a plain cudaMemcpy is not ordered with their kernels, and
// one from pageable memory may return before its data has landed), waited for.
cudaError_t copy_sync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

void free_families(pd_ctx* c) {
  dfree(c->row_ptr);
  dfree(c->col);
  dfree(c->sell.chunk_base);
  dfree(c->sell.chunk_w);
  dfree(c->sell.nbr);
  dfree(c->sell.member);
  dfree(c->sell.rk);
  dfree(c->sell.pos_of);
  dfree(c->xs); dfree(c->us); dfree(c->vsm); dfree(c->ws); dfree(c->geo);
  dfree(c->fs); dfree(c->mh); dfree(c->hgs); dfree(c->vh); dfree(c->bcp); dfree(c->sgp);
  dfree(c->mz_thr);
  dfree(c->mz_bd);
  dfree(c->mz_status);
  dfree(c->halo.visit);
  dfree(c->halo.loc);
  dfree(c->halo.loc0);
  dfree(c->halo.self_loc);
  dfree(c->halo.halo);
  dfree(c->halo.halo_n);
  c->halo = pd::HaloLayout{};
  dfree(c->bxi);
  dfree(c->bgeo);
  dfree(c->blim);
  dfree(c->br2);
  dfree(c->tb);
  dfree(c->rslot);
  dfree(c->ba_lr);
  dfree(c->ba_ex);
  dfree(c->ba_kq0);
  dfree(c->ba_kq1);
  dfree(c->ba_wtri);
  c->sell = pd::SellLayout{};
  c->slab_bnd.clear();
  c->slab_need.clear();
  c->slab_low.clear();
  c->mslab_blk.clear();
  c->mslab_id.clear();
  c->mslab_lo.clear();
  c->mslab_hi.clear();
  c->nnz = 0;
  c->has_families = false;
  clear_graphs(c);
}

void free_particles(pd_ctx* c) {
  free_families(c);
  dfree(c->x); dfree(c->u); dfree(c->v); dfree(c->f); dfree(c->acc);
  dfree(c->vol); dfree(c->kinv22); dfree(c->damage);
  dfree(c->w01); dfree(c->w23); dfree(c->kinv01); dfree(c->mt); dfree(c->hg);
  dfree(c->bc); dfree(c->singular); dfree(c->broken); dfree(c->fam);
  dfree(c->u32);
  c->n = 0;
  c->has_particles = false;
}


int check_params(pd_ctx* c, const pd_params* p) {
  if (!p) return fail(c, PD_ERR_ARG, "params is NULL");
  if (p->precision != PD_FP64 && p->precision != PD_MIXED) return fail(c, PD_ERR_ARG, "unknown precision");
  if (!(p->rho > 0.0) || !(p->dt > 0.0) || !std::isfinite(p->E) || !(p->nu > -1.0 && p->nu < 1.0) ||
      !(p->det_guard >= 0.0) || !(p->k_hg >= 0.0) || !std::isfinite(p->k_hg) || !(p->damage_fail >= 0.0))
    return fail(c, PD_ERR_ARG, "invalid material / time-step parameters");
  if (p->singular_policy != PD_SINGULAR_ZERO && p->singular_policy != PD_SINGULAR_ERROR)
    return fail(c, PD_ERR_ARG, "unknown singular_policy");
  if (p->n1 != 0.0 || p->n2 != 0.0) {
    if (p->precision != PD_FP64) return fail(c, PD_ERR_ARG, "bond-associated weights need PD_FP64");
    if (p->s_c > 0.0 || p->k_hg != 0.0)
      return fail(c, PD_ERR_ARG, "bond-associated weights: no bond breaking (s_c <= 0) and k_hg = 0");
    if (!(p->weight_len > 0.0) || !std::isfinite(p->n1) || !std::isfinite(p->n2))
      return fail(c, PD_ERR_ARG, "bond-associated weights need weight_len > 0 and finite n1, n2");
  }
  return PD_OK;
}

bool bond_assoc(const pd_ctx* c) { return c->p.n1 != 0.0 || c->p.n2 != 0.0; }

// Device-side address of a page-locked host buffer (nullptr if it is not one).
void* mapped_host(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return at.devicePointer;
}

void stiffness(const pd_ctx* c, double* c11, double* c12, double* c33);

Fp64Args fp64_args(pd_ctx* c) {
  Fp64Args a{};
  a.n = c->n;
  a.x = c->x; a.vol = c->vol; a.u = c->u; a.v = c->v; a.f = c->f; a.acc = c->acc;
  a.w01 = c->w01; a.w23 = c->w23; a.kinv01 = c->kinv01; a.kinv22 = c->kinv22; a.mt = c->mt; a.hg = c->hg;
  a.bc = c->bc; a.gkind = c->gkind; a.gval = c->gval;
  a.broken = c->broken; a.damage = c->damage; a.singular = c->singular; a.fam = c->fam;
  a.chunk_base = c->sell.chunk_base; a.chunk_w = c->sell.chunk_w; a.nbr = c->sell.nbr;
  a.bxi = c->bxi; a.bgeo = c->bgeo; a.blim = c->blim; a.br2 = c->br2; a.u32 = c->u32;
  stiffness(c, &a.c11, &a.c12, &a.c33);  // getStiffnessTensor, src/main_seq.cpp:185-187
  a.dt = c->p.dt;
  a.dt2 = c->p.dt * c->p.dt;
  a.inv_rho = 1.0 / c->p.rho;
  a.det_guard = c->p.det_guard;
  a.k_hg = c->p.k_hg;
  a.damage_fail = c->p.damage_fail;
  a.counters = c->counters;
  a.brk = c->p.s_c > 0.0;
  return a;
}

pd::BondAssoc ba_args(pd_ctx* c) {
  pd::BondAssoc b{};
  b.n1 = c->p.n1;
  b.n2 = c->p.n2;
  b.inv_wlen = c->p.weight_len > 0.0 ? 1.0 / c->p.weight_len : 0.0;
  b.tb = c->tb;
  b.rslot = c->rslot;
  b.lr = c->ba_lr;
  b.ex = c->ba_ex;
  b.kq0 = c->ba_kq0;
  b.kq1 = c->ba_kq1;
  b.wtri = c->ba_wtri;
  return b;
}

// Buffers and reverse-slot index of the bond-associated mode, and its
// per-bond constants for the current weights (recomputed on every call: the
// parameters may have changed).
int ensure_ba(pd_ctx* c) {
  if (!bond_assoc(c) || !c->has_families) return PD_OK;
  if (c->max_family > 64) return fail(c, PD_ERR_CAPACITY, "bond-associated mode: families are limited to 64 bonds");
  const size_t ns = (size_t)(c->sell.nslots > 0 ? c->sell.nslots : 1);
  if (c->tb) {
    pd::launch_ba_bonds(fp64_args(c), ba_args(c), c->sell.nslots, c->stream);
    PD_CK(c, cudaGetLastError());
    return PD_OK;
  }
  // (each allocated once: a call that failed part-way is retried without leaking)
  if (!c->ba_lr) PD_CK(c, cudaMalloc(&c->ba_lr, ns * sizeof(double2)));
  if (!c->ba_ex) PD_CK(c, cudaMalloc(&c->ba_ex, ns * sizeof(double2)));
  if (!c->ba_kq0) PD_CK(c, cudaMalloc(&c->ba_kq0, ns * sizeof(double2)));
  if (!c->ba_kq1) PD_CK(c, cudaMalloc(&c->ba_kq1, ns * sizeof(double2)));
  if (!c->ba_wtri)
    PD_CK(c, cudaMalloc(&c->ba_wtri, (size_t)(c->n > 0 ? c->n : 1) * (size_t)pd::kBaTri * sizeof(double)));
  pd::launch_ba_bonds(fp64_args(c), ba_args(c), c->sell.nslots, c->stream);
  if (!c->rslot) PD_CK(c, cudaMalloc(&c->rslot, ns * sizeof(int64_t)));
  PD_CK(c, cudaMalloc(&c->tb, ns * sizeof(double2)));
  PD_CK(c, cudaMemsetAsync(c->tb, 0, ns * sizeof(double2), c->stream));
  PD_CK(c, cudaMemsetAsync(c->counters + pd::CNT_ERROR, 0, sizeof(unsigned long long), c->stream));
  pd::launch_ba_reverse(fp64_args(c), ba_args(c), c->stream);
  PD_CK(c, cudaGetLastError());
  unsigned long long err = 0;
  PD_CK(c, cudaMemcpyAsync(&err, c->counters + pd::CNT_ERROR, sizeof(err), cudaMemcpyDeviceToHost, c->stream));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  if (err & pd::ERR_ASYMMETRIC) return fail(c, PD_ERR_ARG, "bond-associated mode needs symmetric families");
  return PD_OK;
}

bool mixed(const pd_ctx* c) { return c->p.precision == PD_MIXED; }

void stiffness(const pd_ctx* c, double* c11, double* c12, double* c33) {
  const double E = c->p.E, nu = c->p.nu;
  const double pre = E / (1.0 - nu * nu);
  *c11 = c->c_override ? c->c11 : pre;
  *c12 = c->c_override ? c->c12 : nu * pre;
  *c33 = c->c_override ? c->c33 : (1.0 - nu) * pre;
}

pd::MixedArgs mixed_args(pd_ctx* c) {
  pd::MixedArgs a{};
  a.n = c->n;
  a.npos = c->sell.npos;
  a.x = c->x; a.vol = c->vol;
  a.xs = c->xs; a.vh = c->vh; a.us = c->us; a.vs = c->vsm; a.fs = c->fs; a.ws = c->ws; a.geo = c->geo; a.mh = c->mh;
  a.hgs = c->hgs;
  a.bc = c->bcp; a.gkind = c->gkind; a.gvel = c->gvel;
  a.broken = c->broken; a.damage = c->damage; a.singular = c->sgp; a.fam = c->fam;
  a.chunk_base = c->sell.chunk_base; a.chunk_w = c->sell.chunk_w; a.nbr = c->sell.nbr;
  a.member = c->sell.member; a.pos_of = c->sell.pos_of;
  a.visit = c->halo.visit;
  a.nblocks = c->halo.nblocks;
  a.loc = c->halo.loc;
  a.self_loc = c->halo.self_loc;
  a.halo = c->halo.halo;
  a.halo_n = c->halo.halo_n;
  a.halo_cap = pd::kHaloCap;
  a.halo_max = c->halo.halo_max;
  double c11, c12, c33;
  stiffness(c, &c11, &c12, &c33);
  const double es = c11 != 0.0 ? c11 : 1.0;
  a.c11 = (float)(c11 / es);
  a.c12 = (float)(c12 / es);
  a.c33 = (float)(c33 / es);
  a.s2 = c->p.s_c > 0.0 ? (float)(c->p.s_c * (2.0 + c->p.s_c)) : INFINITY;
  a.tau2 = (float)(es * c->p.dt * c->p.dt / (c->p.rho * c->ls * c->ls));
  a.k_hg = (float)(c->p.k_hg * c->vs_scale * c->ls * c->ls / es);
  a.inv_ls = 1.0 / c->ls;
  a.inv_vs = 1.0 / c->vs_scale;
  a.uniform_v = c->uniform_v ? 1 : 0;
  a.v_scale = c->p.dt / c->ls;
  a.f_scale = c->ls / es;
  // the way back by products: an FP64 division costs ~10 operations of the FP64 pipe, ~1/58 of
  // the FP32 rate on this GPU (within an ulp of dividing by the scale)
  a.ls = c->ls;
  a.v_unscale = c->ls / c->p.dt;
  a.f_unscale = es / c->ls;
  a.det_guard = c->p.det_guard;
  a.damage_fail = c->p.damage_fail;
  a.counters = c->counters;
  a.brk = c->p.s_c > 0.0;
  a.wmax = c->max_family;
  return a;
}

// Scaled two-float prescribed velocities for the mixed form.
int upload_gvel(pd_ctx* c) {
  if (!mixed(c) || !c->gvel) return PD_OK;
  std::vector<float> g(4 * PD_MAX_BC_GROUPS, 0.f);
  const double sc = c->p.dt / c->ls;
  for (int k = 0; k < PD_MAX_BC_GROUPS; ++k)
    for (int m = 0; m < 2; ++m) {
      const double v = c->h_gval[2 * k + m] * sc;
      const float hi = (float)v;
      g[4 * k + m] = hi;
      g[4 * k + 2 + m] = (float)(v - (double)hi);
    }
  PD_CK(c, copy_sync(c->gvel, g.data(), g.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  return PD_OK;
}

__global__ void k_fam_from_rowptr(int64_t n, const int64_t* rp, int32_t* fam) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) fam[i] = (int32_t)(rp[i + 1] - rp[i]);
}

// After row_ptr/col exist: SELL layout, bond geometry, per-particle geometry, reset.
int finish_families(pd_ctx* c) {
  cudaStream_t s = c->stream;
  std::string msg;
  PD_CK(c, cudaMemsetAsync(c->counters, 0, pd::CNT_N * sizeof(unsigned long long), s));
  struct Blocks {  // visiting blocks of the mixed form, freed on every return
    int32_t* p = nullptr;
    ~Blocks() { dfree(p); }
  } blocks;
  int64_t nblocks = 0;
  if (mixed(c)) {  // SELL chunks and visiting blocks are spatial tiles; the state follows them
    const int ro = pd::build_spatial_order(c->n, c->x, c->h_x.data(), s, &c->sell, &blocks.p, &nblocks, &msg);
    if (ro != PD_OK) return fail(c, ro, msg);
    const size_t np = (size_t)(c->sell.npos > 0 ? c->sell.npos : 1);
    PD_CK(c, cudaMalloc(&c->xs, np * sizeof(float4)));
    PD_CK(c, cudaMalloc(&c->us, np * sizeof(float4)));
    PD_CK(c, cudaMalloc(&c->vsm, np * sizeof(float4)));
    PD_CK(c, cudaMalloc(&c->ws, np * sizeof(float4)));
    PD_CK(c, cudaMalloc(&c->geo, np * sizeof(float4)));
    PD_CK(c, cudaMalloc(&c->fs, np * sizeof(float2)));
    PD_CK(c, cudaMalloc(&c->mh, np * sizeof(float2)));
    PD_CK(c, cudaMalloc(&c->hgs, np * sizeof(float2)));
    PD_CK(c, cudaMalloc(&c->vh, np * sizeof(float)));
    PD_CK(c, cudaMalloc(&c->bcp, np));
    PD_CK(c, cudaMalloc(&c->sgp, np));
    PD_CK(c, cudaMemsetAsync(c->geo, 0, np * sizeof(float4), s));  // holes stay zero
    PD_CK(c, cudaMemsetAsync(c->mh, 0, np * sizeof(float2), s));
    PD_CK(c, cudaMemsetAsync(c->sgp, 0, np, s));
    pd::launch_bc_by_position(c->sell.npos, c->sell.member, c->bc, c->bcp, s);
  }
  int rc = pd::build_sell(c->n, c->row_ptr, c->col, s, &c->sell, c->counters, &msg);
  if (rc != PD_OK) return fail(c, rc, msg);
  unsigned long long h[pd::CNT_N];
  PD_CK(c, copy_sync(h, c->counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if (h[pd::CNT_ERROR])
    return fail(c, PD_ERR_ARG, "invalid family: neighbour id out of range or a self bond (error word " +
                                   std::to_string(h[pd::CNT_ERROR]) + ")");
  if (!mixed(c)) {
    const size_t ns = (size_t)(c->sell.nslots > 0 ? c->sell.nslots : 1);
    PD_CK(c, cudaMalloc(&c->bxi, ns * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->bgeo, ns * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->blim, ns * sizeof(double)));
    PD_CK(c, cudaMalloc(&c->br2, ns * sizeof(float)));
    pd::launch_bond_geometry_fp64(c->n, c->x, c->vol, c->sell, c->row_ptr, c->p.s_c, c->bxi, c->bgeo, c->blim,
                                  c->br2, s);
  } else {
    // mixed-form scales: Ls = the family cutoff (or the longest bond), Vs = mean volume
    double ls = c->cutoff;
    if (!(ls > 0.0)) {
      std::vector<int64_t> rp(c->n + 1);
      std::vector<int32_t> col((size_t)(c->nnz > 0 ? c->nnz : 1));
      PD_CK(c, copy_sync(rp.data(), c->row_ptr, rp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
      if (c->nnz > 0)
        PD_CK(c, copy_sync(col.data(), c->col, (size_t)c->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
      double m2 = 0.0;
      for (int64_t i = 0; i < c->n; ++i)
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
          const double ex = c->h_x[2 * col[k]] - c->h_x[2 * i], ey = c->h_x[2 * col[k] + 1] - c->h_x[2 * i + 1];
          m2 = std::max(m2, ex * ex + ey * ey);
        }
      ls = m2 > 0.0 ? std::sqrt(m2) : 1.0;
    }
    double vsum = 0.0;
    for (double v : c->h_vol) vsum += v;
    c->ls = ls;
    c->vs_scale = c->n > 0 ? vsum / (double)c->n : 1.0;
    // the scaled volumes as k_positions_mixed forms them: (float)(V_i * (1 / Vs))
    c->uniform_v = c->n > 0;
    for (double v : c->h_vol)
      if ((float)(v * (1.0 / c->vs_scale)) != 1.0f) {
        c->uniform_v = false;
        break;
      }
    const int rch = pd::build_halo_mixed(mixed_args(c), c->sell.nslots, nblocks, blocks.p, c->sell.rk, s, &c->halo,
                                         &msg);
    if (rch != PD_OK) return fail(c, rch, msg);
    int rc2 = upload_gvel(c);
    if (rc2 != PD_OK) return rc2;
  }
  if (c->n > 0) k_fam_from_rowptr<<<(unsigned)pd::blocks_for(c->n), pd::kBlock, 0, s>>>(c->n, c->row_ptr, c->fam);
  PD_CK(c, cudaGetLastError());
  {
    std::vector<int64_t> rp((size_t)c->n + 1);
    PD_CK(c, copy_sync(rp.data(), c->row_ptr, rp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    int64_t m = 0;
    for (int64_t i = 0; i < c->n; ++i) m = std::max(m, rp[i + 1] - rp[i]);
    c->max_family = (int32_t)m;
  }
  c->has_families = true;
  int rcb = ensure_ba(c);
  if (rcb != PD_OK) return rcb;
  return pd_reset(c);
}

}  // namespace

extern "C" {

int pd_abi_version(void) { return PD_ABI_VERSION; }

void pd_default_params(pd_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->precision = PD_FP64;
  p->device = 0;
  p->E = 72e9;
  p->nu = 0.33;
  p->rho = 2440.0;
  p->dt = 1e-8;
  p->s_c = 0.0;
  p->det_guard = 1e-10;
  p->k_hg = 0.0;
  p->damage_fail = 1.0;
  p->n1 = 0.0;
  p->n2 = 0.0;
  p->weight_len = 1.0;
  p->singular_policy = PD_SINGULAR_ZERO;
}

int pd_create(const pd_params* p, pd_ctx** out) {
  if (!out) {
    g_create_err = "out is NULL";
    return PD_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<pd_ctx> c(new (std::nothrow) pd_ctx());
  if (!c) {
    g_create_err = "out of host memory";
    return PD_ERR_CAPACITY;
  }
  int rc = check_params(c.get(), p);
  if (rc != PD_OK) {
    g_create_err = c->err;
    return rc;
  }
  c->p = *p;
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->counters, pd::CNT_N * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->counters, 0, pd::CNT_N * sizeof(unsigned long long), c->stream);
  if (e == cudaSuccess) e = cudaMalloc(&c->gkind, PD_MAX_BC_GROUPS * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&c->gval, PD_MAX_BC_GROUPS * sizeof(double2));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->gkind, 0, PD_MAX_BC_GROUPS * sizeof(int32_t), c->stream);
  if (e == cudaSuccess && p->precision == PD_MIXED) e = cudaMalloc(&c->gvel, PD_MAX_BC_GROUPS * sizeof(float4));
  if (e == cudaSuccess && c->gvel) e = cudaMemsetAsync(c->gvel, 0, PD_MAX_BC_GROUPS * sizeof(float4), c->stream);
  if (e != cudaSuccess) {
    g_create_err = std::string("pd_create: ") + cudaGetErrorString(e);
    pd_destroy(c.release());
    return PD_ERR_CUDA;
  }
  *out = c.release();
  return PD_OK;
}

int pd_destroy(pd_ctx* c) {
  if (!c) return PD_OK;
  if (c->batch) pd_batch_remove(c->batch, c);
  cudaSetDevice(c->p.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_particles(c);
  dfree(c->counters);
  dfree(c->gkind);
  dfree(c->gval);
  dfree(c->gvel);
  for (void* q : c->scratch) cudaFreeHost(q);
  for (cudaEvent_t e : c->slab_ev) cudaEventDestroy(e);
  for (cudaStream_t q : c->io)
    if (q) cudaStreamDestroy(q);
  for (cudaStream_t q : c->ps) cudaStreamDestroy(q);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PD_OK;
}

const char* pd_last_error(const pd_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

int pd_set_params(pd_ctx* c, const pd_params* p) {
  if (!c) return PD_ERR_ARG;
  int rc = check_params(c, p);
  if (rc != PD_OK) return rc;
  if (p->device != c->p.device || p->precision != c->p.precision)
    return fail(c, PD_ERR_ARG, "device and precision are fixed at pd_create");
  PD_CK(c, cudaSetDevice(c->p.device));
  const bool s_changed = p->s_c != c->p.s_c;
  c->p = *p;
  c->c_override = false;
  clear_graphs(c);
  if (c->has_families) {
    int rc2 = upload_gvel(c);
    if (rc2 != PD_OK) return rc2;
    rc2 = ensure_ba(c);
    if (rc2 != PD_OK) return rc2;
  }
  if (c->has_families && s_changed && !mixed(c)) {
    pd::launch_bond_limit_fp64(c->sell.nslots, c->bxi, c->p.s_c, c->sell.nbr, c->blim, c->br2, c->stream);
    PD_CK(c, cudaGetLastError());
    PD_CK(c, cudaStreamSynchronize(c->stream));
  }
  return PD_OK;
}

int pd_set_stiffness(pd_ctx* c, const double* C) {
  if (!c || !C) return PD_ERR_ARG;
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(C[k])) return fail(c, PD_ERR_ARG, "non-finite stiffness");
  if (C[0] != C[4] || C[1] != C[3] || C[2] != 0.0 || C[5] != 0.0 || C[6] != 0.0 || C[7] != 0.0)
    return fail(c, PD_ERR_ARG, "stiffness is not of the plane-stress pattern");
  c->c_override = true;
  c->c11 = C[0];
  c->c12 = C[1];
  c->c33 = C[8];
  clear_graphs(c);
  return PD_OK;
}

int pd_get_params(const pd_ctx* c, pd_params* p) {
  if (!c || !p) return PD_ERR_ARG;
  *p = c->p;
  return PD_OK;
}

int pd_set_particles(pd_ctx* c, int64_t n, const double* x, const double* vol) {
  if (!c) return PD_ERR_ARG;
  if (n < 0 || n > (int64_t)INT32_MAX - 2) return fail(c, PD_ERR_ARG, "n out of range");
  if (n > 0 && (!x || !vol)) return fail(c, PD_ERR_ARG, "x / vol is NULL");
  for (int64_t i = 0; i < 2 * n; ++i)
    if (!std::isfinite(x[i])) return fail(c, PD_ERR_ARG, "non-finite reference position");
  for (int64_t i = 0; i < n; ++i)
    if (!(vol[i] > 0.0) || !std::isfinite(vol[i])) return fail(c, PD_ERR_ARG, "volumes must be positive");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  free_particles(c);
  c->n = n;
  const size_t nn = (size_t)(n > 0 ? n : 1);
  PD_CK(c, cudaMalloc(&c->x, nn * sizeof(double2)));
  PD_CK(c, cudaMalloc(&c->u, nn * sizeof(double2)));
  PD_CK(c, cudaMalloc(&c->v, nn * sizeof(double2)));
  PD_CK(c, cudaMalloc(&c->f, nn * sizeof(double2)));
  PD_CK(c, cudaMalloc(&c->vol, nn * sizeof(double)));
  if (!mixed(c)) {  // (the mixed form's state is allocated with its families: finish_families)
    PD_CK(c, cudaMalloc(&c->acc, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->w01, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->w23, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->kinv01, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->mt, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->hg, nn * sizeof(double2)));
    PD_CK(c, cudaMalloc(&c->u32, nn * sizeof(float2)));
    PD_CK(c, cudaMalloc(&c->kinv22, nn * sizeof(double)));
  }
  PD_CK(c, cudaMalloc(&c->damage, nn * sizeof(double)));
  PD_CK(c, cudaMalloc(&c->bc, nn));
  PD_CK(c, cudaMalloc(&c->singular, nn));
  PD_CK(c, cudaMalloc(&c->broken, nn * sizeof(int32_t)));
  PD_CK(c, cudaMalloc(&c->fam, nn * sizeof(int32_t)));
  PD_CK(c, cudaMemsetAsync(c->bc, 0, nn, c->stream));
  if (n > 0) {
    PD_CK(c, copy_sync(c->x, x, (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
    PD_CK(c, copy_sync(c->vol, vol, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  c->h_x.assign(x, x + 2 * n);
  c->h_vol.assign(vol, vol + n);
  c->has_particles = true;
  return PD_OK;
}

int pd_build_families(pd_ctx* c, double cutoff, int32_t n_cracks, const double* cracks) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_particles) return fail(c, PD_ERR_ORDER, "pd_set_particles first");
  if (n_cracks > 0 && !cracks) return fail(c, PD_ERR_ARG, "cracks is NULL");
  PD_CK(c, cudaSetDevice(c->p.device));
  free_families(c);
  pd::FamilyBuild fb;
  std::string msg;
  c->cutoff = cutoff;
  int rc = pd::build_families_gpu(c->n, c->x, c->h_x.data(), cutoff, n_cracks, cracks, c->stream, &fb, &msg);
  c->row_ptr = fb.row_ptr;
  c->col = fb.col;
  c->nnz = fb.nnz;
  if (rc != PD_OK) return fail(c, rc, msg);
  return finish_families(c);
}

int pd_set_families(pd_ctx* c, const int64_t* row_ptr, const int32_t* col) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_particles) return fail(c, PD_ERR_ORDER, "pd_set_particles first");
  if (!row_ptr) return fail(c, PD_ERR_ARG, "row_ptr is NULL");
  const int64_t n = c->n;
  if (row_ptr[0] != 0) return fail(c, PD_ERR_ARG, "row_ptr[0] must be 0");
  for (int64_t i = 0; i < n; ++i) {
    const int64_t d = row_ptr[i + 1] - row_ptr[i];
    if (d < 0) return fail(c, PD_ERR_ARG, "row_ptr must be non-decreasing");
    if (d > PD_MAX_FAMILY) return fail(c, PD_ERR_CAPACITY, "a family exceeds PD_MAX_FAMILY bonds");
  }
  const int64_t nnz = row_ptr[n];
  if (nnz > 0 && !col) return fail(c, PD_ERR_ARG, "col is NULL");
  PD_CK(c, cudaSetDevice(c->p.device));
  free_families(c);
  c->cutoff = 0.0;
  c->nnz = nnz;
  PD_CK(c, cudaMalloc(&c->row_ptr, (size_t)(n + 1) * sizeof(int64_t)));
  PD_CK(c, cudaMalloc(&c->col, (size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t)));
  PD_CK(c, copy_sync(c->row_ptr, row_ptr, (size_t)(n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
  if (nnz > 0) PD_CK(c, copy_sync(c->col, col, (size_t)nnz * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  return finish_families(c);
}

int pd_num_bonds(const pd_ctx* c, int64_t* nnz) {
  if (!c || !nnz) return PD_ERR_ARG;
  *nnz = c->nnz;
  return PD_OK;
}

int pd_get_families(pd_ctx* c, int64_t* row_ptr, int32_t* col) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "no families");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  if (row_ptr)
    PD_CK(c, copy_sync(row_ptr, c->row_ptr, (size_t)(c->n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  if (col && c->nnz > 0)
    PD_CK(c, copy_sync(col, c->col, (size_t)c->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  return PD_OK;
}

int pd_set_bc(pd_ctx* c, int32_t n_groups, const int32_t* kind, const double* value, const uint8_t* group_of) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_particles) return fail(c, PD_ERR_ORDER, "pd_set_particles first");
  if (n_groups < 0 || n_groups > PD_MAX_BC_GROUPS) return fail(c, PD_ERR_ARG, "n_groups out of range");
  if (n_groups > 0 && (!kind || !value)) return fail(c, PD_ERR_ARG, "kind / value is NULL");
  for (int g = 0; g < n_groups; ++g)
    if (kind[g] != PD_BC_NONE && kind[g] != PD_BC_VELOCITY && kind[g] != PD_BC_FIXED)
      return fail(c, PD_ERR_ARG, "unknown BC kind");
  if (group_of)
    for (int64_t i = 0; i < c->n; ++i)
      if (group_of[i] > n_groups) return fail(c, PD_ERR_ARG, "group_of refers to a missing group");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  std::vector<int32_t> k(PD_MAX_BC_GROUPS, PD_BC_NONE);
  std::vector<double> val(2 * PD_MAX_BC_GROUPS, 0.0);
  for (int g = 0; g < n_groups; ++g) {
    k[g] = kind[g];
    val[2 * g] = value[2 * g];
    val[2 * g + 1] = value[2 * g + 1];
  }
  PD_CK(c, copy_sync(c->gkind, k.data(), k.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  PD_CK(c, copy_sync(c->gval, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  c->h_gval = val;
  if (c->has_families) {
    int rc = upload_gvel(c);
    if (rc != PD_OK) return rc;
  }
  if (c->n > 0) {
    if (group_of)
      PD_CK(c, copy_sync(c->bc, group_of, (size_t)c->n, cudaMemcpyHostToDevice, c->stream));
    else
      PD_CK(c, cudaMemsetAsync(c->bc, 0, (size_t)c->n, c->stream));
  }
  if (mixed(c) && c->has_families) {
    pd::launch_bc_by_position(c->sell.npos, c->sell.member, c->bc, c->bcp, c->stream);
    PD_CK(c, cudaGetLastError());
    PD_CK(c, cudaStreamSynchronize(c->stream));
  }
  return PD_OK;
}

int pd_reset(pd_ctx* c) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  PD_CK(c, cudaSetDevice(c->p.device));
  cudaStream_t s = c->stream;
  const size_t nn = (size_t)(c->n > 0 ? c->n : 1);
  PD_CK(c, cudaMemsetAsync(c->u, 0, nn * sizeof(double2), s));
  PD_CK(c, cudaMemsetAsync(c->v, 0, nn * sizeof(double2), s));
  PD_CK(c, cudaMemsetAsync(c->f, 0, nn * sizeof(double2), s));
  PD_CK(c, cudaMemsetAsync(c->broken, 0, nn * sizeof(int32_t), s));
  PD_CK(c, cudaMemsetAsync(c->damage, 0, nn * sizeof(double), s));
  PD_CK(c, cudaMemsetAsync(c->counters, 0, pd::CNT_N * sizeof(unsigned long long), s));
  pd::launch_sell_reset(c->n, c->row_ptr, c->col, c->sell, s);
  if (mixed(c)) {
    pd::launch_halo_relink(mixed_args(c), c->halo, s);
    const size_t np = (size_t)(c->sell.npos > 0 ? c->sell.npos : 1);
    PD_CK(c, cudaMemsetAsync(c->us, 0, np * sizeof(float4), s));
    PD_CK(c, cudaMemsetAsync(c->vsm, 0, np * sizeof(float4), s));
    PD_CK(c, cudaMemsetAsync(c->ws, 0, np * sizeof(float4), s));
    PD_CK(c, cudaMemsetAsync(c->fs, 0, np * sizeof(float2), s));
    PD_CK(c, cudaMemsetAsync(c->hgs, 0, np * sizeof(float2), s));
    pd::launch_init_geometry_mixed(mixed_args(c), s);
  } else {
    PD_CK(c, cudaMemsetAsync(c->acc, 0, nn * sizeof(double2), s));
    PD_CK(c, cudaMemsetAsync(c->w01, 0, nn * sizeof(double2), s));
    PD_CK(c, cudaMemsetAsync(c->w23, 0, nn * sizeof(double2), s));
    PD_CK(c, cudaMemsetAsync(c->hg, 0, nn * sizeof(double2), s));
    PD_CK(c, cudaMemsetAsync(c->u32, 0, nn * sizeof(float2), s));
    pd::launch_init_geometry_fp64(fp64_args(c), s);
  }
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaStreamSynchronize(s));
  c->steps = 0;
  return PD_OK;
}

int pd_set_state(pd_ctx* c, const double* u, const double* v, const double* f) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_particles) return fail(c, PD_ERR_ORDER, "pd_set_particles first");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  const size_t b = (size_t)c->n * sizeof(double2);
  if (b == 0) return PD_OK;
  if (mixed(c) && !c->has_families) return fail(c, PD_ERR_ORDER, "mixed form: families first (they fix the scales)");
  // one stream, one wait: copies from page-locked buffers run at full link speed
  cudaStream_t s = c->stream;
  if (u) PD_CK(c, cudaMemcpyAsync(c->u, u, b, cudaMemcpyHostToDevice, s));
  if (v) PD_CK(c, cudaMemcpyAsync(c->v, v, b, cudaMemcpyHostToDevice, s));
  if (f) PD_CK(c, cudaMemcpyAsync(c->f, f, b, cudaMemcpyHostToDevice, s));
  if (mixed(c))
    pd::launch_to_mixed(mixed_args(c), u ? c->u : nullptr, v ? c->v : nullptr, f ? c->f : nullptr, s);
  else if (u && c->has_families)
    pd::launch_shadow_fp64(fp64_args(c), s);
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaStreamSynchronize(s));
  return PD_OK;
}

int pd_get_state(pd_ctx* c, double* u, double* v, double* f) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_particles) return fail(c, PD_ERR_ORDER, "pd_set_particles first");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  const size_t b = (size_t)c->n * sizeof(double2);
  if (b == 0) return PD_OK;
  if (mixed(c) && !c->has_families) return fail(c, PD_ERR_ORDER, "mixed form: families first (they fix the scales)");
  cudaStream_t s = c->stream;
  if (mixed(c)) {
    pd::launch_from_mixed(mixed_args(c), u ? c->u : nullptr, v ? c->v : nullptr, f ? c->f : nullptr, s);
    PD_CK(c, cudaGetLastError());
  }
  if (u) PD_CK(c, cudaMemcpyAsync(u, c->u, b, cudaMemcpyDeviceToHost, s));
  if (v) PD_CK(c, cudaMemcpyAsync(v, c->v, b, cudaMemcpyDeviceToHost, s));
  if (f) PD_CK(c, cudaMemcpyAsync(f, c->f, b, cudaMemcpyDeviceToHost, s));
  PD_CK(c, cudaStreamSynchronize(s));
  return PD_OK;
}

int pd_get_damage(pd_ctx* c, double* damage) {
  if (!c || !damage) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  if (c->n > 0)
    PD_CK(c, copy_sync(damage, c->damage, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return PD_OK;
}

int pd_get_bond_mask(pd_ctx* c, uint8_t* alive) {
  if (!c || !alive) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  PD_CK(c, cudaSetDevice(c->p.device));
  if (c->nnz == 0) return PD_OK;
  uint8_t* d = nullptr;
  PD_CK(c, cudaMallocAsync(&d, (size_t)c->nnz, c->stream));
  pd::launch_mask_out(c->n, c->row_ptr, c->col, c->sell, d, c->stream);
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaMemcpyAsync(alive, d, (size_t)c->nnz, cudaMemcpyDeviceToHost, c->stream));
  PD_CK(c, cudaFreeAsync(d, c->stream));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  return PD_OK;
}

int pd_get_counters(pd_ctx* c, pd_counters* out) {
  if (!c || !out) return PD_ERR_ARG;
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  unsigned long long h[pd::CNT_N];
  PD_CK(c, copy_sync(h, c->counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  out->bonds_broken = (int64_t)h[pd::CNT_BROKEN];
  out->singular_events = (int64_t)h[pd::CNT_SINGULAR];
  out->steps = c->steps;
  out->device_error = (int32_t)h[pd::CNT_ERROR];
  out->unstaged_blocks = (int32_t)(c->halo.nblocks - c->halo.staged);
  return PD_OK;
}

}  // extern "C"

namespace {

// Launch sequence of nsteps steps on stream s (graph-capturable).
// One launcher per kernel kind, so graph capture and per-kernel profiling
// issue the same sequence.
struct Launcher {
  pd_ctx* c;
  Fp64Args f;
  pd::MixedArgs m;
  bool brk;
  explicit Launcher(pd_ctx* ctx) : c(ctx), brk(ctx->p.s_c > 0.0) {
    if (mixed(ctx))
      m = mixed_args(ctx);
    else
      f = fp64_args(ctx);
  }
  void drift(cudaStream_t s) {
    if (mixed(c)) pd::launch_drift_mixed(m, s); else pd::launch_drift_fp64(f, s);
  }
  void pass_a(cudaStream_t s) {
    if (mixed(c))
      pd::launch_pass_a_mixed(m, brk, s);
    else if (bond_assoc(c))
      pd::launch_ba_pass_a(f, ba_args(c), s);
    else
      pd::launch_pass_a_fp64(f, brk, s, true);
  }
  void pass_b(bool next_drift, cudaStream_t s) {
    if (mixed(c))
      pd::launch_pass_b_mixed(m, next_drift, s);
    else if (bond_assoc(c))
      pd::launch_ba_pass_b(f, ba_args(c), next_drift ? 1 : 0, s);
    else
      pd::launch_pass_b_fp64(f, next_drift ? 1 : 0, s, true);
  }
};

void enqueue_steps(pd_ctx* c, int32_t nsteps, cudaStream_t s) {
  Launcher L(c);
  L.drift(s);
  for (int32_t k = 0; k < nsteps; ++k) {
    L.pass_a(s);
    L.pass_b(k + 1 < nsteps, s);
  }
}

int check_after_step(pd_ctx* c) {
  if (c->p.singular_policy != PD_SINGULAR_ERROR) return PD_OK;
  unsigned long long h = 0;
  PD_CK(c, cudaMemcpyAsync(&h, c->counters + pd::CNT_SINGULAR, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  if (h) return fail(c, PD_ERR_SINGULAR, "det(K) guard tripped for " + std::to_string(h) + " particle update(s)");
  return PD_OK;
}

// The graph of nsteps steps of c (enqueue_steps' launches), captured on c's stream on first use.
int step_graph(pd_ctx* c, int32_t nsteps, cudaGraphExec_t* out) {
  auto it = c->graphs.find(nsteps);
  if (it == c->graphs.end()) {
    cudaGraph_t g;
    PD_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_steps(c, nsteps, c->stream);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph capture");
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
    if (c->graphs.size() > 16) {  // a bound on the cache (the arguments are not stale)
      for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
      c->graphs.clear();
    }
    it = c->graphs.emplace(nsteps, ge).first;
  }
  *out = it->second;
  return PD_OK;
}

}  // namespace

extern "C" {

int pd_step(pd_ctx* c, int32_t nsteps) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  if (nsteps < 0) return fail(c, PD_ERR_ARG, "nsteps < 0");
  if (nsteps == 0 || c->n == 0) {
    c->steps += nsteps;
    return PD_OK;
  }
  PD_CK(c, cudaSetDevice(c->p.device));
  cudaGraphExec_t ge = nullptr;
  const int rc = step_graph(c, nsteps, &ge);
  if (rc != PD_OK) return rc;
  PD_CK(c, cudaGraphLaunch(ge, c->stream));
  c->steps += nsteps;
  return check_after_step(c);
}

// ---- Mazars damage
namespace {

pd::MazarsArgs mazars_args(pd_ctx* c) {
  pd::MazarsArgs m{};
  m.kappa0 = c->mz.kappa0;
  m.a_t = c->mz.a_t;
  m.b_t = c->mz.b_t;
  m.a_c = c->mz.a_c;
  m.b_c = c->mz.b_c;
  m.thr = c->mz_thr;
  m.bd = c->mz_bd;
  m.status = c->mz_status;
  return m;
}

bool bond_associated(const pd_ctx* c) { return c->p.n1 != 0.0 || c->p.n2 != 0.0; }

}  // namespace

void pd_mazars_default_params(pd_mazars_params* p) {
  if (!p) return;
  p->kappa0 = 3.0 / 3.5e4;
  p->a_t = 0.87;
  p->b_t = 20000.0;
  p->a_c = 0.65;
  p->b_c = 2150.0;
}

int pd_mazars_init(pd_ctx* c, const pd_mazars_params* p) {
  if (!c || !p) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  if (mixed(c)) return fail(c, PD_ERR_ARG, "Mazars damage needs PD_FP64");
  if (!(p->kappa0 >= 0.0) || !std::isfinite(p->kappa0) || !std::isfinite(p->a_t) || !std::isfinite(p->b_t) ||
      !std::isfinite(p->a_c) || !std::isfinite(p->b_c))
    return fail(c, PD_ERR_ARG, "invalid Mazars parameters");
  if (bond_associated(c) && c->max_family > 64)
    return fail(c, PD_ERR_CAPACITY, "bond-associated Mazars damage: families are limited to 64 bonds");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  const size_t ns = (size_t)(c->sell.nslots > 0 ? c->sell.nslots : 1), nn = (size_t)(c->n > 0 ? c->n : 1);
  if (!c->mz_thr) PD_CK(c, cudaMalloc(&c->mz_thr, ns * sizeof(double)));
  if (!c->mz_bd) PD_CK(c, cudaMalloc(&c->mz_bd, ns * sizeof(double)));
  if (!c->mz_status) PD_CK(c, cudaMalloc(&c->mz_status, nn * sizeof(double)));
  c->mz = *p;
  pd::launch_mazars_reset(c->sell.nslots, c->n, mazars_args(c), c->stream);
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaStreamSynchronize(c->stream));
  return PD_OK;
}

int pd_mazars_update(pd_ctx* c) {
  if (!c) return PD_ERR_ARG;
  if (!c->mz_thr) return fail(c, PD_ERR_ORDER, "pd_mazars_init first");
  PD_CK(c, cudaSetDevice(c->p.device));
  const pd::BondAssoc ba = ba_args(c);
  pd::launch_mazars_update(fp64_args(c), bond_associated(c) ? &ba : nullptr, mazars_args(c), c->stream);
  PD_CK(c, cudaGetLastError());
  return PD_OK;
}

int pd_mazars_get(pd_ctx* c, double* thr, double* bd, double* status) {
  if (!c) return PD_ERR_ARG;
  if (!c->mz_thr) return fail(c, PD_ERR_ORDER, "pd_mazars_init first");
  PD_CK(c, cudaSetDevice(c->p.device));
  cudaStream_t s = c->stream;
  if ((thr || bd) && c->nnz > 0) {
    double *dt = nullptr, *db = nullptr;
    if (thr) PD_CK(c, cudaMallocAsync(&dt, (size_t)c->nnz * sizeof(double), s));
    if (bd) PD_CK(c, cudaMallocAsync(&db, (size_t)c->nnz * sizeof(double), s));
    pd::launch_mazars_to_csr(fp64_args(c), c->row_ptr, mazars_args(c), dt, db, s);
    PD_CK(c, cudaGetLastError());
    if (thr) PD_CK(c, cudaMemcpyAsync(thr, dt, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (bd) PD_CK(c, cudaMemcpyAsync(bd, db, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (dt) PD_CK(c, cudaFreeAsync(dt, s));
    if (db) PD_CK(c, cudaFreeAsync(db, s));
  }
  if (status && c->n > 0)
    PD_CK(c, cudaMemcpyAsync(status, c->mz_status, (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, s));
  PD_CK(c, cudaStreamSynchronize(s));
  return PD_OK;
}

int pd_mazars_set(pd_ctx* c, const double* thr, const double* bd) {
  if (!c) return PD_ERR_ARG;
  if (!c->mz_thr) return fail(c, PD_ERR_ORDER, "pd_mazars_init first");
  PD_CK(c, cudaSetDevice(c->p.device));
  cudaStream_t s = c->stream;
  if (c->nnz > 0) {
    double *dt = nullptr, *db = nullptr;
    if (thr) {
      PD_CK(c, cudaMallocAsync(&dt, (size_t)c->nnz * sizeof(double), s));
      PD_CK(c, cudaMemcpyAsync(dt, thr, (size_t)c->nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    if (bd) {
      PD_CK(c, cudaMallocAsync(&db, (size_t)c->nnz * sizeof(double), s));
      PD_CK(c, cudaMemcpyAsync(db, bd, (size_t)c->nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    pd::launch_mazars_from_csr(fp64_args(c), c->row_ptr, mazars_args(c), dt, db, s);
    PD_CK(c, cudaGetLastError());
    if (dt) PD_CK(c, cudaFreeAsync(dt, s));
    if (db) PD_CK(c, cudaFreeAsync(db, s));
  }
  PD_CK(c, cudaStreamSynchronize(s));
  return PD_OK;
}

// ---- checkpoint / restore
namespace {

struct CkptHeader {
  char magic[8];
  int32_t abi, precision;
  int64_t n, nslots, nnz, steps;
  uint64_t problem;  // FNV-1a of the reference positions, volumes, families layout and parameters
  unsigned long long counters[pd::CNT_N];
  int32_t mazars, pad;   // 1: the Mazars history follows the state arrays
  pd_mazars_params mz;
};

uint64_t fnv1a(uint64_t h, const void* p, size_t bytes) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t k = 0; k < bytes; ++k) {
    h ^= b[k];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t problem_hash(const pd_ctx* c) {
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, c->h_x.data(), c->h_x.size() * sizeof(double));
  h = fnv1a(h, c->h_vol.data(), c->h_vol.size() * sizeof(double));
  const double p[] = {c->p.E, c->p.nu, c->p.rho, c->p.dt, c->p.s_c, c->p.k_hg, c->p.damage_fail, c->p.n1, c->p.n2};
  h = fnv1a(h, p, sizeof(p));
  h = fnv1a(h, &c->nnz, sizeof(c->nnz));
  h = fnv1a(h, &c->sell.nslots, sizeof(c->sell.nslots));
  return h;
}

// (device pointer, bytes) of every saved array, in blob order
std::vector<std::pair<void*, size_t>> ckpt_arrays(pd_ctx* c) {
  const size_t n = (size_t)c->n, ns = (size_t)c->sell.nslots;
  std::vector<std::pair<void*, size_t>> a;
  if (mixed(c)) {  // by SELL position
    const size_t np = (size_t)c->sell.npos;
    a.push_back({c->us, np * sizeof(float4)});
    a.push_back({c->vsm, np * sizeof(float4)});
    a.push_back({c->fs, np * sizeof(float2)});
  } else {
    a.push_back({c->u, n * sizeof(double2)});
    a.push_back({c->v, n * sizeof(double2)});
    a.push_back({c->f, n * sizeof(double2)});
    a.push_back({c->acc, n * sizeof(double2)});
  }
  a.push_back({c->broken, n * sizeof(int32_t)});
  a.push_back({c->damage, n * sizeof(double)});
  a.push_back({c->sell.nbr, ns * sizeof(int32_t)});
  if (c->mz_thr) {
    a.push_back({c->mz_thr, ns * sizeof(double)});
    a.push_back({c->mz_bd, ns * sizeof(double)});
    a.push_back({c->mz_status, n * sizeof(double)});
  }
  return a;
}

int ckpt_bytes(pd_ctx* c, int64_t* bytes) {
  int64_t b = (int64_t)sizeof(CkptHeader);
  for (const auto& x : ckpt_arrays(c)) b += (int64_t)x.second;
  *bytes = b;
  return PD_OK;
}

}  // namespace

int pd_checkpoint_size(pd_ctx* c, int64_t* bytes) {
  if (!c || !bytes) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  return ckpt_bytes(c, bytes);
}

int pd_checkpoint_save(pd_ctx* c, void* buf, int64_t bytes) {
  if (!c || !buf) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  int64_t need = 0;
  ckpt_bytes(c, &need);
  if (bytes < need) return fail(c, PD_ERR_CAPACITY, "checkpoint buffer too small (pd_checkpoint_size)");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  CkptHeader h{};
  std::memcpy(h.magic, "PDCKPT01", 8);
  h.abi = PD_ABI_VERSION;
  h.precision = c->p.precision;
  h.n = c->n;
  h.nslots = c->sell.nslots;
  h.nnz = c->nnz;
  h.steps = c->steps;
  h.problem = problem_hash(c);
  h.mazars = c->mz_thr ? 1 : 0;
  h.mz = c->mz;
  PD_CK(c, copy_sync(h.counters, c->counters, sizeof(h.counters), cudaMemcpyDeviceToHost, c->stream));
  unsigned char* o = static_cast<unsigned char*>(buf);
  std::memcpy(o, &h, sizeof(h));
  o += sizeof(h);
  for (const auto& x : ckpt_arrays(c)) {
    if (x.second) PD_CK(c, copy_sync(o, x.first, x.second, cudaMemcpyDeviceToHost, c->stream));
    o += x.second;
  }
  return PD_OK;
}

int pd_checkpoint_load(pd_ctx* c, const void* buf, int64_t bytes) {
  if (!c || !buf) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  CkptHeader h;
  if (bytes < (int64_t)sizeof(h)) return fail(c, PD_ERR_ARG, "not a checkpoint (too short)");
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "PDCKPT01", 8) != 0 || h.abi != PD_ABI_VERSION)
    return fail(c, PD_ERR_ARG, "not a checkpoint of this library version");
  if (h.precision != c->p.precision) return fail(c, PD_ERR_ARG, "checkpoint precision differs from the context's");
  if (h.n != c->n || h.nslots != c->sell.nslots || h.nnz != c->nnz || h.problem != problem_hash(c))
    return fail(c, PD_ERR_ARG, "checkpoint of another problem (particles, families or parameters differ)");
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  // the Mazars history follows the blob: allocated if it has one, dropped if not
  if (h.mazars && !c->mz_thr) {
    const int rc = pd_mazars_init(c, &h.mz);
    if (rc != PD_OK) return rc;
  } else if (!h.mazars && c->mz_thr) {
    dfree(c->mz_thr);
    dfree(c->mz_bd);
    dfree(c->mz_status);
  }
  c->mz = h.mz;
  int64_t need = 0;
  ckpt_bytes(c, &need);
  if (bytes < need) return fail(c, PD_ERR_ARG, "checkpoint truncated");
  const unsigned char* p = static_cast<const unsigned char*>(buf) + sizeof(h);
  for (const auto& x : ckpt_arrays(c)) {
    if (x.second) PD_CK(c, copy_sync(x.first, p, x.second, cudaMemcpyHostToDevice, c->stream));
    p += x.second;
  }
  // derived data: K^-1 / m / singular flags from the restored mask and broken counts,
  // the FP32 shadows (FP64 form) or the live halo indices (mixed form)
  cudaStream_t s = c->stream;
  if (mixed(c)) {
    pd::launch_halo_relink(mixed_args(c), c->halo, s);
    pd::launch_init_geometry_mixed(mixed_args(c), s);
  } else {
    pd::launch_init_geometry_fp64(fp64_args(c), s);
    pd::launch_shadow_fp64(fp64_args(c), s);
  }
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaMemcpyAsync(c->counters, h.counters, sizeof(h.counters), cudaMemcpyHostToDevice, s));
  PD_CK(c, cudaStreamSynchronize(s));
  c->steps = h.steps;
  return PD_OK;
}


// pd_step_host pipeline (FP64 form).  The particles are cut into kSlabs index
// ranges (multiples of 32): 1/64 and 3/64 of the plate, six of 1/8, then 3/32,
// 1/16 and 1/32, so the first pass A starts after a few microseconds of
// copying, the later copies stay ahead of it, and the last slabs, whose pass
// B and write-back end the call, are short (1M-particle plate, ms per one-step
// call: these slabs 0.844-0.848 against 0.864-0.887 for seven of 1/8 after the
// same two; 1/128, 1/128, 1/64, 1/32, 1/16, then seven of 1/8 0.862; 1/32,
// 3/32, 1/8, then four of 3/16 0.862; five of 3/16 after 1/16 0.874; trailing
// 1/16, 1/16, 1/32, 1/64, 1/64 or 3/32, 3/32, 1/16, 1/32, 1/32 0.857-0.866);
// slab_need[k] / slab_low[k] = the last / first slab holding a neighbour of
// slab k's particles.  Streams (io[0], io[1] at high priority): io[1] copies
// u, v, f in slab by slab, io[0] runs each slab's drift as its copy lands (the
// first kZeroCopySlabs slabs' drifts read the input buffers directly),
// pass A of slab k starts on its own stream once slabs 0 .. slab_need[k] are
// in, and, in one-step calls, pass B of slab k (its own stream) once pass A
// of slabs slab_low[k] .. slab_need[k] is done, writing the slab's new state
// straight to the host buffers -- so the device-to-host traffic runs under
// the later slabs' pass A instead of after it.  One stream per launch: an
// FP64 pass A block runs for ~70 us whatever the slab's size (one thread per
// particle, FP64-latency bound when the SM is not full), so slab launches
// queued on shared streams would wait out each other's tails.
constexpr int kSlabs = 11;
// the first slabs are imported by their drift kernel reading the page-locked input directly
// (no copy-engine start-up before the first pass A can begin: 0.852-0.855 -> 0.843-0.846 ms
// per one-step call on the 1M-particle plate); the rest by copy engine
constexpr int kZeroCopySlabs = 2;
enum {
  kEvImport = 0,
  kEvCopy = kSlabs,
  kEvA = 2 * kSlabs,
  kEvB = 3 * kSlabs,
  kEvStart = 4 * kSlabs,
  kEvJoin = 4 * kSlabs + 1,
  kEvCount = 4 * kSlabs + 2
};

constexpr int kMaxSlabs = 16;  // the most slabs either form's pipeline uses
static_assert(kSlabs <= kMaxSlabs, "one pass stream pair per slab");

// The pipeline's streams (io[0], io[1], io[5] at high priority; the per-slab
// pass streams at low priority) and events.
static int pipeline_streams(pd_ctx* c, int nev) {
  if (!c->io[0]) {
    int lo = 0, hi = 0;
    PD_CK(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int q = 0; q < 6; ++q)
      PD_CK(c, cudaStreamCreateWithPriority(&c->io[q], cudaStreamNonBlocking, q < 2 || q == 5 ? hi : lo));
    while ((int)c->ps.size() < 2 * kMaxSlabs) {
      cudaStream_t q;
      PD_CK(c, cudaStreamCreateWithPriority(&q, cudaStreamNonBlocking, lo));
      c->ps.push_back(q);
    }
  }
  while ((int)c->slab_ev.size() < nev) {
    cudaEvent_t e;
    PD_CK(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->slab_ev.push_back(e);
  }
  return PD_OK;
}

static int plan_slabs(pd_ctx* c) {
  if (!c->slab_bnd.empty()) return PD_OK;
  const int rs = pipeline_streams(c, kEvCount);
  if (rs != PD_OK) return rs;
  // the largest and smallest neighbour id of every 32-particle chunk
  const int64_t nch = (c->n + 31) / 32;
  std::vector<int32_t> h((size_t)nch, 0), hl((size_t)nch, 0);
  int32_t* reach = nullptr;
  PD_CK(c, cudaMalloc(&reach, 2 * h.size() * sizeof(int32_t)));
  cudaError_t e = cudaMemsetAsync(reach, 0, h.size() * sizeof(int32_t), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(reach + nch, 0x7f, h.size() * sizeof(int32_t), c->stream);
  if (e == cudaSuccess) {
    pd::launch_slab_reach(c->n, c->row_ptr, c->col, 32, reach, reach + nch, c->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = copy_sync(h.data(), reach, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = copy_sync(hl.data(), reach + nch, hl.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  cudaFree(reach);
  PD_CK(c, e);
  // slab boundaries in chunks: 1/64, 3/64, six of 1/8, then 3/32, 1/16, 1/32
  static const int kShare[kSlabs] = {4, 12, 32, 32, 32, 32, 32, 32, 24, 16, 8};  // of 256
  std::vector<int64_t> bc(kSlabs + 1, 0);
  int acc = 0;
  for (int k = 0; k < kSlabs; ++k) {
    acc += kShare[k];
    bc[k + 1] = k + 1 == kSlabs ? nch : std::min<int64_t>(nch, std::max<int64_t>(bc[k] + 1, nch * acc / 256));
  }
  c->slab_bnd.assign(kSlabs + 1, 0);
  for (int k = 0; k <= kSlabs; ++k) c->slab_bnd[k] = std::min<int64_t>(c->n, bc[k] * 32);
  c->slab_need.assign(kSlabs, 0);
  c->slab_low.assign(kSlabs, 0);
  for (int k = 0; k < kSlabs; ++k) {
    int64_t far = -1, near = INT64_MAX;
    for (int64_t q = bc[k]; q < bc[k + 1]; ++q) {
      far = std::max<int64_t>(far, h[(size_t)q]);
      near = std::min<int64_t>(near, hl[(size_t)q]);
    }
    int need = k, low = k;
    while (need + 1 < kSlabs && far >= c->slab_bnd[need + 1]) ++need;
    while (low > 0 && near < c->slab_bnd[low]) --low;
    c->slab_need[k] = need;
    c->slab_low[k] = low;
  }
  return PD_OK;
}

// Fp64Args restricted to slab k.
static Fp64Args slab_args(const pd_ctx* c, const Fp64Args& a, int k) {
  Fp64Args r = a;
  r.i0 = c->slab_bnd[k];
  r.n = c->slab_bnd[k + 1];
  return r;
}

// Enqueues pd_step_host's pipeline (slabs planned) on the main stream.  (A
// CUDA graph of it measured the same: the GPU, not the enqueue, sets the pace.)
// dropin: pd_compute_velocity's one call instead (nsteps 1; f_in is acce):
// each slab's import takes u, velocity and acce and forms the FP32 shadow
// (no drift), and pass B is the drop-in kick (mode 2), writing velocity,
// acce and the force to out's buffers.
static cudaError_t enqueue_host_step(pd_ctx* c, int32_t nsteps, const double* u_in, const double* v_in,
                                     const double* f_in, const Fp64Args& plain, const Fp64Args& out, bool brk,
                                     bool dropin = false) {
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  cudaStream_t s = c->stream;
  cudaEvent_t* ev = c->slab_ev.data();
  cudaStream_t* io = c->io;
  const size_t b16 = sizeof(double2);
  ck(cudaEventRecord(ev[kEvStart], s));
  for (int q = 0; q < 2; ++q) ck(cudaStreamWaitEvent(io[q], ev[kEvStart], 0));
  cudaStream_t* pa = c->ps.data();           // pass A of slab k: pa[k]
  cudaStream_t* pb = c->ps.data() + kMaxSlabs;  // pass B of slab k: pb[k]
  // enqueued in dependency order (each pass A right after the import it waits for, each
  // pass B right after the last pass A it waits for), so the first pass A is submitted
  // before the host has issued the later imports
  const bool one = nsteps == 1;
  int next_a = 0, next_b = 0;
  for (int k = 0; k < kSlabs; ++k) {
    const Fp64Args a = slab_args(c, plain, k);  // import slab k
    const size_t off = (size_t)a.i0, cnt = (size_t)(a.n - a.i0);
    if (k < kZeroCopySlabs) {  // the import kernel reads the page-locked input itself
      Fp64Args z = a;
      z.in_u = static_cast<const double2*>(mapped_host(u_in));
      z.in_v = static_cast<const double2*>(mapped_host(v_in));
      if (dropin) {
        z.in_a = static_cast<const double2*>(mapped_host(f_in));
        pd::launch_shadow_fp64(z, io[0]);
      } else {
        z.in_f = static_cast<const double2*>(mapped_host(f_in));
        pd::launch_drift_fp64(z, io[0]);
      }
    } else {
      if (cnt > 0) {
        ck(cudaMemcpyAsync(c->u + off, u_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice, io[1]));
        ck(cudaMemcpyAsync(c->v + off, v_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice, io[1]));
        ck(cudaMemcpyAsync((dropin ? c->acc : c->f) + off, f_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice,
                           io[1]));
      }
      ck(cudaEventRecord(ev[kEvCopy + k], io[1]));
      ck(cudaStreamWaitEvent(io[0], ev[kEvCopy + k], 0));
      if (dropin)
        pd::launch_shadow_fp64(a, io[0]);  // on the device copy
      else
        pd::launch_drift_fp64(a, io[0]);  // in place, on the device copy
    }
    ck(cudaEventRecord(ev[kEvImport + k], io[0]));
    for (; next_a < kSlabs && c->slab_need[next_a] <= k; ++next_a) {  // pass A of slabs whose neighbours are in
      cudaStream_t sj = pa[next_a];
      ck(cudaStreamWaitEvent(sj, ev[kEvImport + c->slab_need[next_a]], 0));  // (after the call's start)
      pd::launch_pass_a_fp64(slab_args(c, plain, next_a), brk, sj);
      ck(cudaEventRecord(ev[kEvA + next_a], sj));
      // one-step calls: pass B (with the write-back) of every slab whose neighbours' pass A is in
      for (; one && next_b < kSlabs && c->slab_need[next_b] <= next_a; ++next_b) {
        cudaStream_t sb = pb[next_b];
        for (int q = c->slab_low[next_b]; q <= c->slab_need[next_b]; ++q) ck(cudaStreamWaitEvent(sb, ev[kEvA + q], 0));
        pd::launch_pass_b_fp64(slab_args(c, out, next_b), dropin ? 2 : 0, sb);
        ck(cudaEventRecord(ev[kEvB + next_b], sb));
      }
    }
  }
  if (one && next_b != kSlabs) e = e == cudaSuccess ? cudaErrorLaunchFailure : e;  // (a plan bug)
  // join every stream's work on the main stream
  auto join = [&](cudaStream_t q) {
    ck(cudaEventRecord(ev[kEvJoin], q));
    ck(cudaStreamWaitEvent(s, ev[kEvJoin], 0));
  };
  join(io[0]);
  for (int k = 0; k < kSlabs; ++k) join(pa[k]);
  for (int k = 0; one && k < kSlabs; ++k) join(pb[k]);
  if (!one)
    for (int32_t k = 0; k < nsteps; ++k) {
      const bool last = k + 1 == nsteps;
      if (k > 0) pd::launch_pass_a_fp64(plain, brk, s);
      pd::launch_pass_b_fp64(last ? out : plain, last ? 0 : 1, s);  // the last writes the state back
    }
  ck(cudaGetLastError());
  return e;
}

// pd_step_host pipeline, mixed form: a wavefront over slabs of visiting blocks
// (spatial tiles in order, eight even slabs).  A slab is
// a run of visiting blocks, and everything about it -- which positions it
// imports, which slabs its bonds reach -- is taken through the blocks' visit
// records, since a tile's last block holds fewer chunks than kHaloBlock / 32.
// Moving the state is the cost here: 48 B per particle each way in FP64
// against a step that takes ~0.1 us per 1k particles, over a CPU-GPU link of
// ~200 GB/s each way (~165 GB/s each way when both run).  The input comes in
// by copy engine, by slabs of particle ids, into the context's FP64 staging
// buffers (u, v, f); the output goes straight from each slab's pass B to the
// output buffers (on the 1M-particle plate: 0.56 ms per one-step call,
// against 0.63 with pass B writing the staging buffers and copy engines taking
// id slabs out, and 0.67 with an import kernel reading the host buffers).
// Each slab costs three copies in: 8 even slabs measured 0.556-0.566 ms per
// call (a Python harness) against 0.599-0.603 for 16 (two of 1/64, one of 1/32, then even); 9 or
// 10 slabs with short leading or trailing ones the same as 8, 7 slabs 0.579,
// 6 0.609, 4 0.605 (each a bit-identical result).  The streams:
//   io[1]  copies id slab k in;
//   io[0]  imports slab k (conversion to the scaled state + drift, from the
//          staging buffers) once id slabs 0 .. k are in;
//   its own stream: pass A of slab k once the slabs its bonds reach are
//          imported;
//   its own stream (one-step calls): pass B of slab k once pass A of those
//          slabs is done, writing the new FP64 state by particle id to the
//          output buffers over the link -- while later slabs are still coming in.
// Id slab k ends after the highest id of slabs 0 .. k, so slab k's import
// needs id slabs 0 .. k only (a row-major numbering gives slabs of whole
// rows; any numbering is correct, a scrambled one just pipelines less).  With
// the input and output buffers the same, slab k's pass B overwrites only ids
// of id slabs 0 .. k, whose copies in are complete before its import.
constexpr int kMixedSlabs = 8;
static_assert(kMixedSlabs <= kMaxSlabs, "one pass stream pair per slab");
enum { kMEvIn = 0, kMEvImport = kMixedSlabs, kMEvA = 2 * kMixedSlabs, kMEvB = 3 * kMixedSlabs,
       kMEvStart = 4 * kMixedSlabs, kMEvCount = 4 * kMixedSlabs + 1 };

static int plan_slabs_mixed(pd_ctx* c) {
  if (!c->mslab_blk.empty()) return PD_OK;
  const int rs = pipeline_streams(c, std::max<int>(kEvCount, kMEvCount));
  if (rs != PD_OK) return rs;
  const int64_t nb = c->halo.nblocks;
  std::vector<int64_t> h(5 * (size_t)nb);
  int64_t* d = nullptr;
  PD_CK(c, cudaMalloc(&d, h.size() * sizeof(int64_t)));
  pd::launch_block_reach_mixed(mixed_args(c), d, d + nb, d + 2 * nb, d + 3 * nb, d + 4 * nb, c->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = copy_sync(h.data(), d, h.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
  cudaFree(d);
  PD_CK(c, e);
  const int64_t *lo = h.data(), *hi = lo + nb, *idlo = hi + nb, *idhi = idlo + nb, *cf = idhi + nb;
  // visiting blocks hold ascending runs of chunks: the block of a SELL position is the last
  // block whose first chunk is at or below the position's chunk
  std::vector<int64_t> first((size_t)nb);
  for (int64_t b = 0; b < nb; ++b) first[b] = cf[b] >= 0 ? cf[b] : (b ? first[b - 1] : 0);
  auto block_of_pos = [&](int64_t p) {
    const auto it = std::upper_bound(first.begin(), first.end(), p / 32);
    return (int64_t)(it == first.begin() ? 0 : (it - first.begin()) - 1);
  };
  // even slabs of visiting blocks (a plate of fewer blocks than slabs leaves some empty)
  const int K = kMixedSlabs;
  std::vector<int64_t> bc(K + 1);
  for (int k = 0; k <= K; ++k) bc[k] = nb * k / K;
  auto slab_of_block = [&](int64_t blk) {
    int k = 0;
    while (k + 1 < K && blk >= bc[k + 1]) ++k;
    return k;
  };
  c->mslab_lo.assign(K, 0);
  c->mslab_hi.assign(K, 0);
  std::vector<int64_t> smax(K, -1);  // the highest particle id held by slab k
  for (int k = 0; k < K; ++k) {
    int l = k, u = k;
    for (int64_t b = bc[k]; b < bc[k + 1]; ++b) {
      if (lo[b] >= 0) {
        l = std::min(l, slab_of_block(block_of_pos(lo[b])));
        u = std::max(u, slab_of_block(block_of_pos(hi[b])));
      }
      if (idlo[b] >= 0) smax[k] = std::max(smax[k], idhi[b]);
    }
    c->mslab_lo[k] = l;
    c->mslab_hi[k] = u;
  }
  // id slab k ends after the highest id of slabs 0 .. k
  c->mslab_id.assign(K + 1, 0);
  for (int k = 0; k < K; ++k) c->mslab_id[k + 1] = std::max(c->mslab_id[k], smax[k] + 1);
  c->mslab_id[K] = c->n;
  c->mslab_blk = bc;
  return PD_OK;
}

static pd::MixedArgs mixed_slab(const pd_ctx* c, pd::MixedArgs a, int k) {
  a.blk0 = c->mslab_blk[k];
  a.nblocks = c->mslab_blk[k + 1];
  return a;
}

static cudaError_t enqueue_host_step_mixed(pd_ctx* c, int32_t nsteps, const double* u_in, const double* v_in,
                                           const double* f_in, double* u_out, double* v_out, double* f_out,
                                           bool brk) {
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  cudaStream_t s = c->stream;
  cudaEvent_t* ev = c->slab_ev.data();
  cudaStream_t* io = c->io;
  const int K = kMixedSlabs;
  const size_t b16 = sizeof(double2);
  pd::MixedArgs plain = mixed_args(c), out = plain;
  // the exporting pass B writes the new FP64 state straight to the (page-locked) output buffers
  out.out_u = static_cast<double2*>(mapped_host(u_out));
  out.out_v = static_cast<double2*>(mapped_host(v_out));
  out.out_f = static_cast<double2*>(mapped_host(f_out));
  ck(cudaEventRecord(ev[kMEvStart], s));
  for (int q = 0; q < 6; ++q) ck(cudaStreamWaitEvent(io[q], ev[kMEvStart], 0));
  cudaStream_t* pa = c->ps.data();           // pass A of slab k: pa[k]
  cudaStream_t* pb = c->ps.data() + kMaxSlabs;  // pass B of slab k: pb[k]
  const bool one = nsteps == 1;
  int next_a = 0, next_b = 0;
  for (int k = 0; k < K; ++k) {  // enqueued in dependency order
    const size_t off = (size_t)c->mslab_id[k], cnt = (size_t)(c->mslab_id[k + 1] - off);
    if (cnt > 0) {
      ck(cudaMemcpyAsync(c->u + off, u_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice, io[1]));
      ck(cudaMemcpyAsync(c->v + off, v_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice, io[1]));
      ck(cudaMemcpyAsync(c->f + off, f_in + 2 * off, cnt * b16, cudaMemcpyHostToDevice, io[1]));
    }
    ck(cudaEventRecord(ev[kMEvIn + k], io[1]));
    ck(cudaStreamWaitEvent(io[0], ev[kMEvIn + k], 0));
    pd::launch_import_drift_mixed(plain, c->mslab_blk[k], c->mslab_blk[k + 1], c->u, c->v, c->f, io[0]);
    ck(cudaEventRecord(ev[kMEvImport + k], io[0]));
    for (; next_a < K && c->mslab_hi[next_a] <= k; ++next_a) {
      cudaStream_t sa = pa[next_a];
      ck(cudaStreamWaitEvent(sa, ev[kMEvImport + c->mslab_hi[next_a]], 0));
      pd::launch_slab_pass_a_mixed(mixed_slab(c, plain, next_a), brk, sa);
      ck(cudaEventRecord(ev[kMEvA + next_a], sa));
      for (; one && next_b < next_a && c->mslab_hi[next_b] < next_a; ++next_b) {
        cudaStream_t sb = pb[next_b];
        for (int q = c->mslab_lo[next_b]; q <= c->mslab_hi[next_b]; ++q) ck(cudaStreamWaitEvent(sb, ev[kMEvA + q], 0));
        pd::launch_slab_pass_b_mixed(mixed_slab(c, out, next_b), true, sb);
        ck(cudaEventRecord(ev[kMEvB + next_b], sb));
      }
    }
  }
  for (; one && next_b < K;) {
    cudaStream_t sb = pb[next_b];
    for (int q = c->mslab_lo[next_b]; q <= c->mslab_hi[next_b]; ++q) ck(cudaStreamWaitEvent(sb, ev[kMEvA + q], 0));
    pd::launch_slab_pass_b_mixed(mixed_slab(c, out, next_b), true, sb);
    ck(cudaEventRecord(ev[kMEvB + next_b], sb));
    ++next_b;
  }
  // join every stream's work on the main stream
  auto join = [&](cudaStream_t q) {
    ck(cudaEventRecord(ev[kMEvStart], q));
    ck(cudaStreamWaitEvent(s, ev[kMEvStart], 0));
  };
  for (int q = 0; q < 6; ++q) join(io[q]);
  for (int k = 0; k < K; ++k) join(pa[k]);
  for (int k = 0; one && k < K; ++k) join(pb[k]);
  if (!one) {  // the remaining steps on the whole plate; the last pass B exports
    pd::launch_slab_pass_b_mixed(plain, false, s);  // (plain launch: it follows the join's event waits)
    for (int32_t k = 1; k < nsteps; ++k) {
      pd::launch_pass_a_mixed(plain, brk, s);
      if (k + 1 < nsteps)
        pd::launch_pass_b_mixed(plain, true, s);
      else
        pd::launch_slab_pass_b_mixed(out, true, s);
    }
  }
  ck(cudaGetLastError());
  return e;
}

int pd_step_host(pd_ctx* c, int32_t nsteps, const double* u_in, const double* v_in, const double* f_in, double* u_out,
                 double* v_out, double* f_out) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  if (nsteps < 1) return fail(c, PD_ERR_ARG, "pd_step_host: nsteps >= 1");
  if (!u_in || !v_in || !f_in || !u_out || !v_out || !f_out) return fail(c, PD_ERR_ARG, "pd_step_host: NULL buffer");
  if (c->n == 0) return PD_OK;
  PD_CK(c, cudaSetDevice(c->p.device));
  if (mixed(c)) {
    if (!mapped_host(u_in) || !mapped_host(v_in) || !mapped_host(f_in) || !mapped_host(u_out) ||
        !mapped_host(v_out) || !mapped_host(f_out))
      return fail(c, PD_ERR_ARG, "pd_step_host: buffers must be page-locked host memory (pd_host_alloc)");
    const int rp = plan_slabs_mixed(c);
    if (rp != PD_OK) return rp;
    PD_CK(c, enqueue_host_step_mixed(c, nsteps, u_in, v_in, f_in, u_out, v_out, f_out, c->p.s_c > 0.0));
    PD_CK(c, cudaGetLastError());
    PD_CK(c, cudaStreamSynchronize(c->stream));
    c->steps += nsteps;
    return check_after_step(c);
  }
  Fp64Args in = fp64_args(c), out = fp64_args(c);
  in.in_u = static_cast<const double2*>(mapped_host(u_in));
  in.in_v = static_cast<const double2*>(mapped_host(v_in));
  in.in_f = static_cast<const double2*>(mapped_host(f_in));
  out.out_u = static_cast<double2*>(mapped_host(u_out));
  out.out_v = static_cast<double2*>(mapped_host(v_out));
  out.out_f = static_cast<double2*>(mapped_host(f_out));
  if (!in.in_u || !in.in_v || !in.in_f || !out.out_u || !out.out_v || !out.out_f)
    return fail(c, PD_ERR_ARG, "pd_step_host: buffers must be page-locked host memory (pd_host_alloc)");
  cudaStream_t s = c->stream;
  const Fp64Args plain = fp64_args(c);
  const bool brk = c->p.s_c > 0.0;
  if (bond_assoc(c)) {  // one stream: the state is read and written by the kernels over the CPU-GPU link
    pd::launch_drift_fp64(in, s);
    for (int32_t k = 0; k < nsteps; ++k) {
      const bool last = k + 1 == nsteps;
      pd::launch_ba_pass_a(plain, ba_args(c), s);
      pd::launch_ba_pass_b(last ? out : plain, ba_args(c), last ? 0 : 1, s);
    }
  } else {
    const int rp = plan_slabs(c);
    if (rp != PD_OK) return rp;
    PD_CK(c, enqueue_host_step(c, nsteps, u_in, v_in, f_in, plain, out, brk));
  }
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaStreamSynchronize(s));
  c->steps += nsteps;
  return check_after_step(c);
}

int pd_synchronize(pd_ctx* c) {
  if (!c) return PD_ERR_ARG;
  PD_CK(c, cudaSetDevice(c->p.device));
  PD_CK(c, cudaStreamSynchronize(c->stream));
  if (!c->counters) return PD_OK;
  unsigned long long err = 0;
  PD_CK(c, copy_sync(&err, c->counters + pd::CNT_ERROR, sizeof(err), cudaMemcpyDeviceToHost, c->stream));
  if (err & pd::ERR_STAGE_TIMEOUT) return fail(c, PD_ERR_TIMEOUT, "a bounded wait for a staged bond-index copy gave up");
  return PD_OK;
}

int pd_compute_velocity(pd_ctx* c, const double* u, double* velocity, double* acce, double* netF) {
  if (!c) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  if (!u || !velocity || !acce || !netF) return fail(c, PD_ERR_ARG, "NULL buffer");
  if (mixed(c)) return fail(c, PD_ERR_ARG, "pd_compute_velocity is the FP64 drop-in; create the context with PD_FP64");
  if (c->n == 0) return PD_OK;
  PD_CK(c, cudaSetDevice(c->p.device));
  const size_t b = (size_t)c->n * sizeof(double2);
  cudaStream_t s = c->stream;
  if (!bond_assoc(c) && mapped_host(u) && mapped_host(velocity) && mapped_host(acce) && mapped_host(netF)) {
    // page-locked buffers (pd_host_alloc): pd_step_host's slab pipeline, the
    // copies in overlapping pass A and each slab's pass B writing its results
    // back while later slabs compute; the same results as the staged call
    const int rp = plan_slabs(c);
    if (rp != PD_OK) return rp;
    Fp64Args out = fp64_args(c);
    out.out_v = static_cast<double2*>(mapped_host(velocity));
    out.out_a = static_cast<double2*>(mapped_host(acce));
    out.out_f = static_cast<double2*>(mapped_host(netF));
    PD_CK(c, enqueue_host_step(c, 1, u, velocity, acce, fp64_args(c), out, c->p.s_c > 0.0, true));
    PD_CK(c, cudaGetLastError());
    PD_CK(c, cudaStreamSynchronize(s));
    c->steps += 1;
    return check_after_step(c);
  }
  PD_CK(c, cudaMemcpyAsync(c->u, u, b, cudaMemcpyHostToDevice, s));
  PD_CK(c, cudaMemcpyAsync(c->v, velocity, b, cudaMemcpyHostToDevice, s));
  PD_CK(c, cudaMemcpyAsync(c->acc, acce, b, cudaMemcpyHostToDevice, s));
  const Fp64Args a = fp64_args(c);
  if (bond_assoc(c)) {
    pd::launch_ba_pass_a(a, ba_args(c), s);
    pd::launch_ba_pass_b(a, ba_args(c), 2, s);
  } else {
    pd::launch_shadow_fp64(a, s);
    pd::launch_pass_a_fp64(a, c->p.s_c > 0.0, s);
    pd::launch_pass_b_fp64(a, 2, s);
  }
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaMemcpyAsync(velocity, c->v, b, cudaMemcpyDeviceToHost, s));
  PD_CK(c, cudaMemcpyAsync(acce, c->acc, b, cudaMemcpyDeviceToHost, s));
  PD_CK(c, cudaMemcpyAsync(netF, c->f, b, cudaMemcpyDeviceToHost, s));
  PD_CK(c, cudaStreamSynchronize(s));
  c->steps += 1;
  return check_after_step(c);
}

int pd_step_timed(pd_ctx* c, int32_t nsteps, float* ms) {
  if (!c || !ms) return PD_ERR_ARG;
  PD_CK(c, cudaSetDevice(c->p.device));
  cudaEvent_t e0, e1;
  PD_CK(c, cudaEventCreate(&e0));
  PD_CK(c, cudaEventCreate(&e1));
  PD_CK(c, cudaEventRecord(e0, c->stream));
  int rc = pd_step(c, nsteps);
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int pd_profile_steps(pd_ctx* c, int32_t nsteps, double* ms, int64_t* launches) {
  if (!c || !ms || !launches) return PD_ERR_ARG;
  if (!c->has_families) return fail(c, PD_ERR_ORDER, "families first");
  PD_CK(c, cudaSetDevice(c->p.device));
  for (int k = 0; k < PD_NUM_KERNELS; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  if (nsteps <= 0 || c->n == 0) return PD_OK;
  const int nev = 2 * (1 + 2 * nsteps);
  std::vector<cudaEvent_t> ev(nev);
  for (auto& e : ev) PD_CK(c, cudaEventCreate(&e));
  std::vector<int> kind;
  Launcher L(c);
  cudaStream_t s = c->stream;
  int q = 0;
  cudaEventRecord(ev[q++], s);
  L.drift(s);
  cudaEventRecord(ev[q++], s);
  kind.push_back(PD_KERNEL_DRIFT);
  for (int32_t k = 0; k < nsteps; ++k) {
    cudaEventRecord(ev[q++], s);
    L.pass_a(s);
    cudaEventRecord(ev[q++], s);
    kind.push_back(PD_KERNEL_PASS_A);
    cudaEventRecord(ev[q++], s);
    L.pass_b(k + 1 < nsteps, s);
    cudaEventRecord(ev[q++], s);
    kind.push_back(PD_KERNEL_PASS_B);
  }
  PD_CK(c, cudaGetLastError());
  PD_CK(c, cudaStreamSynchronize(s));
  for (size_t k = 0; k < kind.size(); ++k) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]);
    ms[kind[k]] += t;
    launches[kind[k]] += 1;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  c->steps += nsteps;
  return check_after_step(c);
}

int pd_host_alloc(int64_t bytes, void** p) {
  if (!p || bytes < 0) return PD_ERR_ARG;
  *p = nullptr;
  if (cudaMallocHost(p, (size_t)(bytes > 0 ? bytes : 1)) != cudaSuccess) return PD_ERR_CUDA;
  return PD_OK;
}

int pd_host_free(void* p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return PD_ERR_CUDA;
  return PD_OK;
}

int pd_model_bytes(const pd_ctx* c, double* bytes) {
  if (!c || !bytes) return PD_ERR_ARG;
  const double per_particle = c->p.precision == PD_FP64 ? 248.0 : 148.0;
  *bytes = per_particle * (double)c->n + 11.0 * (double)c->nnz;
  return PD_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batches

namespace {

int bfail(pd_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}

#define PD_BCK(b, call)                                                          \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) return bfail(b, PD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int batch_refresh(pd_batch* b) {
  if (!b->dirty) return PD_OK;
  std::vector<pd::BatchTile> tiles;
  std::vector<unsigned char> plates;
  const size_t asz = b->precision == PD_MIXED ? sizeof(pd::MixedArgs) : sizeof(Fp64Args);
  plates.resize(asz * (b->members.empty() ? 1 : b->members.size()));
  b->particles = 0;
  b->bonds = 0;
  b->smem_a = b->smem_b = 0;
  for (size_t k = 0; k < b->members.size(); ++k) {
    pd_ctx* c = b->members[k];
    if (!c->has_families) return bfail(b, PD_ERR_ORDER, "a member has no families");
    if (b->precision == PD_MIXED) {
      const pd::MixedArgs m = mixed_args(c);
      std::memcpy(plates.data() + k * asz, &m, asz);
      b->smem_a = std::max(b->smem_a, pd::mixed_pass_smem(m, true));
      b->smem_b = std::max(b->smem_b, pd::mixed_pass_smem(m, false));
      // one tile per visiting block (one spatial tile of up to kHaloBlock particles) of the plate
      for (int64_t blk = 0; blk < c->halo.nblocks; ++blk)
        tiles.push_back(pd::BatchTile{(int32_t)k, pd::kHaloBlock, blk});
    } else {
      const Fp64Args f = fp64_args(c);
      std::memcpy(plates.data() + k * asz, &f, asz);
      for (int64_t first = 0; first < c->n; first += b->tile)
        tiles.push_back(pd::BatchTile{(int32_t)k, (int32_t)std::min<int64_t>(b->tile, c->n - first), first});
    }
    b->particles += c->n;
    b->bonds += c->nnz;
  }
  if (plates.size() > b->plates_bytes) {
    if (b->d_plates) cudaFree(b->d_plates);
    b->d_plates = nullptr;
    PD_BCK(b, cudaMalloc(&b->d_plates, plates.size()));
    b->plates_bytes = plates.size();
  }
  if (tiles.size() > b->tiles_cap || !b->d_tiles) {
    if (b->d_tiles) cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    const size_t cap = std::max<size_t>(tiles.size(), 1);
    PD_BCK(b, cudaMalloc(&b->d_tiles, cap * sizeof(pd::BatchTile)));
    b->tiles_cap = cap;
  }
  PD_BCK(b, cudaMemcpyAsync(b->d_plates, plates.data(), plates.size(), cudaMemcpyHostToDevice, b->stream));
  if (!tiles.empty())
    PD_BCK(b, cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(pd::BatchTile), cudaMemcpyHostToDevice,
                              b->stream));
  PD_BCK(b, cudaStreamSynchronize(b->stream));
  b->ntiles = (int)tiles.size();
  clear_batch_graphs(b);
  b->dirty = false;
  return PD_OK;
}

cudaError_t batch_enqueue(pd_batch* b, int32_t nsteps) {
  if (b->precision == PD_MIXED)
    return pd::launch_batch_mixed(static_cast<const pd::MixedArgs*>(b->d_plates), b->d_tiles, b->ntiles, nsteps,
                                  b->cfg, b->smem_a, b->smem_b, b->d_bar, b->nsm, b->stream);
  return pd::launch_batch_fp64(static_cast<const Fp64Args*>(b->d_plates), b->d_tiles, b->ntiles, nsteps, b->cfg,
                               b->d_bar, b->nsm, b->stream);
}

// The graph of nsteps steps of the persistent kernel (persistent == 1) or the phase kernels
// (0), captured on first use.  A runtime that refuses to capture the cooperative launch
// leaves b->direct set and no graph: the kernel is then launched directly.
int batch_graph(pd_batch* b, int32_t nsteps) {
  if ((b->cfg.persistent && b->direct) || b->graphs.count(nsteps)) return PD_OK;
  cudaGraph_t g;
  PD_BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const cudaError_t le = batch_enqueue(b, nsteps);
  const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (ce == cudaSuccess) cudaGraphDestroy(g);
    cudaGetLastError();
    if (!b->cfg.persistent)
      return bfail(b, PD_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
    b->direct = true;
    return PD_OK;
  }
  cudaGraphExec_t ge;
  const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return bfail(b, PD_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ie));
  if (b->graphs.size() > 16) clear_batch_graphs(b);
  b->graphs.emplace(nsteps, ge);
  return PD_OK;
}

// persistent == 2: every member runs its own step graph (pd_step's: the single-plate kernels,
// arguments in parameter space, programmatic launches between its passes) on its own stream,
// forked from and joined back to the batch stream, so the plates meet only at the call's end.
// launch = false captures the members' graphs only.
int batch_step_members(pd_batch* b, int32_t nsteps, bool launch) {
  std::vector<cudaGraphExec_t> ge(b->members.size(), nullptr);
  for (size_t k = 0; k < b->members.size(); ++k) {
    pd_ctx* c = b->members[k];
    if (c->n > 0 && step_graph(c, nsteps, &ge[k]) != PD_OK) return bfail(b, PD_ERR_CUDA, c->err);
  }
  if (!launch) return PD_OK;
  PD_BCK(b, cudaEventRecord(b->done, b->stream));
  for (size_t k = 0; k < b->members.size(); ++k) {
    if (!ge[k]) continue;
    cudaStream_t cs = b->members[k]->stream;
    PD_BCK(b, cudaStreamWaitEvent(cs, b->done, 0));
    PD_BCK(b, cudaGraphLaunch(ge[k], cs));
    PD_BCK(b, cudaEventRecord(b->join, cs));
    PD_BCK(b, cudaStreamWaitEvent(b->stream, b->join, 0));
  }
  return PD_OK;
}

}  // namespace

extern "C" {

int pd_batch_create(int32_t device, int32_t precision, pd_batch** out) {
  if (!out) return PD_ERR_ARG;
  *out = nullptr;
  if (precision != PD_FP64 && precision != PD_MIXED) {
    g_create_err = "pd_batch_create: unknown precision";
    return PD_ERR_ARG;
  }
  std::unique_ptr<pd_batch> b(new (std::nothrow) pd_batch());
  if (!b) return PD_ERR_CAPACITY;
  b->device = device;
  b->precision = precision;
  // every member's own step graph, concurrently (256-plate batch, ms per step: mixed 1.40 against
  // 1.79 for the phase kernels and 1.89 for the persistent kernel; FP64 10.6 against 11.4 / 11.5)
  b->cfg.persistent = 2;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bar, sizeof(pd::GridBarrier));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_bar, 0, sizeof(pd::GridBarrier), b->stream);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    g_create_err = std::string("pd_batch_create: ") + cudaGetErrorString(e);
    pd_batch_destroy(b.release());
    return PD_ERR_CUDA;
  }
  *out = b.release();
  return PD_OK;
}

int pd_batch_destroy(pd_batch* b) {
  if (!b) return PD_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (pd_ctx* c : b->members) c->batch = nullptr;
  clear_batch_graphs(b);
  if (b->d_plates) cudaFree(b->d_plates);
  if (b->d_tiles) cudaFree(b->d_tiles);
  if (b->d_bar) cudaFree(b->d_bar);
  if (b->done) cudaEventDestroy(b->done);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->join) cudaEventDestroy(b->join);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PD_OK;
}

const char* pd_batch_last_error(const pd_batch* b) { return b ? b->err.c_str() : g_create_err.c_str(); }

int pd_batch_add(pd_batch* b, pd_ctx* c) {
  if (!b || !c) return PD_ERR_ARG;
  if (c->batch) return bfail(b, PD_ERR_ARG, "the context is already in a batch");
  if (c->p.device != b->device || c->p.precision != b->precision)
    return bfail(b, PD_ERR_ARG, "batch members share the batch's device and precision");
  if (!c->has_families) return bfail(b, PD_ERR_ORDER, "set particles and families before adding a context");
  if (bond_assoc(c)) return bfail(b, PD_ERR_ARG, "bond-associated contexts are stepped on their own");
  PD_BCK(b, cudaSetDevice(b->device));
  PD_BCK(b, cudaStreamSynchronize(b->stream));
  b->members.push_back(c);
  c->batch = b;
  b->dirty = true;
  clear_batch_graphs(b);
  return PD_OK;
}

int pd_batch_remove(pd_batch* b, pd_ctx* c) {
  if (!b || !c) return PD_ERR_ARG;
  auto it = std::find(b->members.begin(), b->members.end(), c);
  if (it == b->members.end()) return bfail(b, PD_ERR_ARG, "not a member");
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  b->members.erase(it);
  c->batch = nullptr;
  b->dirty = true;
  clear_batch_graphs(b);
  return PD_OK;
}

int pd_batch_info(const pd_batch* b, int32_t* nplates, int64_t* particles, int64_t* bonds) {
  if (!b) return PD_ERR_ARG;
  int64_t np = 0, nb = 0;
  for (const pd_ctx* c : b->members) {
    np += c->n;
    nb += c->nnz;
  }
  if (nplates) *nplates = (int32_t)b->members.size();
  if (particles) *particles = np;
  if (bonds) *bonds = nb;
  return PD_OK;
}

int pd_batch_set_barrier_limits(pd_batch* b, uint64_t spin_limit, uint32_t hold_ns) {
  if (!b) return PD_ERR_ARG;
  if (hold_ns > pd::kBarrierHoldMaxNs) return bfail(b, PD_ERR_ARG, "hold_ns above 100 ms");
  PD_BCK(b, cudaSetDevice(b->device));
  PD_BCK(b, cudaStreamSynchronize(b->stream));
  b->cfg.limits.spins = spin_limit;
  b->cfg.limits.hold_ns = hold_ns;
  clear_batch_graphs(b);  // the limits are launch arguments
  return PD_OK;
}

int pd_batch_set_config(pd_batch* b, const pd_batch_config* cfg) {
  if (!b || !cfg) return PD_ERR_ARG;
  if (cfg->block < 32 || cfg->block > 256 || cfg->block % 32 || cfg->tile < 32 || cfg->tile % 32 ||
      cfg->blocks_per_sm < 1 || cfg->persistent < 0 || cfg->persistent > 2)
    return bfail(b, PD_ERR_ARG, "invalid batch configuration");
  PD_BCK(b, cudaSetDevice(b->device));
  PD_BCK(b, cudaStreamSynchronize(b->stream));
  b->cfg.block = cfg->block;
  b->cfg.blocks_per_sm = cfg->blocks_per_sm;
  b->cfg.persistent = cfg->persistent;
  if (cfg->tile != b->tile) b->dirty = true;
  b->tile = cfg->tile;
  clear_batch_graphs(b);
  return PD_OK;
}

int pd_batch_get_config(const pd_batch* b, pd_batch_config* cfg) {
  if (!b || !cfg) return PD_ERR_ARG;
  cfg->block = b->cfg.block;
  cfg->blocks_per_sm = b->cfg.blocks_per_sm;
  cfg->persistent = b->cfg.persistent;
  cfg->tile = b->tile;
  return PD_OK;
}

int pd_batch_step(pd_batch* b, int32_t nsteps) {
  if (!b) return PD_ERR_ARG;
  if (nsteps < 0) return bfail(b, PD_ERR_ARG, "nsteps < 0");
  if (nsteps == 0 || b->members.empty()) return PD_OK;
  PD_BCK(b, cudaSetDevice(b->device));
  int rc = batch_refresh(b);
  if (rc != PD_OK) return rc;
  // order after every member's pending work
  for (pd_ctx* c : b->members) {
    PD_BCK(b, cudaEventRecord(b->done, c->stream));
    PD_BCK(b, cudaStreamWaitEvent(b->stream, b->done, 0));
  }
  // graphs first (host work), so that t0 .. t1 is the GPU's
  rc = b->cfg.persistent == 2 ? batch_step_members(b, nsteps, false) : batch_graph(b, nsteps);
  if (rc != PD_OK) return rc;
  PD_BCK(b, cudaEventRecord(b->t0, b->stream));
  if (b->cfg.persistent == 2) {
    rc = batch_step_members(b, nsteps, true);
    if (rc != PD_OK) return rc;
  } else {
    if (b->cfg.persistent && b->direct)
      PD_BCK(b, batch_enqueue(b, nsteps));
    else
      PD_BCK(b, cudaGraphLaunch(b->graphs.at(nsteps), b->stream));
  }
  PD_BCK(b, cudaEventRecord(b->t1, b->stream));
  PD_BCK(b, cudaEventRecord(b->done, b->stream));
  for (pd_ctx* c : b->members) {
    PD_BCK(b, cudaStreamWaitEvent(c->stream, b->done, 0));
    c->steps += nsteps;
  }
  return PD_OK;
}

int pd_batch_last_step_ms(pd_batch* b, float* ms) {
  if (!b || !ms) return PD_ERR_ARG;
  *ms = 0.f;
  PD_BCK(b, cudaSetDevice(b->device));
  PD_BCK(b, cudaEventSynchronize(b->t1));
  PD_BCK(b, cudaEventElapsedTime(ms, b->t0, b->t1));
  return PD_OK;
}

int pd_batch_synchronize(pd_batch* b) {
  if (!b) return PD_ERR_ARG;
  PD_BCK(b, cudaSetDevice(b->device));
  PD_BCK(b, cudaStreamSynchronize(b->stream));
  pd::GridBarrier h;
  PD_BCK(b, copy_sync(&h, b->d_bar, sizeof(h), cudaMemcpyDeviceToHost, b->stream));
  if (h.err) return bfail(b, PD_ERR_TIMEOUT, "a grid-barrier wait of the persistent batch kernel gave up");
  return PD_OK;
}

int pd_batch_step_timed(pd_batch* b, int32_t nsteps, float* ms) {
  if (!b || !ms) return PD_ERR_ARG;
  PD_BCK(b, cudaSetDevice(b->device));
  int rc = batch_refresh(b);
  if (rc != PD_OK) return rc;
  cudaEvent_t e0, e1;
  PD_BCK(b, cudaEventCreate(&e0));
  PD_BCK(b, cudaEventCreate(&e1));
  for (pd_ctx* c : b->members) {
    PD_BCK(b, cudaEventRecord(b->done, c->stream));
    PD_BCK(b, cudaStreamWaitEvent(b->stream, b->done, 0));
  }
  if (nsteps > 0 && !b->members.empty()) {  // graphs captured before the clock starts
    rc = b->cfg.persistent == 2 ? batch_step_members(b, nsteps, false) : batch_graph(b, nsteps);
    if (rc != PD_OK) return rc;
  }
  PD_BCK(b, cudaEventRecord(e0, b->stream));
  rc = pd_batch_step(b, nsteps);
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != PD_OK) return rc;
  return pd_batch_synchronize(b);
}

}  // extern "C"
