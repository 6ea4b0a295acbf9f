// Internal types of the GB300 NOSB library (not installed; see include/pd_gb300.h).
//
// Device data layout (HBM), one context = one plate:
//   per particle (n):  x double2, vol double, u/v/f double2 (FP64 state),
//                      w01/w23 double2 (W = V sigma K^-1, rows), kinv01 double2
//                      + kinv22 double (K^-1), mt double2 (m / V), bc uint8,
//                      broken int32, damage double, singular uint8, fam int32.
//   per bond:          SELL-32 ("sliced ELL", chunk = 32 particles = one
//                      warp, column-major inside a chunk): particle i sits at
//                      SELL position p = pos_of[i] (member[p] = i; the FP64
//                      form uses p = i, the mixed form a tiled spatial order
//                      of the reference positions), and its slot k at
//                      chunk_base[p/32] + 32*k + (p%32), so each bond slot of
//                      a warp is one coalesced 128 B (int) or 512 B (double2)
//                      line.  nbr int32 (j, -1 padding,
//                      -2-j broken), bxi double2 (xi = x_j - x_i), bgeo double2
//                      (V_j xi), blim double (((1+s_c)^2-1) |xi|^2).
//   Precomputing the bond geometry trades HBM bytes for FP64 operations: on
//   GB300 one FP64 operation costs as much time as ~12 bytes of HBM traffic.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "pd_batch.cuh"
#include "pd_gb300.h"

namespace pd {

constexpr int kChunk = 32;
constexpr int kBlock = 256;

// SELL position of particle i and particle at position p (null maps: identity).
__host__ __device__ __forceinline__ int64_t sell_pos(const int32_t* pos_of, int64_t i) {
  return pos_of ? (int64_t)pos_of[i] : i;
}
__host__ __device__ __forceinline__ int64_t sell_member(const int32_t* member, int64_t p) {
  return member ? (int64_t)member[p] : p;
}
// First slot (k = 0) of the particle at SELL position p.
__host__ __device__ __forceinline__ int64_t sell_slot0(const int64_t* chunk_base, int64_t p) {
  return chunk_base[p >> 5] + (p & 31);
}
// Threads (= particles) of one visiting block of the mixed single-plate and
// batched passes: kHaloBlock consecutive SELL positions (a 32 x 8 tile of
// the reference positions) share a halo.
constexpr int kHaloBlock = 256;
// Halo staging of the mixed passes: a block stages at most kHaloCap
// distinct particles (a power of two).
constexpr int kHaloCap = 2048;

// Counters word layout (device int64 array).
enum { CNT_BROKEN = 0, CNT_SINGULAR = 1, CNT_ERROR = 2, CNT_N = 4 };
// Device error bits (CNT_ERROR).
enum { ERR_FAMILY_OVERFLOW = 1, ERR_BAD_NEIGHBOR = 2, ERR_SELF_BOND = 4, ERR_ASYMMETRIC = 8, ERR_STAGE_TIMEOUT = 16 };

struct Fp64Args {
  int64_t n;
  int64_t i0;  // drift and the passes run particles i0 <= i < n (a slab; 0 for the whole plate)
  const double2* __restrict__ x;
  const double* __restrict__ vol;
  double2* u;
  double2* v;
  double2* f;
  double2* acc;  // drop-in mode only (pd_compute_velocity)
  double2* w01;
  double2* w23;
  double2* kinv01;
  double* kinv22;
  double2* mt;
  const uint8_t* __restrict__ bc;
  const int32_t* __restrict__ gkind;
  const double2* __restrict__ gval;
  int32_t* broken;
  double* damage;
  uint8_t* singular;
  const int32_t* __restrict__ fam;
  const int64_t* __restrict__ chunk_base;
  const int32_t* __restrict__ chunk_w;
  int32_t* nbr;  // the FP64 form's SELL position of particle i is i
  const double2* __restrict__ bxi;
  const double2* __restrict__ bgeo;
  const double* __restrict__ blim;
  const float* __restrict__ br2;  // (s_c |xi|)^2 (1 - 1e-5), rounded toward 0: FP32 stretch certificate
  float2* u32;                    // u rounded to FP32 (shadow for the certificate)
  double2* hg;  // 2 k_hg sum_j V_j (u_j - u_i), pass A -> pass B
  // pd_step_host: the drift takes the state from page-locked host memory
  // (read over the CPU-GPU link by the kernel itself) and the last pass B
  // writes it back there; pd_compute_velocity with page-locked buffers: the
  // import (k_shadow) takes u, velocity, acce (in_a) from there and pass B
  // (mode 2) writes velocity, acce (out_a) and the force back; null otherwise
  const double2* in_u;
  const double2* in_v;
  const double2* in_f;
  const double2* in_a;
  double2* out_u;
  double2* out_v;
  double2* out_f;
  double2* out_a;
  double c11, c12, c33;
  double dt, dt2, inv_rho, det_guard, k_hg, damage_fail;
  unsigned long long* counters;
  int32_t brk;  // bond breaking on (s_c > 0)
  int32_t pad;
};

// Bond-associated mode (pd_bondassoc.cu): weights and per-bond force states.
struct BondAssoc {
  double n1, n2, inv_wlen;
  double2* tb;     // T_ij per bond slot
  int64_t* rslot;  // slot of the reverse bond (j, i)
  double2* lr;     // per bond slot: |xi|, 1 / |xi|
  double2* ex;     // per bond slot: exp(n1 |xi| / l), exp(-n1 |xi| / l) (for the weights n1, l of the call)
  double2* kq0;    // per bond slot: K_b^-1 (q11, q12)
  double2* kq1;    // per bond slot: (q22, 1 if K_b fails the det guard else 0)
  double* wtri;    // per particle with <= 32 bonds: its weight matrix's lower triangle (kBaTri doubles)
};
constexpr int64_t kBaTri = 32 * 33 / 2;

// Mazars damage (pd_mazars.cu): law constants and per-slot history.
struct MazarsArgs {
  double kappa0, a_t, b_t, a_c, b_c;
  double* thr;     // per SELL slot: history threshold
  double* bd;      // per SELL slot: bond damage
  double* status;  // per particle: sum of bond damage / family size
};

// Chunk a warp runs in the mixed passes: warp w of visiting block b runs
// visit[b * kHaloBlock / 32 + w].
struct alignas(16) VisitRec {
  int32_t chunk;    // chunk id (-1: the warp has none)
  int16_t w, live;  // width (slot rows); lanes 0 .. live-1 hold particles (the rest are holes)
  int64_t base;     // first slot
};

// Mixed form (pd_mixed.cu): scaled two-float state, FP32 bond arithmetic.
// The scaled state (xs .. hgs), bc, singular and self_loc are stored in SELL
// position order (npos entries; holes hold zeros): a warp's per-particle
// loads are coalesced and halo gathers follow space whatever the particle
// numbering.  x, vol, broken, damage and fam are per particle (i = member[p]).
struct MixedArgs {
  int64_t n, npos;
  const double2* __restrict__ x;    // FP64 reference positions (K^-1 recompute)
  const double* __restrict__ vol;   // FP64 volumes
  float4* xs;                       // x^ two-float {hi.x, hi.y, lo.x, lo.y}
  float* vh;                        // V^
  float4* us;                       // u^ two-float
  float4* vs;                       // v^ = v dt / Ls, two-float
  float2* fs;                       // f^ = f Ls / Es
  float4* ws;                       // W^ = V^ sigma^ K^-1 (row-major 2x2)
  float4* geo;                      // {K^-1 11, 12, 22, V^_i}
  float2* mh;                       // m^ / V^_i
  float2* hgs;                      // 2 k^ sum_j V^_j du^ (pass A -> pass B)
  const uint8_t* __restrict__ bc;   // BC group by position
  const int32_t* __restrict__ gkind;
  const float4* __restrict__ gvel;  // prescribed v^ per group, two-float
  int32_t* broken;
  double* damage;
  uint8_t* singular;                // by position
  const int32_t* __restrict__ fam;
  const int64_t* __restrict__ chunk_base;
  const int32_t* __restrict__ chunk_w;
  int32_t* nbr;                             // particle ids (the FP64 form's encoding)
  const int32_t* __restrict__ member;       // SELL position -> particle (-1: a hole)
  const int32_t* __restrict__ pos_of;       // particle -> SELL position
  const VisitRec* __restrict__ visit;       // per warp of each visiting block: its chunk
  int64_t nblocks;                          // visiting blocks (kHaloBlock threads, one tile each)
  uint16_t* loc;                            // per slot: position in the block's halo (padding / broken: the
                                            // particle's own position, whose data adds exact zeros)
  const uint16_t* __restrict__ self_loc;    // per position: the particle's own entry in its block's halo
  const int32_t* __restrict__ halo;         // per block: SELL positions of its halo (halo_cap entries per block)
  const int32_t* __restrict__ halo_n;       // per block: halo size, -1 = not staged
  int32_t halo_cap, halo_max;               // halo_max: largest halo (multiple of 8), sizes shared memory
  float c11, c12, c33;  // C / Es
  float s2, tau2;       // stretch limit factor, Es dt^2 / (rho Ls^2)
  float k_hg;           // k Vs Ls^2 / Es
  double inv_ls, inv_vs, v_scale, f_scale, det_guard, damage_fail;
  double ls, v_unscale, f_unscale;  // 1 / inv_ls, 1 / v_scale, 1 / f_scale: the FP64 state out by products
  unsigned long long* counters;
  int32_t brk;  // bond breaking on (s_c > 0)
  int32_t wmax;  // widest SELL chunk (slot rows), sizes the staged passes' shared memory
  // pd_step_host: a pass launch covers visiting blocks blk0 .. nblocks - 1 (0: all), and
  // the exporting pass B writes the new FP64 state by particle id to these (host-mapped)
  double2* out_u;
  double2* out_v;
  double2* out_f;
  int64_t blk0;
  int32_t uniform_v;  // every particle's V^ is exactly 1 (pass A leaves the V^ gathers out)
};

// ---- family build (pd_family.cu)
struct FamilyBuild {
  int64_t nnz = 0;
  int64_t* row_ptr = nullptr;  // device, n+1
  int32_t* col = nullptr;      // device, nnz
};
// GPU cell list -> CSR.  Returns PD_OK or an error code with msg set.
int build_families_gpu(int64_t n, const double2* d_x, const double* h_x, double cutoff, int n_cracks,
                       const double* h_cracks, cudaStream_t s, FamilyBuild* out, std::string* msg);
// SELL-32 layout of a CSR family (+ FP64 bond geometry).  d_* are device pointers.
struct SellLayout {
  int64_t npos = 0;  // SELL positions: n, or more when member leaves holes (-1 entries)
  int64_t nchunks = 0, nslots = 0;
  int64_t* chunk_base = nullptr;
  int32_t* chunk_w = nullptr;
  int32_t* nbr = nullptr;
  int32_t* member = nullptr;  // SELL position -> particle, -1 = hole (set with npos before build_sell)
  int32_t* pos_of = nullptr;  // particle -> SELL position
  // null: a particle's slots follow its family order (the reference's summation
  // order); else in ascending rk[j] of the neighbours (set before build_sell)
  uint64_t* rk = nullptr;
};
// Spatial layout of the mixed form (pd_order.cu): sets L->member, pos_of, rk
// and npos; *d_blocks (device, caller frees) = *nblocks x (kHaloBlock / 32)
// chunk ids (-1: none) of the visiting blocks.  h_x: the positions on the host.
int build_spatial_order(int64_t n, const double2* d_x, const double* h_x, cudaStream_t s, SellLayout* L,
                        int32_t** d_blocks, int64_t* nblocks, std::string* msg);
int build_sell(int64_t n, const int64_t* d_row_ptr, const int32_t* d_col, cudaStream_t s, SellLayout* out,
               unsigned long long* d_counters, std::string* msg);
void launch_bond_geometry_fp64(int64_t n, const double2* x, const double* vol, const SellLayout& L,
                               const int64_t* row_ptr, double s_c, double2* bxi, double2* bgeo, double* blim,
                               float* br2, cudaStream_t s);
void launch_bond_limit_fp64(int64_t nslots, const double2* bxi, double s_c, const int32_t* nbr, double* blim,
                            float* br2, cudaStream_t s);
void launch_mask_out(int64_t n, const int64_t* row_ptr, const int32_t* col, const SellLayout& L, uint8_t* alive,
                     cudaStream_t s);
void launch_sell_reset(int64_t n, const int64_t* row_ptr, const int32_t* col, const SellLayout& L, cudaStream_t s);
// exclusive scan of int64 in[0..n) -> out[0..n], out[n] = total (device)
void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s);

// ---- FP64 step (pd_fp64.cu)
void launch_init_geometry_fp64(const Fp64Args& a, cudaStream_t s);
void launch_drift_fp64(const Fp64Args& a, cudaStream_t s);
void launch_shadow_fp64(const Fp64Args& a, cudaStream_t s);  // [import in_u, in_v, in_a,] u32 := (float)u; i0 <= i < n
// reach[k] := max(reach[k], largest neighbour id of slab k); reach zeroed by the caller
void launch_slab_reach(int64_t n, const int64_t* row_ptr, const int32_t* col, int64_t slab, int32_t* reach,
                       int32_t* low, cudaStream_t s);
// hourglass term if a.k_hg != 0; pdl: programmatic stream serialization (the plain step loop)
void launch_pass_a_fp64(const Fp64Args& a, bool breaking, cudaStream_t s, bool pdl = false);
// mode 0: kick; 1: kick + next step's drift; 2: drop-in kick (acc array in/out)
void launch_pass_b_fp64(const Fp64Args& a, int mode, cudaStream_t s, bool pdl = false);

// batched steps (BatchLaunch / BatchTile / GridBarrier in pd_batch.cuh)
cudaError_t launch_batch_fp64(const Fp64Args* d_plates, const BatchTile* d_tiles, int ntiles, int nsteps,
                              const BatchLaunch& cfg, GridBarrier* d_bar, int nsm, cudaStream_t s);
int batch_occupancy_fp64(const BatchLaunch& cfg);  // resident persistent blocks per SM

// ---- bond-associated FP64 step (pd_bondassoc.cu); families <= 64 bonds
void launch_ba_reverse(const Fp64Args& a, const BondAssoc& b, cudaStream_t s);
// lr, ex, then kq0, kq1 (the weighted shape tensors' inverses: the mode breaks no bond, so K_b is fixed)
void launch_ba_bonds(const Fp64Args& a, const BondAssoc& b, int64_t nslots, cudaStream_t s);
void launch_ba_pass_a(const Fp64Args& a, const BondAssoc& b, cudaStream_t s);
void launch_ba_pass_b(const Fp64Args& a, const BondAssoc& b, int mode, cudaStream_t s);

// ---- Mazars damage (pd_mazars.cu), FP64 contexts; ba != nullptr: bond-associated weights
void launch_mazars_reset(int64_t nslots, int64_t n, const MazarsArgs& m, cudaStream_t s);
void launch_mazars_update(const Fp64Args& a, const BondAssoc* ba, const MazarsArgs& m, cudaStream_t s);
void launch_mazars_to_csr(const Fp64Args& a, const int64_t* row_ptr, const MazarsArgs& m, double* thr_csr,
                          double* bd_csr, cudaStream_t s);
void launch_mazars_from_csr(const Fp64Args& a, const int64_t* row_ptr, const MazarsArgs& m, const double* thr_csr,
                            const double* bd_csr, cudaStream_t s);

// ---- mixed step (pd_mixed.cu)
void launch_init_geometry_mixed(const MixedArgs& a, cudaStream_t s);
// per-block halos of the single-plate passes (needs the SELL layout)
struct HaloLayout {
  int64_t nblocks = 0, staged = 0;
  VisitRec* visit = nullptr;
  uint16_t* loc = nullptr;   // live 16-bit indices
  uint16_t* loc0 = nullptr;  // pristine (all bonds intact)
  uint16_t* self_loc = nullptr;
  int32_t* halo = nullptr;
  int32_t* halo_n = nullptr;
  int32_t halo_max = 0;
};
// block_chunks: nblocks x (kHaloBlock / 32) chunk ids (-1: none) of the
// visiting blocks; halos are sorted by the spatial key rk
int build_halo_mixed(const MixedArgs& a, int64_t nslots, int64_t nblocks, const int32_t* block_chunks,
                     const uint64_t* rk, cudaStream_t s, HaloLayout* out, std::string* msg);
void launch_halo_relink(const MixedArgs& a, const HaloLayout& h, cudaStream_t s);
// bcp[p] = bc[member[p]] (0 for holes): the mixed form's BC groups by SELL position
void launch_bc_by_position(int64_t npos, const int32_t* member, const uint8_t* bc, uint8_t* bcp, cudaStream_t s);
void launch_drift_mixed(const MixedArgs& a, cudaStream_t s);
void launch_pass_a_mixed(const MixedArgs& a, bool breaking, cudaStream_t s);
void launch_pass_b_mixed(const MixedArgs& a, bool drift, cudaStream_t s);
void launch_to_mixed(const MixedArgs& a, const double2* u, const double2* v, const double2* f, cudaStream_t s);
// pd_step_host (mixed): slabbed passes over visiting blocks a.blk0 .. a.nblocks - 1 in plain
// stream order; the fused import + drift of the positions of visiting blocks blk0 .. blk1 - 1
// from FP64 state by particle id; and, per visiting block, the lowest / highest SELL position
// its bonds reach, the lowest / highest particle id it holds and its first chunk.
void launch_slab_pass_a_mixed(const MixedArgs& a, bool breaking, cudaStream_t s);
void launch_slab_pass_b_mixed(const MixedArgs& a, bool exporting, cudaStream_t s);
void launch_import_drift_mixed(const MixedArgs& a, int64_t blk0, int64_t blk1, const double2* u, const double2* v,
                               const double2* f, cudaStream_t s);
void launch_block_reach_mixed(const MixedArgs& a, int64_t* lo, int64_t* hi, int64_t* idlo, int64_t* idhi,
                              int64_t* cfirst, cudaStream_t s);
void launch_from_mixed(const MixedArgs& a, double2* u, double2* v, double2* f, cudaStream_t s);
// mixed tiles: {plate, particles <= 256, first = visiting block}; smem = the
// largest mixed_pass_smem of the batch's plates for pass A (smem_a) and pass B (smem_b)
cudaError_t launch_batch_mixed(const MixedArgs* d_plates, const BatchTile* d_tiles, int ntiles, int nsteps,
                               const BatchLaunch& cfg, size_t smem_a, size_t smem_b, GridBarrier* d_bar, int nsm,
                               cudaStream_t s);
int batch_occupancy_mixed(const BatchLaunch& cfg, size_t smem);
size_t mixed_pass_smem(const MixedArgs& a, bool pass_a);  // dynamic shared memory of a mixed pass

inline int64_t blocks_for(int64_t n, int64_t per = kBlock) { return (n + per - 1) / per; }

}  // namespace pd
