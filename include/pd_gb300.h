/* pd_gb300.h -- C ABI of the GB300 (sm_103a) explicit NOSB peridynamics step.
 *
 * This is the drop-in boundary that replaces the reference's mechanics call
 * surface (EricYJA/2D_PD_GPU).  Every entry point below names the reference
 * interface it stands in for.  Plain C types only; every call returns an int
 * status (PD_OK = 0, negative on error) and pd_last_error() explains it.  The
 * reference has no return codes (errors go to cout, src/main_seq.cpp:61).
 *
 * Model: 2-D plane-stress classic NOSB (correspondence) peridynamics,
 * influence function 1, critical-stretch bond breaking, velocity Verlet in
 * the reference's step order (src/main_seq.cpp:686-699):
 *     velocity BC -> drift (updatePositions) -> fixed BC -> force + kick.
 * State lives on the device (one context = one plate = one CUDA stream);
 * the host only crosses at set-up, explicit get/set, and step launches.
 *
 * Units are the caller's (the reference uses mm/s/kg/MPa, the plate
 * workloads SI).  Positions are [n][2] interleaved doubles, as the
 * reference's Particle::initialPositions.
 */
#ifndef PD_GB300_H
#define PD_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PD_ABI_VERSION 1

/* status codes */
#define PD_OK 0
#define PD_ERR_ARG (-1)       /* bad argument (size, pointer, value) */
#define PD_ERR_CUDA (-2)      /* CUDA runtime error (see pd_last_error) */
#define PD_ERR_ORDER (-3)     /* call out of order (e.g. step before families) */
#define PD_ERR_CAPACITY (-4)  /* a family exceeds PD_MAX_FAMILY, or out of memory */
#define PD_ERR_SINGULAR (-5)  /* det(K) guard tripped and policy is PD_SINGULAR_ERROR */
#define PD_ERR_DEVICE (-6)    /* a device-side check failed (error word set) */
#define PD_ERR_TIMEOUT (-7)   /* a bounded device wait gave up */

#define PD_MAX_FAMILY 128     /* bonds per particle */
#define PD_MAX_BC_GROUPS 255
#define PD_MAX_CRACKS 64

/* numerical form */
#define PD_FP64 0   /* IEEE binary64 throughout; bit-identical to the oracle */
#define PD_MIXED 1  /* FP32 bond arithmetic, FP64 K^-1 + det guard, compensated sums */

/* boundary-condition group kinds (src/main_seq.cpp:15-46) */
#define PD_BC_NONE 0
#define PD_BC_VELOCITY 1  /* applyVelocityBC: v := value at the start of each step */
#define PD_BC_FIXED 2     /* applyFixedBC: position := reference position after the drift */

/* what a singular shape tensor does (the reference GPU path substitutes the
 * identity, include/mechanics.cuh:29-37; its CPU path divides by zero,
 * src/matrix.cpp:121-126) */
#define PD_SINGULAR_ZERO 0   /* S_i := 0 for that particle, counted in pd_counters */
#define PD_SINGULAR_ERROR 1  /* pd_step returns PD_ERR_SINGULAR */

typedef struct pd_ctx pd_ctx;

typedef struct pd_params {
  int32_t precision;       /* PD_FP64 or PD_MIXED */
  int32_t device;          /* CUDA device ordinal */
  double E;                /* Young's modulus */
  double nu;               /* Poisson ratio (plane stress, src/main_seq.cpp:180-188) */
  double rho;              /* mass density (src/main_seq.cpp:389 massDensity) */
  double dt;               /* time step (src/main_seq.cpp:657 stepSize) */
  double s_c;              /* critical stretch; <= 0 disables bond breaking */
  double det_guard;        /* singular if det(K) <= det_guard * K11 * K22 */
  /* Zero-energy-mode (hourglass) penalty coefficient k (force density per
   * volume per length^2; 0 = the reference's correspondence model exactly).
   * Adds T_ij += k (eta_ij - F_i xi_ij) to every bond, so the force gains
   * 2k sum_j V_j (u_j - u_i) - k G_i m_i - k sum_j V_j G_j xi_ij (G = F - I).
   * The classic model has zero-energy modes (the reference has no control,
   * its bond-associated n1/n2 weights aside); without this, the plate
   * workloads' velocity loading grows them until bonds fail spuriously and
   * the run diverges.  A common choice is k = G_s C11 / (mean V * cutoff^2)
   * with G_s ~ 0.25 at dt = 0.8 CFL. */
  double k_hg;
  /* Material-point failure: a particle whose damage exceeds damage_fail
   * carries no stress (S_i = 0; the penalty still acts on its intact bonds).
   * A particle held by a few bonds has a small K and a correspondence
   * stiffness the time step cannot follow; without this the plate workloads
   * diverge once cracks grow (>= 1: never, the reference's semantics). */
  double damage_fail;
  /* Bond-associated weights of the reference (computeShapeTensors,
   * src/main_seq.cpp:114-118): w = exp(-n1 |L_b - L_k| / weight_len)
   * (0.5 + 0.5 cos)^n2 with weight_len = horizon * dx.  n1 = n2 = 0 is the
   * classic model; otherwise every bond gets its own shape tensor and stress
   * (FP64 only, families <= 64 bonds, no bond breaking, k_hg = 0). */
  double n1, n2, weight_len;
  int32_t singular_policy; /* PD_SINGULAR_ZERO / PD_SINGULAR_ERROR */
  int32_t reserved;
} pd_params;

typedef struct pd_counters {
  int64_t bonds_broken;    /* total bonds broken since pd_reset */
  int64_t singular_events; /* det-guard trips since pd_reset */
  int64_t steps;           /* steps taken since pd_reset */
  int32_t device_error;    /* device error word (0 = none) */
  int32_t unstaged_blocks; /* mixed form: visiting blocks whose halo exceeds the shared-memory
                              cap and whose passes gather neighbour data from HBM (0: FP64) */
} pd_counters;

/* ---------------------------------------------------------------- context */

int pd_abi_version(void);
void pd_default_params(pd_params* p);

/* Creates a context (device buffers are allocated by later calls).  There is
 * no reference counterpart: the reference GPU wrapper allocates, copies and
 * frees everything on every call (include/mechanics.cuh:963-1135). */
int pd_create(const pd_params* p, pd_ctx** out);
int pd_destroy(pd_ctx* ctx);
/* Message for the last failing call on ctx (ctx == NULL: last pd_create). */
const char* pd_last_error(const pd_ctx* ctx);
/* Material / time-step / stretch update; bond data is refreshed in place. */
int pd_set_params(pd_ctx* ctx, const pd_params* p);
int pd_get_params(const pd_ctx* ctx, pd_params* p);
/* Plane-stress stiffness given as the reference's 3x3 Voigt matrix
 * C[9] (row-major, sigma = C [e11, e22, e12], getStiffnessTensor
 * src/main_seq.cpp:180-201) instead of (E, nu).  Requires the plane-stress
 * pattern C[0] == C[4], C[1] == C[3], C[2] == C[5] == C[6] == C[7] == 0.
 * Stays in force until the next pd_set_params. */
int pd_set_stiffness(pd_ctx* ctx, const double* C);

/* --------------------------------------------------------------- problem */

/* Reference positions x[n][2] and volumes vol[n].  Replaces the particle
 * arrays built by computeInitialPositions / readMeshFile
 * (include/SetupParticleSystem.h:24-25) and the per-call H2D copies of
 * include/mechanics.cuh:1050-1060. */
int pd_set_particles(pd_ctx* ctx, int64_t n, const double* x, const double* vol);

/* Families on the GPU: every j != i with sqrt(|x_j - x_i|^2) < cutoff,
 * ascending j, minus bonds that properly cross one of the n_cracks crack
 * segments cracks[c] = (ax, ay, bx, by).  Replaces findNeighbor
 * (src/SetupParticleSystem.cpp:100-121; the reference passes
 * cutoff = 1.01 * dx * horizon) and buildLocalNeighborlist
 * (src/main_seq.cpp:49-68).  Resets the state. */
int pd_build_families(pd_ctx* ctx, double cutoff, int32_t n_cracks, const double* cracks);

/* Families from the host, CSR (row_ptr[n+1] int64, col[row_ptr[n]] int32,
 * ascending per row), e.g. the reference's Particle::neighbors.  Resets. */
int pd_set_families(pd_ctx* ctx, const int64_t* row_ptr, const int32_t* col);

int pd_num_bonds(const pd_ctx* ctx, int64_t* nnz);
int pd_get_families(pd_ctx* ctx, int64_t* row_ptr, int32_t* col);

/* Boundary-condition groups: group_of[i] = 0 (free) or g in 1..n_groups;
 * group g-1 has kind[g-1] and value[g-1][2] (velocity for PD_BC_VELOCITY).
 * Replaces the index sets of defineBoundarySet
 * (src/SetupParticleSystem.cpp:513-529) as used by applyVelocityBC /
 * applyFixedBC (src/main_seq.cpp:28-46).  A particle is in at most one group. */
int pd_set_bc(pd_ctx* ctx, int32_t n_groups, const int32_t* kind, const double* value,
              const uint8_t* group_of);

/* ----------------------------------------------------------------- state */

/* u = v = f = 0, every family bond intact, damage 0, counters 0. */
int pd_reset(pd_ctx* ctx);
/* Any pointer may be NULL (left unchanged).  u = current - reference position. */
int pd_set_state(pd_ctx* ctx, const double* u, const double* v, const double* f);
int pd_get_state(pd_ctx* ctx, double* u, double* v, double* f);
/* damage[n] = broken / family size (the reference's Particle::damageStatus,
 * src/main_seq.cpp:588, with the critical-stretch law instead of Mazars). */
int pd_get_damage(pd_ctx* ctx, double* damage);
/* alive[nnz] in family (CSR) order, 1 = intact. */
int pd_get_bond_mask(pd_ctx* ctx, uint8_t* alive);
int pd_get_counters(pd_ctx* ctx, pd_counters* c);

/* Checkpoint / restore of a device-resident solve (no reference counterpart;
 * used to preempt a served request and resume it later).  The blob holds the
 * dynamic state in the context's own precision (the mixed form's scaled
 * two-float state as stored, so a restored run continues bit for bit): u, v,
 * f, the drop-in acceleration, the bond mask, broken counts, damage,
 * counters and the step count.  It does not hold the problem (particles,
 * families, BCs, parameters): restore into a context built from the same
 * inputs; a blob from another problem, precision or ABI is rejected with
 * PD_ERR_ARG.  Derived data (K^-1, shadows, halo indices) is recomputed on
 * load. */
int pd_checkpoint_size(pd_ctx* ctx, int64_t* bytes);
int pd_checkpoint_save(pd_ctx* ctx, void* buf, int64_t bytes);
int pd_checkpoint_load(pd_ctx* ctx, const void* buf, int64_t bytes);

/* ---------------------------------------------------------- Mazars damage
 * The reference's damage law (computeDamageStatus, src/main_seq.cpp:473-598,
 * called at the start of each step of its main, :683; it does not feed the
 * forces).  Per bond: history threshold and damage; per particle: damage
 * status = sum of its bonds' damage / family size.  FP64 contexts, classic
 * or bond-associated weights (the context's n1, n2).  The tensile and
 * compressive strain parts start at zero (the reference leaves them
 * uninitialised, :509-515). */
typedef struct pd_mazars_params {
  double kappa0;              /* initial threshold: tensile strength / E (reference main: 3 / 3.5e4) */
  double a_t, b_t, a_c, b_c;  /* 0.87, 20000, 0.65, 2150 (src/main_seq.cpp:481) */
} pd_mazars_params;
void pd_mazars_default_params(pd_mazars_params* p);
/* Allocates the history (thresholds = kappa0, damage = 0).  Families first. */
int pd_mazars_init(pd_ctx* ctx, const pd_mazars_params* p);
/* One computeDamageStatus from the context's current displacements
 * (asynchronous on the context's stream). */
int pd_mazars_update(pd_ctx* ctx);
/* Per-bond history in family (CSR) order and per-particle status; any NULL. */
int pd_mazars_get(pd_ctx* ctx, double* threshold, double* bond_damage, double* status);
int pd_mazars_set(pd_ctx* ctx, const double* threshold, const double* bond_damage);

/* ------------------------------------------------------------------ step */

/* nsteps full steps on the device (one CUDA graph per distinct nsteps).
 * Equivalent to nsteps passes of the reference loop body
 * src/main_seq.cpp:686-699 (applyVelocityBC, updatePositions, applyFixedBC,
 * computeVelocity).  Asynchronous unless an error check needs the host. */
int pd_step(pd_ctx* ctx, int32_t nsteps);
/* nsteps steps from a host state to a host state, both precisions (no
 * reference counterpart; the end-to-end form of the reference's per-call
 * host-buffer contract, include/mechanics.cuh:867-881).  u_in, v_in, f_in
 * ([n][2] doubles, page-locked: pd_host_alloc) are copied in by slabs of
 * particles while the first pass runs on the slabs already in.  FP64
 * contexts: in one-step calls each slab's pass B writes its new state to
 * u_out, v_out, f_out directly over the CPU-GPU link while later slabs'
 * pass A runs (in longer calls, the last pass B does); mixed contexts the
 * same, through the mixed form's own slabs of spatial tiles.  In and out may
 * be the same buffers.
 * Synchronous; the device state and the outputs are those of pd_set_state +
 * pd_step + pd_get_state, bit for bit. */
int pd_step_host(pd_ctx* ctx, int32_t nsteps, const double* u_in, const double* v_in, const double* f_in,
                 double* u_out, double* v_out, double* f_out);
/* Waits for the context's stream.  PD_ERR_TIMEOUT if a bounded device wait
 * (the bulk copy that stages bond indices in shared memory) gave up since the
 * last pd_reset; the state is then not trustworthy. */
int pd_synchronize(pd_ctx* ctx);

/* One force + kick with host buffers, the reference GPU wrapper's contract
 * (compute_velocity_GPU_host, include/mechanics.cuh:867-1136, called from
 * src/main.cu:628): reads the displacement u[n][2] (current position minus
 * reference position), velocity[n][2] and acce[n][2]; writes
 * velocity += 0.5 (acce + f/rho) dt, acce = f/rho and netF = f.  Device
 * buffers stay allocated between calls.  The bond mask persists across calls
 * and breaks bonds as in pd_step when s_c > 0.  When all four buffers are
 * page-locked (pd_host_alloc) and the context is in the plain mode, the call
 * runs pd_step_host's slab pipeline: the copies in overlap the first pass,
 * and each slab's results go back while later slabs compute; the results are
 * the same bit for bit. */
int pd_compute_velocity(pd_ctx* ctx, const double* u, double* velocity, double* acce, double* netF);

/* One FP64 force + kick, pd_compute_velocity's arithmetic, on CALLER-OWNED
 * DEVICE buffers and without allocating any device memory.  No counterpart
 * in the reference: it exists for callers that cannot call cudaMalloc -- a
 * host application whose own pool owns every device allocation, or a
 * latency-critical loop where cudaMalloc/cudaFree would synchronise the
 * device.  All array arguments are device pointers: x[n][2], vol[n], the
 * CSR families row_ptr[n+1] / col[row_ptr[n]] (every bond intact; no bond
 * breaking here), u[n][2] (displacement), velocity[n][2] and acce[n][2]
 * (read and written, as pd_compute_velocity), netF[n][2] (written).  p
 * gives E, nu, rho, dt, det_guard, k_hg (plane stress); p->precision must be
 * PD_FP64, n1 = n2 = 0 and s_c = 0 (anything else returns PD_ERR_ARG: this
 * path has no mixed form, bond-associated weights or bond breaking), and
 * damage_fail has no effect (no bond breaks, so no particle is damaged).
 * The caller owns the families' validity: row_ptr[0] = 0, rows
 * non-decreasing, col holding row_ptr[n] indices in [0, n).  The kernels
 * check this as they walk it (the call itself does not read device
 * memory): a particle whose row or indices break it reads nothing out of
 * range and gets NaN in its velocity, acce and netF, as do particles whose
 * families reach it.  stream is a cudaStream_t
 * (NULL: the legacy default stream); the call only enqueues work, so results
 * are ready once that stream is synchronised.  The per-particle scratch
 * between its two kernels lives in a static device array sized for
 * PD_NOALLOC_MAX_PARTICLES particles (4 MiB on every device that loads the
 * library, until exit): larger n returns PD_ERR_CAPACITY.  Every call
 * shares that array, so calls that overlap on the GPU race.  The first call
 * in a CUDA context (normally once per device; again after cudaDeviceReset
 * replaces the device's context) looks up the array's device address
 * (cudaGetSymbolAddress) and caches it for that context; make that first
 * call before any stream capture.  errbuf (may be NULL) receives a message
 * on failure. */
#define PD_NOALLOC_MAX_PARTICLES 65536
int pd_compute_velocity_noalloc(int64_t n, const double* x, const double* vol, const int64_t* row_ptr,
                                const int32_t* col, const double* u, double* velocity, double* acce, double* netF,
                                const pd_params* p, void* stream, char* errbuf, int errlen);

/* ------------------------------------------------------- batched plates */

/* Many independent plates (contexts) of uneven size stepped together by one
 * persistent kernel (or one graph of phase kernels), e.g. the ragged-plate
 * workload and the serving loop.  No reference counterpart (the reference
 * steps one particle system per process).  Members keep their own device
 * state and parameters; a plate's results are identical alone and in any
 * batch.  All members share the batch's device and precision. */
typedef struct pd_batch pd_batch;
typedef struct pd_batch_config {
  int32_t block;          /* threads per block (64..256) */
  int32_t blocks_per_sm;  /* persistent grid = SMs x this (capped at occupancy) */
  int32_t persistent;     /* 1: one cooperative persistent kernel per call; 0: phase kernels;
                             2 (the default): every member's own pd_step graph on its own
                             stream, the members' graphs running concurrently (block, tile,
                             blocks_per_sm unused) */
  int32_t tile;           /* particles per work item (multiple of 32) */
} pd_batch_config;
int pd_batch_create(int32_t device, int32_t precision, pd_batch** out);
int pd_batch_destroy(pd_batch* b);
const char* pd_batch_last_error(const pd_batch* b);
int pd_batch_add(pd_batch* b, pd_ctx* ctx);     /* a context is in at most one batch */
int pd_batch_remove(pd_batch* b, pd_ctx* ctx);  /* pd_destroy also removes it */
int pd_batch_info(const pd_batch* b, int32_t* nplates, int64_t* particles, int64_t* bonds);
int pd_batch_set_config(pd_batch* b, const pd_batch_config* cfg);
int pd_batch_get_config(const pd_batch* b, pd_batch_config* cfg);
/* nsteps steps of every member (asynchronous; members' later calls are
 * ordered after it).  PD_ERR_TIMEOUT if a grid-barrier wait gave up. */
int pd_batch_step(pd_batch* b, int32_t nsteps);
int pd_batch_synchronize(pd_batch* b);
int pd_batch_step_timed(pd_batch* b, int32_t nsteps, float* ms);
/* The persistent kernel's grid-barrier controls (persistent = 1; no
 * reference counterpart -- the reference has no device waits).  spin_limit:
 * polls before a barrier wait gives up and the call reports PD_ERR_TIMEOUT
 * (0: the default, >= 4 s of waiting).  hold_ns: block 0 sleeps this long
 * before it arrives at every barrier (0: never; at most 100 ms) -- a
 * fault-injection control, so a test can make the other blocks' waits run
 * out without faulting anything.  After a timeout the members' state is not
 * trustworthy: pd_reset them (or restore a checkpoint). */
int pd_batch_set_barrier_limits(pd_batch* b, uint64_t spin_limit, uint32_t hold_ns);
/* GPU time of the last pd_batch_step call's kernels (CUDA events on the
 * batch stream, from its first kernel to its last; waits for them). */
int pd_batch_last_step_ms(pd_batch* b, float* ms);

/* Page-locked host buffers for pd_set_state / pd_get_state /
 * pd_compute_velocity (full-bandwidth host<->device copies).  No reference
 * counterpart (the reference copies from pageable std::vector storage,
 * include/mechanics.cuh:976-991). */
int pd_host_alloc(int64_t bytes, void** p);
int pd_host_free(void* p);

/* ---------------------------------------------------------- measurement */

/* pd_step(nsteps) bracketed by CUDA events on the context's stream;
 * *ms = elapsed device time. */
int pd_step_timed(pd_ctx* ctx, int32_t nsteps, float* ms);

#define PD_KERNEL_DRIFT 0
#define PD_KERNEL_PASS_A 1   /* stretch test, D, stress, W = V sigma K^-1 */
#define PD_KERNEL_PASS_B 2   /* force gather + kick (+ next drift) */
#define PD_NUM_KERNELS 3
/* nsteps steps launched kernel by kernel with an event pair around every
 * launch; ms[k] = summed device time of kernel k, launches[k] = launch count. */
int pd_profile_steps(pd_ctx* ctx, int32_t nsteps, double* ms, int64_t* launches);

/* Measured FMA issue rates of the device (FMA lane-operations per second,
 * FP64 and FP32): the FP64 form's ALU roofline denominator.  No reference
 * counterpart. */
int pd_probe_fma_rates(int32_t device, double* fp64_fma_per_s, double* fp32_fma_per_s);

/* Measured copy-engine rates (GB/s) of `bytes` (16 B .. 4 GiB) between
 * page-locked host memory and the device: host to device alone, device to
 * host alone, and each direction while both run at once -- the link bound of
 * pd_step_host.  Allocates its own buffers.  No reference counterpart. */
int pd_probe_link_rates(int32_t device, int64_t bytes, double* h2d_gbs, double* d2h_gbs, double* both_gbs);

/* Algorithmic bytes per step of the dominant kernels (fixed byte model:
 * FP64 248 B/particle + 11 B/bond, mixed 148 B/particle + 11 B/bond). */
int pd_model_bytes(const pd_ctx* ctx, double* bytes_per_step);

#ifdef __cplusplus
}
#endif
#endif /* PD_GB300_H */
