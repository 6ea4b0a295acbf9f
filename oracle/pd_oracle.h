/* TEST ORACLE -- not part of the product.
 *
 * CPU restatement (C11 + OpenMP, IEEE binary64, no implicit FMA) of the
 * reference's sequential NOSB step (src/main_seq.cpp:386-470, with the
 * bond-associated weights at n1 = n2 = 0, i.e. the classic correspondence
 * model) plus the critical-stretch bond mask and damage that the drop-in
 * adds.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it, and only as the checker / CPU baseline.
 *
 * It is pinned against the reference itself: oracle/_ref (the reference's own
 * main_seq.cpp + SetupParticleSystem.cpp + matrix.cpp compiled by
 * oracle/Makefile) reproduces the reference's shipped golden files
 * byte-for-byte, and tests/golden/ holds full-precision outputs of that
 * build which this restatement must match (tests/test_oracle_golden.py).
 *
 * The operation sequence here is canonical: the CUDA FP64 kernels perform
 * the same IEEE operations in the same order (explicit fma() where written,
 * no contraction elsewhere), so the two agree bit-for-bit.
 */
#ifndef PD_ORACLE_H
#define PD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { PDO_BC_NONE = 0, PDO_BC_VELOCITY = 1, PDO_BC_FIXED = 2 };

typedef struct pdo_problem {
  int64_t n;               /* particles */
  const double* x;         /* [n][2] reference positions */
  const double* vol;       /* [n] volumes */
  const int64_t* row_ptr;  /* [n+1] family CSR */
  const int32_t* col;      /* [row_ptr[n]] neighbour ids, ascending per row */
  const uint8_t* bc;       /* [n] 0 = free, g >= 1 = BC group g-1 (may be NULL) */
  int32_t n_groups;        /* BC groups */
  const int32_t* group_kind; /* [n_groups] PDO_BC_VELOCITY / PDO_BC_FIXED */
  const double* group_val;   /* [n_groups][2] prescribed velocity (VELOCITY) */
  double E, nu, rho, dt;
  double s_c;              /* critical stretch; <= 0 disables breaking */
  double det_guard;        /* relative det(K) guard, e.g. 1e-10 */
  double k_hg;             /* zero-energy-mode penalty coefficient (0: the reference's model) */
  double damage_fail;      /* a particle with damage > this carries no stress (>= 1: never) */
  double n1, n2;           /* bond-associated weights (0, 0: classic) */
  double wlen;             /* length scale of the weight's length ratio (horizon * dx) */
  int32_t nthreads;        /* OpenMP threads, <= 0: runtime default */
} pdo_problem;

typedef struct pdo_state {
  double* u;          /* [n][2] displacements (current position - x) */
  double* v;          /* [n][2] velocities */
  double* f;          /* [n][2] net force density (reference netF) */
  uint8_t* alive;     /* [nnz] 1 = bond intact */
  int32_t* broken;    /* [n] broken-bond count */
  double* damage;     /* [n] broken / family size */
  double* kinv;       /* [n][3] K^-1 (11, 12, 22) of the alive bonds */
  double* mt;         /* [n][2] (sum_j V_j xi_ij) / V_i */
  double* w;          /* [n][4] V_i (S_i - k_hg G_i), S = sigma K^-1, G = F - I */
  double* hg;         /* [n][2] 2 k_hg sum_j V_j (u_j - u_i) */
  uint8_t* singular;  /* [n] 1 if det guard tripped (S_i = 0) */
  double* tb;         /* [nnz][2] bond-associated force states T_ij (n1, n2 != 0 only) */
  int64_t* rev;       /* [nnz] family position of the reverse bond (j, i) (n1, n2 != 0 only) */
} pdo_state;

/* Families within `cutoff` (strict: sqrt(d2) < cutoff, as
 * src/SetupParticleSystem.cpp:100-121), ascending neighbour id, minus bonds
 * that properly cross any crack segment cracks[c] = (ax, ay, bx, by).
 * Two-call protocol: col == NULL returns the bond count in *nnz_out.
 * Returns 0 on success, -1 if cap is too small. */
int pdo_build_families(int64_t n, const double* x, double cutoff, int32_t n_cracks, const double* cracks,
                       int64_t* row_ptr, int32_t* col, int64_t cap, int64_t* nnz_out, int32_t nthreads);

/* u = v = f = 0, all bonds alive, K^-1 / mt from the full families. */
int pdo_init(const pdo_problem* pb, pdo_state* st);

/* nsteps reference steps (src/main_seq.cpp:686-699 order).  Returns the
 * number of bonds broken during these steps (>= 0). */
int64_t pdo_step(const pdo_problem* pb, pdo_state* st, int32_t nsteps);

/* rev[s] = family position of bond (j, i) for every bond s = (i, j); the
 * families must be symmetric (returns -1 otherwise). */
int pdo_reverse_bonds(int64_t n, const int64_t* row_ptr, const int32_t* col, int64_t* rev);

/* Mazars damage (src/main_seq.cpp:473-598, computeDamageStatus; it does not
 * feed the forces).  kappa0 is the initial per-bond threshold (the
 * reference's tensileStrength / E), a_t .. b_c the law's constants
 * (src/main_seq.cpp:481: 0.87, 20000, 0.65, 2150). */
typedef struct pdo_mazars {
  double kappa0, a_t, b_t, a_c, b_c;
} pdo_mazars;

/* One computeDamageStatus call from the state's displacements.  Per bond
 * (family order): thr[nnz] (the history threshold) and bd[nnz] (bond damage)
 * are updated in place where the bond's equivalent strain exceeds thr;
 * status[n] = sum over the family of bd / family size (Particle::damageStatus).
 * Classic weights: the strain of bond (i, j) is particle i's
 * sym(D K^-1) over its intact bonds; bond-associated weights (n1, n2 != 0):
 * bond b's own sym(D_b K_b^-1).  The reference accumulates the tensile and
 * compressive strain parts into uninitialised matrices (:509-515, :547-554);
 * here they start at zero.  Returns 0, or -1 for a family > 256 bonds in the
 * bond-associated mode. */
int pdo_mazars_update(const pdo_problem* pb, const pdo_state* st, const pdo_mazars* mp, double* thr, double* bd,
                      double* status);

/* Plane-stress constants exactly as the device receives them:
 * c[0] = C11 = C22, c[1] = C12, c[2] = C33 (src/main_seq.cpp:180-201). */
void pdo_stiffness(double E, double nu, double c[3]);

#ifdef __cplusplus
}
#endif
#endif
