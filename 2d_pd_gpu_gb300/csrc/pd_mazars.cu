// Mazars damage on the device (FP64; compiled with --fmad=false like the FP64
// step, so the strain of the classic model is bit-identical to the oracle's).
//
// Reference: computeDamageStatus (src/main_seq.cpp:473-598), called by the
// reference main at the start of every step (:683); it does not feed the
// forces.  For every bond b = (i, nb) of a family: the bond's strain
// eps = sym(F) - I (classic weights: particle i's F = I + D K^-1 over its
// intact bonds; bond-associated weights: the bond's own F_b), its principal
// values (closed-form 2x2 symmetric eigen-decomposition, ascending), the
// equivalent strain eq = |<eps>_+|; where eq exceeds the bond's history
// threshold kappa_b the tensile / compressive split (alpha_t, alpha_c) and
//   d_t = 1 - kappa_b (1 - a_t) / eq - a_t / exp(b_t (eq - kappa_b))   (d_c alike)
// give the bond damage d_b = alpha_t d_t + alpha_c d_c and kappa_b := eq.
// Per particle, status_i = sum_b d_b / family size (Particle::damageStatus),
// summed in family order.  The reference accumulates the tensile and
// compressive parts into uninitialised matrices (:509-515, :547-554); here
// they start at zero, as in the oracle restatement.
#include "pd_internal.h"

namespace pd {

namespace {

// Eigen's SelfAdjointEigenSolver contract for a 2x2 symmetric [[p, o], [o, q]]:
// ascending eigenvalues, unit eigenvector columns vec[.][k].
__device__ void sym_eig2(double p, double o, double q, double lam[2], double vec[2][2]) {
  const double mean = 0.5 * (p + q), h = 0.5 * (p - q);
  const double rad = sqrt(h * h + o * o);
  lam[0] = mean - rad;
  lam[1] = mean + rad;
  if (o == 0.0) {
    const bool swap = p > q;
    vec[0][0] = swap ? 0.0 : 1.0;
    vec[1][0] = swap ? 1.0 : 0.0;
    vec[0][1] = swap ? 1.0 : 0.0;
    vec[1][1] = swap ? 0.0 : 1.0;
    return;
  }
  for (int k = 0; k < 2; ++k) {
    const double x = o, y = lam[k] - p;
    const double nrm = sqrt(x * x + y * y);
    vec[0][k] = x / nrm;
    vec[1][k] = y / nrm;
  }
}

struct MzPoint {
  double eq, at, ac;
};

// Equivalent strain and the (alpha_t, alpha_c) split of strain (e11, e12, e22).
__device__ MzPoint mazars_point(double e11, double e12, double e22) {
  double lam[2], v[2][2];
  sym_eig2(e11, e12, e22, lam, v);
  double s2 = 0.0;
  for (int i = 0; i < 2; ++i)
    if (lam[i] > 0.0) s2 += lam[i] * lam[i];
  MzPoint r{s2 > 0.0 ? sqrt(s2) : 0.0, 0.0, 0.0};
  if (!(r.eq > 0.0)) return r;
  double st[2][2] = {{0.0, 0.0}, {0.0, 0.0}}, sc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int i = 0; i < 2; ++i) {
    if (lam[i] > 0.0) {
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) st[j][k] += lam[i] * v[j][i] * v[k][i];
    } else if (lam[i] < 0.0) {
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) sc[j][k] += lam[i] * v[j][i] * v[k][i];
    }
  }
  double tl[2], tv[2][2], cl[2], cv[2][2];
  sym_eig2(st[0][0], 0.5 * (st[0][1] + st[1][0]), st[1][1], tl, tv);
  sym_eig2(sc[0][0], 0.5 * (sc[0][1] + sc[1][0]), sc[1][1], cl, cv);
  for (int i = 0; i < 2; ++i) {
    if (tl[i] > 0.0) r.at += tl[i] * (tl[i] + cl[i]) / (r.eq * r.eq);
    if (cl[i] > 0.0) r.ac += cl[i] * (tl[i] + cl[i]) / (r.eq * r.eq);
  }
  return r;
}

__device__ __forceinline__ void mazars_bond(const MzPoint& p, const MazarsArgs& m, double* thr, double* bd) {
  const double k = *thr;
  if (!(p.eq > k)) return;
  const double dt = 1.0 - k * (1 - m.a_t) / p.eq - m.a_t / exp(m.b_t * (p.eq - k));
  const double dc = 1.0 - k * (1 - m.a_c) / p.eq - m.a_c / exp(m.b_c * (p.eq - k));
  *bd = p.at * dt + p.ac * dc;
  *thr = p.eq;
}

__device__ __forceinline__ void family_status(const Fp64Args& a, const MazarsArgs& m, int64_t i, int64_t s0,
                                              int fam) {
  double sum = 0.0;
  for (int k = 0; k < fam; ++k) sum += m.bd[s0 + (int64_t)k * kChunk] / (double)fam;
  m.status[i] = sum;
}

// Classic weights: one strain per particle, from the same D sum as pass A.
__global__ void __launch_bounds__(kBlock) k_mazars_classic(Fp64Args a, MazarsArgs m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t s0 = a.chunk_base[i >> 5] + (i & 31);
  const int fam = a.fam[i];
  const double2 ui = a.u[i];
  double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0;
  for (int k = 0; k < fam; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = a.nbr[s];
    if (j < 0) continue;  // broken: no strain contribution (its history still updates below)
    const double2 uj = a.u[j];
    const double dx = uj.x - ui.x, dy = uj.y - ui.y;
    const double2 t = a.bgeo[s];
    d11 = fma(dx, t.x, d11);
    d12 = fma(dx, t.y, d12);
    d21 = fma(dy, t.x, d21);
    d22 = fma(dy, t.y, d22);
  }
  MzPoint p{0.0, 0.0, 0.0};
  if (!a.singular[i]) {
    const double2 k01 = a.kinv01[i];
    const double k11 = k01.x, k12 = k01.y, k22 = a.kinv22[i];
    const double g11 = fma(d11, k11, d12 * k12), g12 = fma(d11, k12, d12 * k22);
    const double g21 = fma(d21, k11, d22 * k12), g22 = fma(d21, k12, d22 * k22);
    p = mazars_point(g11, 0.5 * (g12 + g21), g22);
  }
  for (int k = 0; k < fam; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    mazars_bond(p, m, &m.thr[s], &m.bd[s]);
  }
  family_status(a, m, i, s0, fam);
}

// Bond-associated weights: every bond's own K_b, D_b (families <= kMzMax).
constexpr int kMzMax = 64;

__device__ __forceinline__ double mz_weight(const BondAssoc& b, double bx, double by, double lb, double kx, double ky,
                                            double lk) {
  double c = (bx * kx + by * ky) / (lb * lk);
  if (c > 1.0) c = 1.0;
  else if (c < -1.0) c = -1.0;
  const double lr = fabs(lb - lk) * b.inv_wlen;
  return exp(-b.n1 * lr) * pow(0.5 + 0.5 * c, b.n2);
}

__global__ void __launch_bounds__(128) k_mazars_ba(Fp64Args a, BondAssoc ba, MazarsArgs m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t s0 = a.chunk_base[i >> 5] + (i & 31);
  const int fam = a.fam[i] < kMzMax ? a.fam[i] : kMzMax;
  double ex[kMzMax], ey[kMzMax], el[kMzMax], vv[kMzMax], dx[kMzMax], dy[kMzMax];
  const double2 ui = a.u[i];
  for (int k = 0; k < fam; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int v = a.nbr[s];
    const int j = v >= 0 ? v : -2 - v;
    const double2 e = a.bxi[s];
    const double2 uj = a.u[j];
    ex[k] = e.x;
    ey[k] = e.y;
    el[k] = sqrt(e.x * e.x + e.y * e.y);
    vv[k] = a.vol[j];
    dx[k] = uj.x - ui.x;
    dy[k] = uj.y - ui.y;
  }
  for (int q = 0; q < fam; ++q) {
    double k11 = 0.0, k12 = 0.0, k22 = 0.0, d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0;
    for (int k = 0; k < fam; ++k) {
      const double wv = mz_weight(ba, ex[q], ey[q], el[q], ex[k], ey[k], el[k]) * vv[k];
      const double t0 = wv * ex[k], t1 = wv * ey[k];
      k11 = fma(t0, ex[k], k11);
      k12 = fma(t0, ey[k], k12);
      k22 = fma(t1, ey[k], k22);
      d11 = fma(dx[k], t0, d11);
      d12 = fma(dx[k], t1, d12);
      d21 = fma(dy[k], t0, d21);
      d22 = fma(dy[k], t1, d22);
    }
    MzPoint p{0.0, 0.0, 0.0};
    const double det = fma(k11, k22, -(k12 * k12));
    if (det > a.det_guard * (k11 * k22)) {
      const double r = 1.0 / det;
      const double q11 = k22 * r, q12 = -k12 * r, q22 = k11 * r;
      const double g11 = fma(d11, q11, d12 * q12), g12 = fma(d11, q12, d12 * q22);
      const double g21 = fma(d21, q11, d22 * q12), g22 = fma(d21, q12, d22 * q22);
      p = mazars_point(g11, 0.5 * (g12 + g21), g22);
    }
    const int64_t s = s0 + (int64_t)q * kChunk;
    mazars_bond(p, m, &m.thr[s], &m.bd[s]);
  }
  family_status(a, m, i, s0, a.fam[i]);
}

// Per-bond history <-> family (CSR) order, and statuses from the bond damage.
__global__ void k_mz_to_csr(int64_t n, const int64_t* __restrict__ row_ptr, const int64_t* __restrict__ chunk_base,
                            const double* __restrict__ thr, const double* __restrict__ bd, double* thr_csr,
                            double* bd_csr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s0 = chunk_base[i >> 5] + (i & 31), r0 = row_ptr[i], deg = row_ptr[i + 1] - r0;
  for (int64_t k = 0; k < deg; ++k) {
    if (thr_csr) thr_csr[r0 + k] = thr[s0 + k * kChunk];
    if (bd_csr) bd_csr[r0 + k] = bd[s0 + k * kChunk];
  }
}

__global__ void k_mz_from_csr(Fp64Args a, MazarsArgs m, const int64_t* __restrict__ row_ptr,
                              const double* __restrict__ thr_csr, const double* __restrict__ bd_csr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t s0 = a.chunk_base[i >> 5] + (i & 31), r0 = row_ptr[i], deg = row_ptr[i + 1] - r0;
  for (int64_t k = 0; k < deg; ++k) {
    if (thr_csr) m.thr[s0 + k * kChunk] = thr_csr[r0 + k];
    if (bd_csr) m.bd[s0 + k * kChunk] = bd_csr[r0 + k];
  }
  family_status(a, m, i, s0, (int)deg);
}

__global__ void k_mz_fill(int64_t nslots, double kappa0, double* thr, double* bd) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  thr[s] = kappa0;
  bd[s] = 0.0;
}

}  // namespace

void launch_mazars_reset(int64_t nslots, int64_t n, const MazarsArgs& m, cudaStream_t s) {
  if (nslots > 0) k_mz_fill<<<(unsigned)blocks_for(nslots), kBlock, 0, s>>>(nslots, m.kappa0, m.thr, m.bd);
  if (n > 0) cudaMemsetAsync(m.status, 0, (size_t)n * sizeof(double), s);
}

void launch_mazars_update(const Fp64Args& a, const BondAssoc* ba, const MazarsArgs& m, cudaStream_t s) {
  if (a.n <= 0) return;
  if (ba)
    k_mazars_ba<<<(unsigned)blocks_for(a.n, 128), 128, 0, s>>>(a, *ba, m);
  else
    k_mazars_classic<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, m);
}

void launch_mazars_to_csr(const Fp64Args& a, const int64_t* row_ptr, const MazarsArgs& m, double* thr_csr,
                          double* bd_csr, cudaStream_t s) {
  if (a.n > 0)
    k_mz_to_csr<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a.n, row_ptr, a.chunk_base, m.thr, m.bd, thr_csr, bd_csr);
}

void launch_mazars_from_csr(const Fp64Args& a, const int64_t* row_ptr, const MazarsArgs& m, const double* thr_csr,
                            const double* bd_csr, cudaStream_t s) {
  if (a.n > 0) k_mz_from_csr<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, m, row_ptr, thr_csr, bd_csr);
}

}  // namespace pd
