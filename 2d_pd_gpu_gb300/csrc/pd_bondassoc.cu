// Bond-associated NOSB (the reference's default model, n1 / n2 != 0), FP64.
//
// Reference: computeShapeTensors (src/main_seq.cpp:71-156) gives every bond
// b = (i, nb) its own weighted shape tensors
//   K_b = sum_k w(b,k) V_k xi_k (x) xi_k,   N_b = K_b + D_b (D: displacements),
//   w(b,k) = exp(-n1 |L_b - L_k| / (horizon dx)) (0.5 + 0.5 cos(b,k))^n2,
// computeStressTensor (:204-268) its stress sigma_b, and
// computeForceDensityStates (:271-380) the force state
//   T_ij = (1/V_h) sum_b w(j,b) V_b sigma_b K_b^-1 xi_ij,
// with the net force f_i = sum_j (T_ij - T_ji) V_j (computeVelocity :396-470).
// The reference recomputes sigma_b K_b^-1 inside the (i, j) loop (O(n^3) per
// particle).  Here pass A forms P_b = sigma_b K_b^-1 once per bond and T_ij
// once per bond (O(n^2) per particle), storing T per bond slot; pass B reads
// T_ji through the reverse slot index and applies the kick (+ the next
// drift) as the classic form.
//
// The mode breaks no bond, and the weights depend on the reference geometry
// and the parameters only, so what does not involve the displacements is
// formed once, at set-up and on every parameter change, by the set-up form of
// pass A (k_ba_pass_a<true>, after k_ba_bonds): per slot |xi|, 1/|xi|,
// exp(+-n1 |xi| / l) and K_b^-1 with its det-guard flag; per particle with
// <= 32 bonds, the lower triangle of its weight matrix.
//
// Pass A runs one warp per particle and one lane per bond (families <= 64
// bonds, two per lane): the family's bond data is staged in shared memory,
// the weight triangle is loaded into a 32 x 32 matrix there, lane q sums D_q
// over k in family order (the oracle's order) and forms V_q P_q, and, once
// every P_b is in shared memory, lane j sums T_ij over b: 8 FP64 fma per
// ordered pair of bonds.  A family of more than 32 bonds evaluates each lane's
// weight row inside its D_q loop and keeps the rows of the first 32 bonds.
// The weight matrix is symmetric bit for bit (its products commute, and the
// exponential factor is ordered by the two lengths), so only its lower
// triangle is evaluated, spread over all 32 lanes.  The weight is evaluated in
// factored form: exp(-n1 |L_b - L_k| / l) = e+(min L) e-(max L) with
// e+-(L) = exp(+-n1 L / l) per bond, the cosine as (xi_b . xi_k) (1/L_b)(1/L_k),
// and an integer n2 <= 64 by repeated squaring (pow otherwise; the direct exp
// where n1 L / l could overflow).  The sums run in the oracle's order
// (ba_pass_a; --fmad=false, explicit fma()), but the per-bond products
// V_k xi_k (x) xi_k, V_k d_k (x) xi_k and V_b P_b are formed once per bond and
// then weighted (the oracle weights V_k first), and the weights differ from
// its libm exp / pow / division by a few ulp, so GPU and oracle agree to
// rounding (1e-12 normwise), not bit for bit.  No bond breaking here (the
// reference has none).
#include "pd_internal.h"

namespace pd {

namespace {

constexpr int kBaMax = 64;
constexpr int kBaWarps = 2;  // particles per block of pass A (28 KB of shared memory per block: 7 per SM)

struct BaFamily {  // one particle's bonds, in family order
  double ex[kBaMax], ey[kBaMax], vv[kBaMax];
  // pass A: V_k d_k (x) xi_k (dx xi_x, dx xi_y, dy xi_x, dy xi_y); the K table: V_k xi_k (x) xi_k (xx, xy, yy)
  double S[kBaMax][4];
  double P[kBaMax][4];  // V_b sigma_b K_b^-1
  int64_t slot[kBaMax];
  double wrow[32][32];  // wrow[k][l] = w(l, k) for bonds l, k < 32
};

struct BaWeight {
  double n1, inv_wlen, n2;
  const double2* __restrict__ lr;  // per slot: |xi|, 1/|xi|
  const double2* __restrict__ ex;  // per slot: exp(+-n1 |xi| / l)
  int n2i;      // n2 as a small integer (-1: use pow)
  bool direct;  // exp(-n1 |L_b - L_k| / l) evaluated directly (the factors could overflow)
  // The comparisons run on the integer pipe, on the bit patterns (the FP64 pipe
  // is the kernel's bound): c is finite, so |c| > 1 exactly when its magnitude
  // bits exceed those of 1.0, and lengths are >= 0, whose bit patterns order as
  // their values.  The power starts from its first factor and skips the last,
  // unused squaring: the same products as pw = 1, pw *= base for each set bit.
  __device__ __forceinline__ double operator()(const BaFamily& F, int b, int k) const {
    const int64_t sb = F.slot[b], sk = F.slot[k];
    const double2 lb = lr[sb], lk = lr[sk];  // |xi|, 1/|xi| (k_ba_bonds)
    double c = fma(F.ex[b], F.ex[k], F.ey[b] * F.ey[k]) * (lb.y * lk.y);
    const long long cb = __double_as_longlong(c);
    if ((cb & 0x7FFFFFFFFFFFFFFFll) > 0x3FF0000000000000ll) c = cb < 0 ? -1.0 : 1.0;
    const double x = fma(0.5, c, 0.5);
    double pw;
    if (n2i >= 0) {
      pw = 1.0;
      double base = x;
      bool first = true;
      for (int e = n2i; e;) {
        if (e & 1) {
          pw = first ? base : pw * base;
          first = false;
        }
        e >>= 1;
        if (e) base *= base;
      }
    } else {
      pw = pow(x, n2);
    }
    double ew;
    if (direct)
      ew = exp(-n1 * (fabs(lb.x - lk.x) * inv_wlen));
    else
      ew = __double_as_longlong(lb.x) >= __double_as_longlong(lk.x) ? ex[sk].x * ex[sb].y : ex[sb].x * ex[sk].y;
    return ew * pw;
  }
};

// KTAB: the set-up form (launch_ba_bonds), which evaluates the weights (kept
// per particle for families of <= 32 bonds), forms every bond's weighted
// shape tensor K_b and writes K_b^-1 and its det-guard flag per slot (the
// mode breaks no bond and the weights depend on the reference geometry and
// the parameters only, so both are fixed); the same operations in the same
// order as the pass itself would, so reading them back changes no result.
template <bool KTAB>
__global__ void __launch_bounds__(32 * kBaWarps) k_ba_pass_a(Fp64Args a, BondAssoc b) {
  __shared__ BaFamily fam[kBaWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kBaWarps + warp;
  if (i >= a.n) return;  // warp-uniform
  BaFamily& F = fam[warp];
  const int64_t c0 = i >> 5;
  const int w = a.chunk_w[c0];
  const int64_t s0 = a.chunk_base[c0] + (i & 31);
  const double2 ui = a.u[i];
  BaWeight wf;
  wf.n1 = b.n1;
  wf.inv_wlen = b.inv_wlen;
  wf.n2 = b.n2;
  wf.lr = b.lr;
  wf.ex = b.ex;
  wf.n2i = (b.n2 >= 0.0 && b.n2 <= 64.0 && b.n2 == floor(b.n2)) ? (int)b.n2 : -1;
  // stage the family (slots k = lane, lane + 32, compacted past empty slots in order)
  int n = 0;
  double lmax = 0.0;
  for (int k0 = 0; k0 < w; k0 += 32) {
    const int k = k0 + lane;
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = k < w ? a.nbr[s] : -1;
    const unsigned m = __ballot_sync(0xffffffffu, j >= 0);
    const int q = n + __popc(m & ((1u << lane) - 1u));
    if (j >= 0 && q < kBaMax) {
      const double2 e = a.bxi[s];
      const double l = b.lr[s].x;  // k_ba_bonds
      F.ex[q] = e.x;
      F.ey[q] = e.y;
      const double vj = a.vol[j];
      const double t0 = vj * e.x, t1 = vj * e.y;
      F.vv[q] = vj;
      if (KTAB) {
        F.S[q][0] = t0 * e.x;
        F.S[q][1] = t0 * e.y;
        F.S[q][2] = t1 * e.y;
      } else {
        const double2 uj = a.u[j];
        const double dx = uj.x - ui.x, dy = uj.y - ui.y;
        F.S[q][0] = dx * t0;
        F.S[q][1] = dx * t1;
        F.S[q][2] = dy * t0;
        F.S[q][3] = dy * t1;
      }
      F.slot[q] = s;
      lmax = fmax(lmax, l);
    }
    n += __popc(m);
  }
  n = n < kBaMax ? n : kBaMax;
  for (int o = 16; o; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  wf.direct = !(fabs(b.n1) * lmax * b.inv_wlen < 600.0);
  __syncwarp();
  const bool tri = n <= 32;
  if (tri) {  // pair p = k (k + 1) / 2 + q, q <= k, of the lower triangle
    // (the set-up form evaluates it and keeps it per particle; the step reads it back)
    const int npair = n * (n + 1) / 2;
    double* wt = b.wtri + i * kBaTri;
    for (int p = lane; p < npair; p += 32) {
      int k = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
      if ((k + 1) * (k + 2) / 2 <= p) ++k;
      if (k * (k + 1) / 2 > p) --k;
      const int q = p - k * (k + 1) / 2;
      double wqk;
      if (KTAB) {
        wqk = wf(F, q, k);
        wt[p] = wqk;
      } else {
        wqk = wt[p];
      }
      F.wrow[k][q] = wqk;
      F.wrow[q][k] = wqk;
    }
    __syncwarp();
  }
  // P_b = sigma_b K_b^-1 of bond q (KTAB: K_b^-1)
  for (int q = lane; q < n; q += 32) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;  // KTAB: k11, k12, k22; else d11, d12, d21, d22
    for (int k = 0; k < n; ++k) {
      double wqk;
      if (tri) {
        wqk = F.wrow[k][q];
      } else {
        wqk = wf(F, q, k);
        if (q < 32 && k < 32) F.wrow[k][q] = wqk;  // (q == lane: the thread's own row, read back below)
      }
      s0 = fma(wqk, F.S[k][0], s0);
      s1 = fma(wqk, F.S[k][1], s1);
      s2 = fma(wqk, F.S[k][2], s2);
      if (!KTAB) s3 = fma(wqk, F.S[k][3], s3);
    }
    const int64_t sl = F.slot[q];
    if (KTAB) {
      const double k11 = s0, k12 = s1, k22 = s2;
      const double det = fma(k11, k22, -(k12 * k12));
      if (!(det > a.det_guard * (k11 * k22))) {
        b.kq0[sl] = make_double2(0.0, 0.0);
        b.kq1[sl] = make_double2(0.0, 1.0);
        continue;
      }
      const double r = 1.0 / det;
      b.kq0[sl] = make_double2(k22 * r, -k12 * r);
      b.kq1[sl] = make_double2(k11 * r, 0.0);
      continue;
    }
    const double d11 = s0, d12 = s1, d21 = s2, d22 = s3;
    const double2 kq0 = b.kq0[sl], kq1 = b.kq1[sl];
    if (__double_as_longlong(kq1.y) != 0) {  // K_b failed the det guard
      F.P[q][0] = F.P[q][1] = F.P[q][2] = F.P[q][3] = 0.0;
      continue;
    }
    const double q11 = kq0.x, q12 = kq0.y, q22 = kq1.x;
    const double g11 = fma(d11, q11, d12 * q12), g12 = fma(d11, q12, d12 * q22);
    const double g21 = fma(d21, q11, d22 * q12), g22 = fma(d21, q12, d22 * q22);
    const double e11 = g11, e22 = g22, e12 = 0.5 * (g12 + g21);
    const double s11 = fma(a.c11, e11, a.c12 * e22);
    const double s22 = fma(a.c12, e11, a.c11 * e22);
    const double s12 = a.c33 * e12;
    const double vq = F.vv[q];
    F.P[q][0] = vq * fma(s11, q11, s12 * q12);
    F.P[q][1] = vq * fma(s11, q12, s12 * q22);
    F.P[q][2] = vq * fma(s12, q11, s22 * q12);
    F.P[q][3] = vq * fma(s12, q12, s22 * q22);
  }
  if (KTAB) return;
  // V_h in family order (as the oracle), then T_ij of bond jj
  double vh = 0.0;
  for (int k = 0; k < n; ++k) vh = vh + F.vv[k];
  __syncwarp();
  const double rv = 1.0 / vh;
  for (int jj = lane; jj < n; jj += 32) {
    double m11 = 0.0, m12 = 0.0, m21 = 0.0, m22 = 0.0;
    for (int q = 0; q < n; ++q) {
      // w(jj, q) = w(q, jj), kept for pairs of bonds < 32, recomputed for the others
      const double w = jj < 32 && q < 32 ? F.wrow[q][jj] : wf(F, jj, q);
      m11 = fma(w, F.P[q][0], m11);
      m12 = fma(w, F.P[q][1], m12);
      m21 = fma(w, F.P[q][2], m21);
      m22 = fma(w, F.P[q][3], m22);
    }
    const double ex = F.ex[jj], ey = F.ey[jj];
    b.tb[F.slot[jj]] = make_double2(fma(m11 * rv, ex, (m12 * rv) * ey), fma(m21 * rv, ex, (m22 * rv) * ey));
  }
}

// Velocity BC, drift, fixed BC (as pd_fp64.cu's drift_one).
__device__ __forceinline__ void ba_drift(const Fp64Args& a, int64_t i, double2& v, double2& u, double anx,
                                         double any) {
  const int g = a.bc[i];
  const int kind = g ? a.gkind[g - 1] : PD_BC_NONE;
  if (kind == PD_BC_VELOCITY) v = a.gval[g - 1];
  u.x = u.x + (v.x * a.dt + (0.5 * anx) * a.dt2);
  u.y = u.y + (v.y * a.dt + (0.5 * any) * a.dt2);
  if (kind == PD_BC_FIXED) u = make_double2(0.0, 0.0);
}

template <int MODE>
__global__ void __launch_bounds__(kBlock) k_ba_pass_b(Fp64Args a, BondAssoc b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t c0 = i >> 5;
  const int w = a.chunk_w[c0];
  const int64_t s0 = a.chunk_base[c0] + (i & 31);
  double fx = 0.0, fy = 0.0;
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = a.nbr[s];
    if (j < 0) continue;
    const double2 tij = b.tb[s], tji = b.tb[b.rslot[s]];
    const double vj = a.vol[j];
    fx = fma(tij.x - tji.x, vj, fx);
    fy = fma(tij.y - tji.y, vj, fy);
  }
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
    ba_drift(a, i, v, u, anx, any);
    a.u[i] = u;
  }
  a.v[i] = v;
  if (a.out_v) {  // pd_step_host's last pass
    a.out_u[i] = a.u[i];
    a.out_v[i] = v;
    a.out_f[i] = make_double2(fx, fy);
  }
}

// The per-bond constants of the weights, once per slot (they depend on the
// reference geometry and on n1 and l only): |xi|, 1/|xi|, exp(+-n1 |xi| / l);
// k_ba_pass_a<true> then forms the weights and K_b^-1 from them.
__global__ void k_ba_bonds(Fp64Args a, BondAssoc b, int64_t nslots) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots || a.nbr[s] < 0) return;
  const double2 e = a.bxi[s];
  const double l = sqrt(e.x * e.x + e.y * e.y);
  b.lr[s] = make_double2(l, 1.0 / l);
  b.ex[s] = make_double2(exp(b.n1 * (l * b.inv_wlen)), exp(-b.n1 * (l * b.inv_wlen)));
}

// rslot[s] = slot of (j, i) in j's SELL rows, for every slot s = (i, j).
__global__ void k_ba_reverse(Fp64Args a, BondAssoc b, unsigned long long* counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t c0 = i >> 5;
  const int w = a.chunk_w[c0];
  const int64_t s0 = a.chunk_base[c0] + (i & 31);
  for (int k = 0; k < w; ++k) {
    const int64_t s = s0 + (int64_t)k * kChunk;
    const int j = a.nbr[s];
    if (j < 0) continue;
    const int64_t cj = (int64_t)j >> 5;
    const int wj = a.chunk_w[cj];
    const int64_t sj0 = a.chunk_base[cj] + (j & 31);
    int64_t found = -1;
    for (int q = 0; q < wj; ++q)
      if (a.nbr[sj0 + (int64_t)q * kChunk] == (int)i) {
        found = sj0 + (int64_t)q * kChunk;
        break;
      }
    if (found < 0) {
      atomicOr(counters + CNT_ERROR, (unsigned long long)ERR_ASYMMETRIC);
      found = s;  // T_ij - T_ij = 0: the bond is inert
    }
    b.rslot[s] = found;
  }
}

}  // namespace

void launch_ba_reverse(const Fp64Args& a, const BondAssoc& b, cudaStream_t s) {
  if (a.n > 0) k_ba_reverse<<<(unsigned)blocks_for(a.n), kBlock, 0, s>>>(a, b, a.counters);
}

void launch_ba_bonds(const Fp64Args& a, const BondAssoc& b, int64_t nslots, cudaStream_t s) {
  if (nslots > 0) k_ba_bonds<<<(unsigned)((nslots + kBlock - 1) / kBlock), kBlock, 0, s>>>(a, b, nslots);
  if (a.n > 0) k_ba_pass_a<true><<<(unsigned)((a.n + kBaWarps - 1) / kBaWarps), 32 * kBaWarps, 0, s>>>(a, b);
}

void launch_ba_pass_a(const Fp64Args& a, const BondAssoc& b, cudaStream_t s) {
  if (a.n > 0) k_ba_pass_a<false><<<(unsigned)((a.n + kBaWarps - 1) / kBaWarps), 32 * kBaWarps, 0, s>>>(a, b);
}

void launch_ba_pass_b(const Fp64Args& a, const BondAssoc& b, int mode, cudaStream_t s) {
  if (a.n <= 0) return;
  const unsigned nb = (unsigned)blocks_for(a.n);
  if (mode == 0)
    k_ba_pass_b<0><<<nb, kBlock, 0, s>>>(a, b);
  else if (mode == 1)
    k_ba_pass_b<1><<<nb, kBlock, 0, s>>>(a, b);
  else
    k_ba_pass_b<2><<<nb, kBlock, 0, s>>>(a, b);
}

}  // namespace pd
