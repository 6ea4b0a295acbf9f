// pd_compute_velocity_noalloc: one FP64 force + kick on caller-owned device
// buffers, for callers that must not allocate device memory.
//
// Who needs it: a host application that owns every device allocation through
// its own pool (and forbids other allocators in its address space), and code
// on a latency-critical path, where cudaMalloc/cudaFree would synchronise
// the device.  Such a caller hands in its own buffers for inputs and
// outputs; the only memory beyond them is the per-particle scratch between
// the two kernels (W, m / V and the zero-energy-mode penalty term, 8 doubles
// per particle), and that lives in the file-scope array below, sized for
// PD_NOALLOC_MAX_PARTICLES particles (8 * 8 * 65536 B = 4 MiB, held by every
// device that loads the library until the process exits).
//
// The arithmetic is the FP64 form's, operation for operation (this file is
// compiled with --fmad=false, like pd_fp64.cu), walking the caller's CSR
// families directly; with the same inputs and no broken bonds its results
// equal pd_compute_velocity's bit for bit.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "pd_internal.h"

namespace {

constexpr int kNoallocBlock = 256;
constexpr int kScratchPerParticle = 8;  // W (4) + m / V (2) + penalty term (2)

// The scratch.  Every call shares it and it keeps the previous call's
// contents; each call writes every entry it later reads, so nothing needs
// clearing.  Two calls whose kernels overlap on the GPU (different streams,
// or different host threads) race on it.
static __device__ __align__(256) double g_noalloc_scratch[(size_t)PD_NOALLOC_MAX_PARTICLES * kScratchPerParticle];

struct NoallocArgs {
  int64_t n;
  const double2* x;
  const double* vol;
  const int64_t* row_ptr;
  const int32_t* col;
  const double2* u;
  double2* v;
  double2* acc;
  double2* f;
  double2* w01;  // scratch
  double2* w23;  // scratch
  double2* mt;   // scratch
  double2* hg;   // scratch
  double c11, c12, c33, dt, inv_rho, det_guard, k_hg;
};

// Pass A: K^-1 and m/V over the given family, D, stress, W (no bond breaking).
__global__ void __launch_bounds__(kNoallocBlock) k_noalloc_pass_a(NoallocArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double2 xi = a.x[i], ui = a.u[i];
  const int64_t r0 = a.row_ptr[i], r1 = a.row_ptr[i + 1];
  double k11 = 0.0, k12 = 0.0, k22 = 0.0, mx = 0.0, my = 0.0;
  double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0, ax = 0.0, ay = 0.0;
  for (int64_t s = r0; s < r1; ++s) {
    const int j = a.col[s];
    const double2 xj = a.x[j], uj = a.u[j];
    const double ex = xj.x - xi.x, ey = xj.y - xi.y;
    const double vj = a.vol[j];
    const double t0 = vj * ex, t1 = vj * ey;
    k11 = fma(t0, ex, k11);
    k12 = fma(t0, ey, k12);
    k22 = fma(t1, ey, k22);
    mx = mx + t0;
    my = my + t1;
    const double dx = uj.x - ui.x, dy = uj.y - ui.y;
    d11 = fma(dx, t0, d11);
    d12 = fma(dx, t1, d12);
    d21 = fma(dy, t0, d21);
    d22 = fma(dy, t1, d22);
    ax = fma(vj, dx, ax);
    ay = fma(vj, dy, ay);
  }
  const double k2 = 2.0 * a.k_hg;
  a.hg[i] = make_double2(k2 * ax, k2 * ay);
  const double det = fma(k11, k22, -(k12 * k12));
  if (r1 == r0 || !(det > a.det_guard * (k11 * k22))) {
    a.w01[i] = make_double2(0.0, 0.0);
    a.w23[i] = make_double2(0.0, 0.0);
    a.mt[i] = make_double2(0.0, 0.0);
    return;
  }
  const double r = 1.0 / det;
  const double q11 = k22 * r, q12 = -k12 * r, q22 = k11 * r;
  const double rv = 1.0 / a.vol[i];
  a.mt[i] = make_double2(mx * rv, my * rv);
  const double g11 = fma(d11, q11, d12 * q12), g12 = fma(d11, q12, d12 * q22);
  const double g21 = fma(d21, q11, d22 * q12), g22 = fma(d21, q12, d22 * q22);
  const double e11 = g11, e22 = g22, e12 = 0.5 * (g12 + g21);
  const double s11 = fma(a.c11, e11, a.c12 * e22);
  const double s22 = fma(a.c12, e11, a.c11 * e22);
  const double s12 = a.c33 * e12;
  const double vi = a.vol[i], kh = -a.k_hg;
  a.w01[i] = make_double2(vi * fma(kh, g11, fma(s11, q11, s12 * q12)), vi * fma(kh, g12, fma(s11, q12, s12 * q22)));
  a.w23[i] = make_double2(vi * fma(kh, g21, fma(s12, q11, s22 * q12)), vi * fma(kh, g22, fma(s12, q12, s22 * q22)));
}

// Pass B: gather force, velocity-Verlet kick, acce := f / rho.
__global__ void __launch_bounds__(kNoallocBlock) k_noalloc_pass_b(NoallocArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double2 xi = a.x[i], wa = a.w01[i], wb = a.w23[i], m = a.mt[i], h = a.hg[i];
  double fx = fma(wa.x, m.x, fma(wa.y, m.y, h.x));
  double fy = fma(wb.x, m.x, fma(wb.y, m.y, h.y));
  for (int64_t s = a.row_ptr[i]; s < a.row_ptr[i + 1]; ++s) {
    const int j = a.col[s];
    const double2 xj = a.x[j], ja = a.w01[j], jb = a.w23[j];
    const double ex = xj.x - xi.x, ey = xj.y - xi.y;
    fx = fma(ja.x, ex, fx);
    fx = fma(ja.y, ey, fx);
    fy = fma(jb.x, ex, fy);
    fy = fma(jb.y, ey, fy);
  }
  const double2 ao = a.acc[i];
  const double anx = fx * a.inv_rho, any = fy * a.inv_rho;
  double2 v = a.v[i];
  v.x = v.x + (0.5 * (ao.x + anx)) * a.dt;
  v.y = v.y + (0.5 * (ao.y + any)) * a.dt;
  a.v[i] = v;
  a.f[i] = make_double2(fx, fy);
  a.acc[i] = make_double2(anx, any);
}

// Device address of the scratch, looked up once per device with that device
// current (a host-side use of the symbol's name would be a host address).
std::mutex g_scratch_mu;
double* g_scratch_ptr[64] = {nullptr};

void set_err(char* errbuf, int errlen, const char* msg) {
  if (errbuf && errlen > 0) {
    std::strncpy(errbuf, msg, (size_t)errlen - 1);
    errbuf[errlen - 1] = '\0';
  }
}

}  // namespace

extern "C" int pd_compute_velocity_noalloc(int64_t n, const double* x, const double* vol, const int64_t* row_ptr,
                                           const int32_t* col, const double* u, double* velocity, double* acce,
                                           double* netF, const pd_params* p, void* stream, char* errbuf,
                                           int errlen) {
  if (n < 0 || n > PD_NOALLOC_MAX_PARTICLES) {
    char m[160];
    std::snprintf(m, sizeof(m), "pd_compute_velocity_noalloc: n = %lld is outside [0, %d] (PD_NOALLOC_MAX_PARTICLES)",
                  (long long)n, PD_NOALLOC_MAX_PARTICLES);
    set_err(errbuf, errlen, m);
    return PD_ERR_CAPACITY;
  }
  if (!p || !x || !vol || !row_ptr || (!col && n > 0) || !u || !velocity || !acce || !netF) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: NULL argument");
    return PD_ERR_ARG;
  }
  if (!(p->rho > 0.0) || !(p->dt > 0.0)) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: rho and dt must be positive");
    return PD_ERR_ARG;
  }
  if (n == 0) return PD_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: no current CUDA device");
    return PD_ERR_CUDA;
  }
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* q = nullptr;
      e = cudaGetSymbolAddress(&q, g_noalloc_scratch);
      if (e != cudaSuccess) {
        char m[200];
        std::snprintf(m, sizeof(m), "pd_compute_velocity_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        set_err(errbuf, errlen, m);
        return PD_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<double*>(q);
    }
    scratch = g_scratch_ptr[dev];
  }
  NoallocArgs a;
  a.n = n;
  a.x = reinterpret_cast<const double2*>(x);
  a.vol = vol;
  a.row_ptr = row_ptr;
  a.col = col;
  a.u = reinterpret_cast<const double2*>(u);
  a.v = reinterpret_cast<double2*>(velocity);
  a.acc = reinterpret_cast<double2*>(acce);
  a.f = reinterpret_cast<double2*>(netF);
  a.w01 = reinterpret_cast<double2*>(scratch);
  a.w23 = reinterpret_cast<double2*>(scratch + 2 * (size_t)PD_NOALLOC_MAX_PARTICLES);
  a.mt = reinterpret_cast<double2*>(scratch + 4 * (size_t)PD_NOALLOC_MAX_PARTICLES);
  a.hg = reinterpret_cast<double2*>(scratch + 6 * (size_t)PD_NOALLOC_MAX_PARTICLES);
  const double pre = p->E / (1.0 - p->nu * p->nu);  // plane stress, as pd_create's contexts
  a.c11 = pre;
  a.c12 = p->nu * pre;
  a.c33 = (1.0 - p->nu) * pre;
  a.dt = p->dt;
  a.inv_rho = 1.0 / p->rho;
  a.det_guard = p->det_guard;
  a.k_hg = p->k_hg;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)((n + kNoallocBlock - 1) / kNoallocBlock);
  k_noalloc_pass_a<<<nb, kNoallocBlock, 0, s>>>(a);
  k_noalloc_pass_b<<<nb, kNoallocBlock, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    char m[200];
    std::snprintf(m, sizeof(m), "pd_compute_velocity_noalloc: launch: %s", cudaGetErrorString(e));
    set_err(errbuf, errlen, m);
    return PD_ERR_CUDA;
  }
  return PD_OK;
}
