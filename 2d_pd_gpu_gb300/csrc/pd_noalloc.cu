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
//
// The caller's CSR is checked on the device as it is walked: a particle whose
// row is not a range inside [row_ptr[0] = 0, row_ptr[n]], or whose family
// names an index outside [0, n), reads nothing out of range and gets NaN in
// its velocity, acce and netF (so do the particles whose families reach it),
// which the caller sees in its own outputs without a synchronisation.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
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

// A particle's row [r0, r1) is walkable when it lies inside [0, row_ptr[n]]
// (the caller's col holds row_ptr[n] entries) and row_ptr[0] is 0.
__device__ __forceinline__ bool row_ok(const NoallocArgs& a, int64_t i, int64_t* r0, int64_t* r1) {
  *r0 = a.row_ptr[i];
  *r1 = a.row_ptr[i + 1];
  return a.row_ptr[0] == 0 && 0 <= *r0 && *r0 <= *r1 && *r1 <= a.row_ptr[a.n];
}

// Pass A: K^-1 and m/V over the given family, D, stress, W (no bond breaking).
__global__ void __launch_bounds__(kNoallocBlock) k_noalloc_pass_a(NoallocArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double2 xi = a.x[i], ui = a.u[i];
  int64_t r0, r1;
  bool ok = row_ok(a, i, &r0, &r1);
  double k11 = 0.0, k12 = 0.0, k22 = 0.0, mx = 0.0, my = 0.0;
  double d11 = 0.0, d12 = 0.0, d21 = 0.0, d22 = 0.0, ax = 0.0, ay = 0.0;
  for (int64_t s = r0; ok && s < r1; ++s) {
    const int j = a.col[s];
    if (j < 0 || j >= a.n) {  // a bad index: read nothing, poison this particle
      ok = false;
      break;
    }
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
  if (!ok) {
    const double q = nan("");
    a.hg[i] = make_double2(q, q);
    a.w01[i] = make_double2(q, q);
    a.w23[i] = make_double2(q, q);
    a.mt[i] = make_double2(q, q);
    return;
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
  int64_t r0, r1;
  bool ok = row_ok(a, i, &r0, &r1);
  for (int64_t s = r0; ok && s < r1; ++s) {
    const int j = a.col[s];
    if (j < 0 || j >= a.n) {
      ok = false;
      break;
    }
    const double2 xj = a.x[j], ja = a.w01[j], jb = a.w23[j];
    const double ex = xj.x - xi.x, ey = xj.y - xi.y;
    fx = fma(ja.x, ex, fx);
    fx = fma(ja.y, ey, fx);
    fy = fma(jb.x, ex, fy);
    fy = fma(jb.y, ey, fy);
  }
  if (!ok) fx = fy = nan("");
  const double2 ao = a.acc[i];
  const double anx = fx * a.inv_rho, any = fy * a.inv_rho;
  double2 v = a.v[i];
  v.x = v.x + (0.5 * (ao.x + anx)) * a.dt;
  v.y = v.y + (0.5 * (ao.y + any)) * a.dt;
  a.v[i] = v;
  a.f[i] = make_double2(fx, fy);
  a.acc[i] = make_double2(anx, any);
}

// Device address of the scratch.  In host code the array's name is only a
// host-side stand-in, so the address is looked up with cudaGetSymbolAddress
// in the CUDA context that is current at the call, once per context, and
// cached under that context's unique id (cuCtxGetId: never reused in a
// process, so a context destroyed by cudaDeviceReset cannot leave a stale
// address behind; its replacement is looked up afresh).  The driver entry
// points come through the runtime, so the library does not link libcuda.
std::mutex g_scratch_mu;
struct ScratchEntry {
  unsigned long long ctx_id;
  double* ptr;
};
constexpr int kScratchCache = 64;
ScratchEntry g_scratch_cache[kScratchCache] = {};
int g_scratch_next = 0;
PFN_cuCtxGetCurrent_v4000 g_ctx_get_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_get_id = nullptr;

// The current context's id; 0 with *err set when it cannot be had.
unsigned long long current_context_id(cudaError_t* err) {
  *err = cudaSuccess;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
      *err = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : cudaErrorSymbolNotFound);
      return 0;
    }
    g_ctx_get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
    g_ctx_get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&c) == CUDA_SUCCESS && !c) {
    // No context bound to this thread yet: bind the current device's primary
    // context, as any runtime call would (a context the caller made current
    // itself is left as it is).
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaSetDevice(dev);
    g_ctx_get_current(&c);
  }
  if (!c || g_ctx_get_id(c, &id) != CUDA_SUCCESS) {
    *err = cudaErrorDeviceUninitialized;
    return 0;
  }
  return id;
}

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
  if (!p) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: NULL params");
    return PD_ERR_ARG;
  }
  if (!(p->rho > 0.0) || !(p->dt > 0.0)) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: rho and dt must be positive");
    return PD_ERR_ARG;
  }
  // What this path does not implement is refused, not ignored.
  if (p->precision != PD_FP64) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: FP64 only (precision must be PD_FP64)");
    return PD_ERR_ARG;
  }
  if (p->n1 != 0.0 || p->n2 != 0.0) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: classic weights only (n1 = n2 = 0)");
    return PD_ERR_ARG;
  }
  if (p->s_c > 0.0) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: no bond breaking here (s_c must be 0)");
    return PD_ERR_ARG;
  }
  if (!x || !vol || !row_ptr || (!col && n > 0) || !u || !velocity || !acce || !netF) {
    set_err(errbuf, errlen, "pd_compute_velocity_noalloc: NULL argument");
    return PD_ERR_ARG;
  }
  if (n == 0) return PD_OK;
  cudaError_t e = cudaSuccess;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    const unsigned long long id = current_context_id(&e);
    if (id == 0) {
      char m[200];
      std::snprintf(m, sizeof(m), "pd_compute_velocity_noalloc: no current CUDA context: %s", cudaGetErrorString(e));
      set_err(errbuf, errlen, m);
      return PD_ERR_CUDA;
    }
    for (int k = 0; k < kScratchCache; ++k)
      if (g_scratch_cache[k].ctx_id == id) scratch = g_scratch_cache[k].ptr;
    if (!scratch) {  // first call in this context: set-up
      void* q = nullptr;
      e = cudaGetSymbolAddress(&q, g_noalloc_scratch);
      if (e != cudaSuccess || !q) {
        char m[200];
        std::snprintf(m, sizeof(m), "pd_compute_velocity_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        set_err(errbuf, errlen, m);
        return PD_ERR_CUDA;
      }
      scratch = static_cast<double*>(q);
      g_scratch_cache[g_scratch_next] = {id, scratch};
      g_scratch_next = (g_scratch_next + 1) % kScratchCache;
    }
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
