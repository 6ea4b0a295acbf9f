// pd_probe_fma_rates: measured FMA issue rates of this GPU (FP64 and FP32),
// the denominators of the FP64 form's ALU roofline.
// pd_probe_link_rates: measured copy-engine rates between page-locked host
// memory and this GPU (each direction alone, and both at once), the
// denominator of pd_step_host's end-to-end bound.
//  GB300's FP64 rate is a
// small fraction of its FP32 rate, so the FP64 step is bounded by the FP64
// pipe long before HBM; bench.py reports that fraction next to the HBM one.
//
// FMA rates: each thread runs 8 independent FMA chains for a fixed iteration count (no
// memory traffic in the loop); grid = 8 blocks per SM x 256 threads.  The
// result store keeps the chains alive.  Timed with CUDA events after a
// warm-up launch.
#include <cstring>

#include <cuda_runtime.h>

#include "pd_gb300.h"

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int rate(int device, int iters, double* per_s) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PD_ERR_CUDA;
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * threads) != cudaSuccess) return PD_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, threads>>>(out, 16, (T)1.0000001, (T)1e-9);
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)1.0000001, (T)1e-9);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return PD_ERR_CUDA;
  *per_s = 8.0 * iters * (double)blocks * threads / (ms * 1e-3);
  return PD_OK;
}

}  // namespace

extern "C" int pd_probe_fma_rates(int32_t device, double* fp64_fma_per_s, double* fp32_fma_per_s) {
  if (!fp64_fma_per_s || !fp32_fma_per_s) return PD_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PD_ERR_CUDA;
  int rc = rate<double>(device, 2000, fp64_fma_per_s);
  if (rc == PD_OK) rc = rate<float>(device, 20000, fp32_fma_per_s);
  return rc;
}

namespace {

struct LinkProbe {
  void *h_in = nullptr, *h_out = nullptr, *d_a = nullptr, *d_b = nullptr;
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  ~LinkProbe() {
    if (s0) cudaStreamSynchronize(s0);
    if (s1) cudaStreamSynchronize(s1);
    cudaFreeHost(h_in);
    cudaFreeHost(h_out);
    cudaFree(d_a);
    cudaFree(d_b);
    if (s0) cudaStreamDestroy(s0);
    if (s1) cudaStreamDestroy(s1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e2) cudaEventDestroy(e2);
  }
};

// Best of `reps` timed repetitions (after two untimed ones) of fn, in ms.
template <typename F>
cudaError_t best_ms(LinkProbe& p, int reps, F fn, float* out) {
  float b = 1e30f;
  for (int r = 0; r < reps + 2; ++r) {
    cudaError_t e = cudaEventRecord(p.e0, p.s0);
    if (e == cudaSuccess) e = fn();
    if (e == cudaSuccess) e = cudaEventRecord(p.e1, p.s0);
    if (e == cudaSuccess) e = cudaEventSynchronize(p.e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.e0, p.e1);
    if (e != cudaSuccess) return e;
    if (r >= 2 && ms < b) b = ms;
  }
  *out = b;
  return cudaSuccess;
}

}  // namespace

extern "C" int pd_probe_link_rates(int32_t device, int64_t bytes, double* h2d_gbs, double* d2h_gbs,
                                   double* both_gbs) {
  if (!h2d_gbs || !d2h_gbs || !both_gbs || bytes < 16 || bytes > (int64_t{1} << 32)) return PD_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PD_ERR_CUDA;
  const size_t b = (size_t)bytes;
  LinkProbe p;
  if (cudaHostAlloc(&p.h_in, b, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc(&p.h_out, b, cudaHostAllocDefault) != cudaSuccess || cudaMalloc(&p.d_a, b) != cudaSuccess ||
      cudaMalloc(&p.d_b, b) != cudaSuccess || cudaStreamCreateWithFlags(&p.s0, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p.s1, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&p.e0) != cudaSuccess ||
      cudaEventCreate(&p.e1) != cudaSuccess || cudaEventCreate(&p.e2) != cudaSuccess)
    return PD_ERR_CUDA;
  memset(p.h_in, 1, b);
  if (cudaMemset(p.d_b, 0, b) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return PD_ERR_CUDA;
  float t1 = 0.f, t2 = 0.f, t3 = 0.f;
  cudaError_t e = best_ms(p, 6, [&] { return cudaMemcpyAsync(p.d_a, p.h_in, b, cudaMemcpyHostToDevice, p.s0); }, &t1);
  if (e == cudaSuccess)
    e = best_ms(p, 6, [&] { return cudaMemcpyAsync(p.h_out, p.d_b, b, cudaMemcpyDeviceToHost, p.s0); }, &t2);
  if (e == cudaSuccess)
    e = best_ms(p, 6, [&] {
      cudaError_t r = cudaMemcpyAsync(p.d_a, p.h_in, b, cudaMemcpyHostToDevice, p.s0);
      if (r == cudaSuccess) r = cudaStreamWaitEvent(p.s1, p.e0, 0);
      if (r == cudaSuccess) r = cudaMemcpyAsync(p.h_out, p.d_b, b, cudaMemcpyDeviceToHost, p.s1);
      if (r == cudaSuccess) r = cudaEventRecord(p.e2, p.s1);
      if (r == cudaSuccess) r = cudaStreamWaitEvent(p.s0, p.e2, 0);
      return r;
    }, &t3);
  if (e != cudaSuccess) return PD_ERR_CUDA;
  *h2d_gbs = (double)b / (t1 * 1e-3) / 1e9;
  *d2h_gbs = (double)b / (t2 * 1e-3) / 1e9;
  *both_gbs = (double)b / (t3 * 1e-3) / 1e9;
  return PD_OK;
}
