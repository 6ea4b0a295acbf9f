// pd_probe_fma_rates: measured FMA issue rates of this GPU (FP64 and FP32),
// the denominators of the FP64 form's ALU roofline.  GB300's FP64 rate is a
// small fraction of its FP32 rate, so the FP64 step is bounded by the FP64
// pipe long before HBM; bench.py reports that fraction next to the HBM one.
//
// Each thread runs 8 independent FMA chains for a fixed iteration count (no
// memory traffic in the loop); grid = 8 blocks per SM x 256 threads.  The
// result store keeps the chains alive.  Timed with CUDA events after a
// warm-up launch.
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
