// k_probe.cu -- live measurement of the FP64 pipe throughput of this GPU.
//
// The FP64 step is bound by the FP64 pipe, not by HBM, so the roofline that
// binds it is the measured rate of dependent-chain-free DFMA and of IEEE
// double division, taken here on the same GPU right before the benchmark.
#include <cuda_runtime.h>
#include "../../include/euler2d_gb300.h"

namespace {

__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ddiv(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3 + 1, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < iters; ++i) {
    x0 = a / x0 + b; x1 = a / x1 + b; x2 = a / x2 + b; x3 = a / x3 + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

}  // namespace

extern "C" int e2d_measure_fp64_peak(double* dfma_per_s, double* ddiv_per_s) {
  if (!dfma_per_s || !ddiv_per_s) return E2D_ERR_INVALID_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess) {
    cudaGetLastError();
    return E2D_ERR_NO_DEVICE;
  }
  const int threads = 256, blocks = sms * 8;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)threads * blocks * sizeof(double)) != cudaSuccess) return E2D_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0;
  const long long n = (long long)threads * blocks;
  k_dfma<<<blocks, threads>>>(out, 16, 0.999, 0.5);
  cudaEventRecord(e0);
  const int it_fma = 4000;
  k_dfma<<<blocks, threads>>>(out, it_fma, 0.999, 0.5);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  *dfma_per_s = (double)n * it_fma * 8 / (ms * 1e-3);
  const int it_div = 400;
  cudaEventRecord(e0);
  k_ddiv<<<blocks, threads>>>(out, it_div, 0.999, 0.5);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  *ddiv_per_s = (double)n * it_div * 4 / (ms * 1e-3);
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return e == cudaSuccess ? E2D_OK : E2D_ERR_CUDA;
}
