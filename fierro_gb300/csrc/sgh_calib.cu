// FP64 roof calibration: the SGH path's binding resource on GB300 is the FP64
// pipe, so its roofline needs a measured FP64 rate beside the measured HBM rate.
// Eight independent fused-multiply-add chains per thread keep the pipe busy;
// the grid covers every SM several times over.
#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_internal.h"

namespace {

constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_dfma_rate(double* out, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
  for (int i = 0; i < kIters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int fierro_measure_fp64_rate(double* dfma_per_second) {
  using fierro::set_error;
  if (!dfma_per_second) return set_error(FIERRO_EINVAL, "NULL output");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return set_error(FIERRO_ECUDA, "no CUDA device");
  const int blocks = sms * 8, threads = 256;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return set_error(FIERRO_ENOMEM, "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_dfma_rate<<<blocks, threads>>>(d, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "%s", cudaGetErrorString(err));
  *dfma_per_second = 8.0 * kIters * (double)blocks * threads / (best * 1e-3);
  return FIERRO_OK;
}
