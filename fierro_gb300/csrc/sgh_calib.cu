// FP64 roof calibration: the SGH path's binding resource on GB300 is the FP64
// pipe, so its roofline needs a measured FP64 rate beside the measured HBM rate.
// Eight independent fused-multiply-add chains per thread keep the pipe busy;
// the grid covers every SM several times over.
#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_device.h"
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

// The FP64 pipe on a pure stream: CH independent chains per thread of one
// operation (0 fma, 1 add, 2 mul), for the peak survey of fierro_fp64_stream_rate.
template <int CH, int OP>
__global__ void k_fp64_stream(double* out, double a, double b, int iters) {
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      if (OP == 0) x[c] = fma(x[c], a, b);
      else if (OP == 1) x[c] = x[c] + b;
      else x[c] = x[c] * a;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int CH>
void launch_stream(int op, int blocks, int threads, double* d, int iters) {
  if (op == 0) k_fp64_stream<CH, 0><<<blocks, threads>>>(d, 0.999, 1e-3, iters);
  else if (op == 1) k_fp64_stream<CH, 1><<<blocks, threads>>>(d, 0.999, 1e-3, iters);
  else k_fp64_stream<CH, 2><<<blocks, threads>>>(d, 0.999, 1e-3, iters);
}

}  // namespace

extern "C" int fierro_fp64_stream_rate(int chains, int op, int threads, int blocks_per_sm,
                                       double* ops_per_second) {
  using fierro::set_error;
  if (!ops_per_second) return set_error(FIERRO_EINVAL, "NULL output");
  if ((chains != 1 && chains != 2 && chains != 4 && chains != 8 && chains != 16) || op < 0 || op > 2 ||
      threads < 32 || threads > 1024 || threads % 32 || blocks_per_sm < 1 || blocks_per_sm > 32)
    return set_error(FIERRO_EINVAL, "fp64 stream: chains 1/2/4/8/16, op 0..2, threads 32..1024, blocks/SM 1..32");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return set_error(FIERRO_ECUDA, "no CUDA device");
  const int blocks = sms * blocks_per_sm, iters = 2048;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return set_error(FIERRO_ENOMEM, "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    switch (chains) {
      case 1: launch_stream<1>(op, blocks, threads, d, iters); break;
      case 2: launch_stream<2>(op, blocks, threads, d, iters); break;
      case 4: launch_stream<4>(op, blocks, threads, d, iters); break;
      case 8: launch_stream<8>(op, blocks, threads, d, iters); break;
      default: launch_stream<16>(op, blocks, threads, d, iters); break;
    }
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
  *ops_per_second = (double)chains * iters * (double)blocks * threads / (best * 1e-3);
  return FIERRO_OK;
}

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

// The arithmetic mode's square and cube roots, quotients and reciprocals against
// the library's (the FMA mode's Newton forms; the exact mode calls the library).
extern "C" int fierro_root_check(int fp_mode, int which, long long n, unsigned long long seed, int lo_exp,
                                 int hi_exp, unsigned long long* out) {
  using fierro::set_error;
  if (!out) return set_error(FIERRO_EINVAL, "NULL output");
  if ((fp_mode != FIERRO_FP_EXACT && fp_mode != FIERRO_FP_FMA) || which < 0 || which > 8 || n < 8 ||
      n > (1LL << 36) || lo_exp < -1022 || hi_exp > 1023 || lo_exp > hi_exp)
    return set_error(FIERRO_EINVAL, "root check: fp_mode 0/1, which 0 sqrt / 1 cbrt / 2 quotient / 3 reciprocal / 4..6 near-boundary "
                                    "sqrt, quotient, reciprocal / 7, 8 fast reciprocal, rsqrt, 8 <= n <= 2^36, "
                                    "-1022 <= lo_exp <= hi_exp <= 1023");
  const fierro::KernelSet& ks = fp_mode == FIERRO_FP_FMA ? fierro::kernels_fma() : fierro::kernels_exact();
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return set_error(FIERRO_ENOMEM, "cudaMalloc");
  cudaError_t err = cudaMemset(d, 0, 3 * sizeof(unsigned long long));
  if (err == cudaSuccess) {
    ks.root_check(which, n, seed, lo_exp, hi_exp, d, 0);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(out, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "%s", cudaGetErrorString(err));
  return FIERRO_OK;
}
