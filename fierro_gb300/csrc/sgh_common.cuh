// Device helpers shared by the cycle kernels (sgh_kernels.cu) and the adjoint
// kernels (sgh_adjoint.cu).  Included inside each unit's implementation
// namespace; FIERRO_FMA selects the arithmetic mode.  The adjoint recomputes
// forward values with these same functions, so its branch decisions (limiter,
// CFL minimum) are taken on bit-identical values.
#pragma once

// Order-preserving map from a double to a signed 64-bit key (integer min/max run
// on the integer pipes instead of the FP64 pipe).  -0.0 sorts just below +0.0.
__device__ __forceinline__ long long okey(double d) {
  const long long b = __double_as_longlong(d);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double okey_decode(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}

// pow(v, 1.0/3.0) as the reference computes it (force_sgh.cpp:319-320).
// The exponent is fl(1/3) = 1/3 - d, d = 2^-54/3, so the target is
// cbrt(v) * v^-d = cbrt(v) * (1 - d ln v + O(d^2 ln^2 v)).  c0 = cbrt(v) (<= 1 ulp)
// is refined by one Newton step for t^3 = v whose residual v - c0^3 is formed
// with error-free products (fma), and the -c0 d ln v term is added; both are
// sub-ulp corrections, so ln v and the step only need ~1e-6 relative accuracy.
// The result is the correctly rounded power except within ~1e-6 ulp of a
// rounding boundary.  Non-positive, subnormal and non-finite inputs use pow().
__device__ __forceinline__ double pow_third(double v) {
#if FIERRO_FMA
  return cbrt(v);
#else
  if (!(v > 1.0e-290 && v < 1.0e290)) return pow(v, 1.0 / 3.0);
  const double c0 = cbrt(v);
  const double p = c0 * c0;
  const double pe = fma(c0, c0, -p);
  const double q = p * c0;
  const double qe = fma(p, c0, -q) + pe * c0;
  const double r = (v - q) - qe;  // v - q is exact (Sterbenz), qe carries the rest
  const float rf = (float)r;
  const float inv3p = __frcp_rn(3.0f * (float)p);
  const float step = rf * inv3p;  // (v - c0^3) / (3 c0^2)
  // ln v from the exponent and a single-precision log of the significand
  const long long bits = __double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7FF) - 1023;
  const double m = __longlong_as_double((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const float lnv = (float)ex * 0.69314718f + __logf((float)m);
  const float dlog = lnv * 1.8503717077085943e-17f;  // d = 2^-54 / 3
  const double lo = (double)step - c0 * (double)dlog;
  return c0 + lo;
#endif
}

__device__ __forceinline__ long long block_min_key(long long k) {
  for (int o = 16; o > 0; o >>= 1) {
    long long t = __shfl_xor_sync(0xFFFFFFFFu, k, o);
    k = t < k ? t : k;
  }
  __shared__ long long warp_min[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_min[wid] = k;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    k = lane < nw ? warp_min[lane] : 0x7FFFFFFFFFFFFFFFLL;
    for (int o = 16; o > 0; o >>= 1) {
      long long t = __shfl_xor_sync(0xFFFFFFFFu, k, o);
      k = t < k ? t : k;
    }
  }
  return k;  // valid in thread 0
}
