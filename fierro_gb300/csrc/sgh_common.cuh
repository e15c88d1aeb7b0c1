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

#if FIERRO_FMA && !defined(FIERRO_LIBRARY_ROOTS)
// Square and cube roots of the fused-multiply-add mode (FIERRO_LIBRARY_ROOTS
// builds the FMA mode with the library's sqrt and cbrt instead, for comparison): Newton-Raphson iterations
// in FP64 from a single-precision seed (Markstein's scheme, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev.
// 34(1), 1990).  The argument is split into a significand m in [1, 4) (square
// root) or [1, 8) (cube root) and a power of two by integer operations; the seed
// comes from the single-precision hardware reciprocal square root / the
// single-precision cube root of m's truncated image (about 2^-22 relative); two
// Newton steps, each one DMUL/DFMA pair around an exactly formed residual, carry
// it to about 2^-88, so the result is the rounded root up to the final fma's
// rounding.  Measured on 2^28 random inputs against the library: the square
// root differs in 1 of 10^6 results by 1 ulp, the cube root in 8.6% by 1 ulp
// (the library's cube root is not correctly rounded either); both run 1.3x /
// 1.8x the library's throughput on the FP64 pipe, which bounds these kernels.
// Zero, negative, subnormal and non-finite arguments take the library's path.

// Single-precision image of a positive double within float range (truncated).
__device__ __forceinline__ float f32_image(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  return __int_as_float((e << 23) | (int)((b >> 29) & 0x7FFFFF));
}
// The double of a positive normal float, exactly, from its bits.
__device__ __forceinline__ double f64_of(float f) {
  const unsigned b = __float_as_uint(f);
  const long long e = (long long)((b >> 23) & 0xFF) - 127 + 1023;
  return __longlong_as_double((e << 52) | ((long long)(b & 0x7FFFFF) << 29));
}
__device__ __forceinline__ double mode_sqrt(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (!(x > 0.0) || ex == 0 || ex == 0x7FF) return sqrt(x);
  const int k = (ex - 1023) >> 1;                                      // x = m 4^k
  const double m = __longlong_as_double(b - ((long long)(2 * k) << 52));  // [1, 4)
  const double r = f64_of(rsqrtf(f32_image(m)));                       // ~ 1 / sqrt(m)
  const double h = __longlong_as_double(__double_as_longlong(r) - (1LL << 52));  // r / 2
  double y = m * r;
  y = fma(h, fma(-y, y, m), y);
  y = fma(h, fma(-y, y, m), y);
  return __longlong_as_double(__double_as_longlong(y) + ((long long)k << 52));
}
__device__ __forceinline__ double mode_cbrt(double v) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (!(v > 0.0) || ex == 0 || ex == 0x7FF) return cbrt(v);
  const int E = ex - 1023;
  const int k = E >= 0 ? E / 3 : -((2 - E) / 3);                        // floor(E / 3)
  const double m = __longlong_as_double(b - ((long long)(3 * k) << 52));  // [1, 8)
  const float cf = cbrtf(f32_image(m));
  const double c0 = f64_of(cf);
  const double inv = f64_of(__frcp_rn(3.0f * cf * cf));                // ~ 1 / (3 c^2)
  double c = fma(fma(-(c0 * c0), c0, m), inv, c0);
  c = fma(fma(-(c * c), c, m), inv, c);
  return __longlong_as_double(__double_as_longlong(c) + ((long long)k << 52));
}
#else
__device__ __forceinline__ double mode_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double mode_cbrt(double v) { return cbrt(v); }
#endif

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
  return mode_cbrt(v);
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
