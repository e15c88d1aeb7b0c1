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

// Square roots and quotients by Newton-Raphson iteration from single-precision
// seeds (Markstein's scheme, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990), arranged so that
// most of the work runs on the FP32 and integer pipes: the FP64 pipe bounds
// these kernels, and GB300 issues FP64 at a small fraction of its FP32 rate.
//
// The argument (divisor) is split into a significand m in [1, 4) ([1, 2)) and a
// power of two by integer operations, and m into a pair of floats mh + ml (its
// top 24 significand bits, exactly, and the next 29 bits rounded).  A
// single-precision root y0 (hardware reciprocal square root; ~2^-22 relative) or
// reciprocal r0 is refined by one Newton step evaluated in single precision on
// the pair -- the residual m - y0^2 (1 - m r0) formed from the products' exact
// low parts (fmaf) -- which carries the float pair's sum to ~2^-43.  One FP64
// Newton step around an exactly formed residual then leaves ~2^-64 (square
// root) or ~2^-89 (quotient) relative error before the final rounding: three
// FP64 operations per square root, four per quotient (one reciprocal shared by
// several quotients: three each), three per reciprocal, and in the exact mode
// one more for the remainder test below.  The single-precision
// steps use the _rn intrinsics, which are never contracted (a fused mh - y0*y0
// would count the product's low part twice).
//
// FMA mode: these results as they are (square roots within an ulp, quotients
// the IEEE ones but for ~2^-37 of an ulp around rounding boundaries).
// Exact mode (square roots, and quotients that share a divisor; its single
// quotients and reciprocals keep the library's division, which the remainder
// test would make no cheaper): correctly rounded, so bit for bit the IEEE square
// root and division.  With the result
// y (q) within an ulp, the remainder x - y^2 (a - b q) is exactly representable
// and one fma forms it; y is the correctly rounded root iff |x - y^2| < ulp(y) y
// (up to 2^-52 relative), q the correctly rounded quotient iff
// |a - b q| < |b| ulp(q) / 2.  The remainder is compared with that bound on the
// bits, and the result kept only where it lies below the bound by more than
// 2^-20 of it; elsewhere (about one result in 10^6; above the bound cannot
// happen within the error above) and where y (q) is a power of two (the ulp
// below is half the ulp above) the library's operation gives it.
//
// Arguments outside 2^-900 .. 2^900 (square root) or 2^-250 .. 2^251
// (quotients), zero, subnormal and non-finite ones included, take the library's
// operation too (tested on the bits); zeros are returned as they are (their
// root is themselves; a 256^3 Sedov cycle, most of whose mesh is at rest, and a
// Noh cycle, where every node moves, take the same time).  The library's
// operations are reached through calls: inline under the exact mode's
// data-dependent test they were if-converted and ran on every lane (the exact
// cycle 12 % slower).
// FIERRO_LIBRARY_ROOTS / FIERRO_LIBRARY_DIV build either mode with the
// library's square and cube roots / divisions throughout, for comparison.

constexpr long long kAbsMask = 0x7FFFFFFFFFFFFFFFLL;
constexpr long long kMantMask = 0x000FFFFFFFFFFFFFLL;
constexpr long long kHardBand = 1LL << 32;  // 2^-20 relative, on the bits

// Single-precision image of a positive double within float range (truncated).
__device__ __forceinline__ float f32_image(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  return __int_as_float((e << 23) | (int)((b >> 29) & 0x7FFFFF));
}
// What f32_image drops: the low 29 significand bits of a positive double with
// exponent in [0, 2], rounded to single precision.
__device__ __forceinline__ float f32_rest(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  return (float)(int)(b & 0x1FFFFFFF) * __int_as_float((127 + e - 52) << 23);
}
// The double of a positive normal float, exactly, from its bits.
__device__ __forceinline__ double f64_of(float f) {
  const unsigned b = __float_as_uint(f);
  const long long e = (long long)((b >> 23) & 0xFF) - 127 + 1023;
  return __longlong_as_double((e << 52) | ((long long)(b & 0x7FFFFF) << 29));
}
// The double of a float of either sign, exactly; zero for zero and subnormal floats.
__device__ __forceinline__ double f64_of_signed(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFF;
  const long long bits = ((long long)(b >> 31) << 63) | ((long long)(e + (1023 - 127)) << 52) |
                         ((long long)(b & 0x7FFFFF) << 29);
  return __longlong_as_double(e == 0 ? 0LL : bits);
}

// sqrt(x) to ~2^-64 before the final rounding; b = x's bits, x positive and
// normal, ex its biased exponent.
__device__ __forceinline__ double sqrt_newton(double x, long long b, int ex) {
  const int k = (ex - 1023) >> 1;                                      // x = m 4^k
  const double m = __longlong_as_double(b - ((long long)(2 * k) << 52));  // [1, 4)
  const float mh = f32_image(m);
  const float r = rsqrtf(mh);                                          // ~ 1 / sqrt(m)
  const double h = __longlong_as_double(__double_as_longlong(f64_of(r)) - (1LL << 52));  // r / 2
#ifdef FIERRO_ROOTS_FP64_NEWTON
  // the earlier form: two FP64 Newton steps from the float seed
  double y = m * f64_of(r);
  y = fma(h, fma(-y, y, m), y);
  y = fma(h, fma(-y, y, m), y);
#else
  const float y0 = __fmul_rn(mh, r);
  const float p = __fmul_rn(y0, y0);
  const float pe = fmaf(y0, y0, -p);                                   // y0^2 = p + pe exactly
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(mh, p), pe), f32_rest(m));  // m - y0^2 (mh - p exact)
  const float c = __fmul_rn(d, __fmul_rn(0.5f, r));
  double y = __dadd_rn(f64_of(y0), f64_of_signed(c));
  y = fma(h, fma(-y, y, m), y);
#endif
  return __longlong_as_double(__double_as_longlong(y) + ((long long)k << 52));
}

// The library's operations for the arguments the Newton forms leave to it.
__device__ __noinline__ double lib_sqrt(double x) { return sqrt(x); }
__device__ __noinline__ double lib_div(double a, double b) { return a / b; }

#if defined(FIERRO_LIBRARY_ROOTS)
__device__ __forceinline__ double mode_sqrt(double x) { return sqrt(x); }
#else
__device__ __forceinline__ double mode_sqrt(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
#if FIERRO_FMA
  if (b <= 0 || ex == 0 || ex == 0x7FF) return (b & kAbsMask) == 0 ? x : lib_sqrt(x);  // sqrt(+-0) = +-0
  return sqrt_newton(x, b, ex);
#else
  if (b <= 0 || (unsigned)(ex - (1023 - 900)) > 1800u) return (b & kAbsMask) == 0 ? x : lib_sqrt(x);
  const double y = sqrt_newton(x, b, ex);
  const long long yb = __double_as_longlong(y);
  const long long tb = yb + ((long long)((int)(yb >> 52) - 1023 - 52) << 52);  // y ulp(y)
  const long long gap = (__double_as_longlong(fma(-y, y, x)) & kAbsMask) - tb;
  return (yb & kMantMask) == 0 || gap > -kHardBand ? lib_sqrt(x) : y;
#endif
}
#endif

// Cube root, the same way: the float root c0 = cbrtf(mh) refined once on the
// pair (residual m - c0^3 from the exact low parts of c0^2 and c0^3), then one
// FP64 step whose residual rounds y^2 once (within an ulp of the library's cube
// root, which is not correctly rounded either).  Four FP64 operations.  v
// positive and normal; b its bits, ex its biased exponent.
__device__ __forceinline__ double cbrt_newton(double v, long long b, int ex) {
  const int E = ex - 1023;
  const int k = E >= 0 ? E / 3 : -((2 - E) / 3);                        // floor(E / 3)
  const double m = __longlong_as_double(b - ((long long)(3 * k) << 52));  // [1, 8)
  const float mh = f32_image(m);
  const float c0 = cbrtf(mh);
#ifdef FIERRO_ROOTS_FP64_NEWTON
  const double c0d = f64_of(c0);
  const double inv = f64_of(__frcp_rn(3.0f * c0 * c0));                // ~ 1 / (3 c^2)
  double c = fma(fma(-(c0d * c0d), c0d, m), inv, c0d);
  c = fma(fma(-(c * c), c, m), inv, c);
#else
  const float p = __fmul_rn(c0, c0);
  const float pe = fmaf(c0, c0, -p);                                   // c0^2 = p + pe exactly
  const float q = __fmul_rn(p, c0);
  const float qe = __fadd_rn(fmaf(p, c0, -q), __fmul_rn(pe, c0));      // c0^3 ~ q + qe
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(mh, q), qe), f32_rest(m));  // m - c0^3 (mh - q exact)
  const float inv = __frcp_rn(__fmul_rn(3.0f, p));                     // ~ 1 / (3 c0^2)
  double c = __dadd_rn(f64_of(c0), f64_of_signed(__fmul_rn(d, inv)));
  const double c2 = c * c;
  c = fma(fma(-c2, c, m), f64_of(inv), c);
#endif
  return __longlong_as_double(__double_as_longlong(c) + ((long long)k << 52));
}

#if FIERRO_FMA && !defined(FIERRO_LIBRARY_ROOTS)
// The FMA mode's cube root; the exact mode keeps the library's cbrt (its pow
// takes the Newton cube root as a starting value only, pow_third below).
__device__ __forceinline__ double mode_cbrt(double v) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (b <= 0 || ex == 0 || ex == 0x7FF) return cbrt(v);
  return cbrt_newton(v, b, ex);
}
#else
__device__ __forceinline__ double mode_cbrt(double v) { return cbrt(v); }
#endif

// 2^-250 <= |x| < 2^251: the operands of the Newton quotients.
__device__ __forceinline__ bool plain_range(long long bits) {
  return (unsigned)((bits >> 52) & 0x7FF) - 773u <= 500u;
}
// ~ 1/b to ~2^-44: the float pair's sum for b's significand bm in [1, 2) as a
// double, scaled by b's power of two and given b's sign (b within plain_range).
__device__ __forceinline__ double rcp_seed(long long bb) {
  const int eb = (int)((bb >> 52) & 0x7FF) - 1023;
  const double bm = __longlong_as_double((bb & kMantMask) | 0x3FF0000000000000LL);  // [1, 2)
  const float bh = f32_image(bm);
  const float r0 = __frcp_rn(bh);
  const float p = __fmul_rn(bh, r0);
  const float pe = fmaf(bh, r0, -p);                                    // bh r0 = p + pe exactly
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(f32_rest(bm), r0));  // 1 - bm r0
  const double r = __dadd_rn(f64_of(r0), f64_of_signed(__fmul_rn(r0, e)));
  return __longlong_as_double((__double_as_longlong(r) - ((long long)eb << 52)) ^ (bb & ~kAbsMask));
}
// Reciprocal and reciprocal square root to ~2^-43 relative, for derivative
// terms that have no parity target (the adjoint's reverse arithmetic): the float
// pair of the Newton forms above as a double, without their FP64 step (one FP64
// addition each).  Arguments outside 2^-250 .. 2^251 (reciprocal) or zero,
// negative, subnormal and non-finite ones (reciprocal square root) take the
// library's operation.
__device__ __forceinline__ double fast_rcp(double b) {
  const long long bb = __double_as_longlong(b);
  return plain_range(bb) ? rcp_seed(bb) : 1.0 / b;
}
__device__ __forceinline__ double fast_rsqrt(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (b <= 0 || ex == 0 || ex == 0x7FF) return rsqrt(x);
  const int k = (ex - 1023) >> 1;                                      // x = m 4^k
  const double m = __longlong_as_double(b - ((long long)(2 * k) << 52));  // [1, 4)
  const float mh = f32_image(m);
  const float r0 = rsqrtf(mh);
  const float p = __fmul_rn(r0, r0);
  const float pe = fmaf(r0, r0, -p);                                   // r0^2 = p + pe exactly
  const float q = __fmul_rn(mh, p);
  const float qe = fmaf(mh, p, -q);                                    // mh p = q + qe exactly
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, q), qe),
                            __fadd_rn(__fmul_rn(mh, pe), __fmul_rn(f32_rest(m), p)));  // 1 - m r0^2 (1 - q exact)
  const double r = __dadd_rn(f64_of(r0), f64_of_signed(__fmul_rn(__fmul_rn(0.5f, r0), e)));  // r0 (1 + e/2)
  return __longlong_as_double(__double_as_longlong(r) - ((long long)k << 52));
}
// A divisor prepared once for the quotients that share it.
struct Divisor {
  double b, r;
  bool plain;
};
__device__ __forceinline__ Divisor divisor(double b) {
  const long long bb = __double_as_longlong(b);
  return Divisor{b, rcp_seed(bb), plain_range(bb)};
}
// The exact mode's test of a Newton quotient q of a / b: false only where q is
// the correctly rounded quotient (see above).
__device__ __forceinline__ bool quot_hard(double a, double b, double q) {
  const long long qb = __double_as_longlong(q);
  const int eq = (int)((qb >> 52) & 0x7FF) - 1023;
  const long long tb = (__double_as_longlong(b) & kAbsMask) + ((long long)(eq - 53) << 52);  // |b| ulp(q) / 2
  const long long gap = (__double_as_longlong(fma(-b, q, a)) & kAbsMask) - tb;
  return (qb & kMantMask) == 0 || gap > -kHardBand;
}
__device__ __forceinline__ double quot(double a, const Divisor& d) {
#ifdef FIERRO_LIBRARY_DIV
  return a / d.b;
#else
  const long long ab = __double_as_longlong(a);
  if (!d.plain || !plain_range(ab))  // +-0 / b: the signed zero a r
    return d.plain && (ab & kAbsMask) == 0 ? a * d.r : lib_div(a, d.b);
  const double q0 = a * d.r;
  const double q = fma(fma(-d.b, q0, a), d.r, q0);
#if FIERRO_FMA
  return q;
#else
  return quot_hard(a, d.b, q) ? lib_div(a, d.b) : q;
#endif
#endif
}
// A single quotient or reciprocal: the Newton form in the FMA mode; the
// library's division in the exact mode, where the remainder test makes the
// Newton form no cheaper unless several quotients share the divisor's seed
// (measured: the exact element pass 1.4 % faster with the library's).
#if FIERRO_FMA
__device__ __forceinline__ double mode_div(double a, double b) { return quot(a, divisor(b)); }
#else
__device__ __forceinline__ double mode_div(double a, double b) { return a / b; }
#endif
__device__ __forceinline__ double mode_rcp(double b) {
#if defined(FIERRO_LIBRARY_DIV) || !FIERRO_FMA
  return 1.0 / b;
#else
  const long long bb = __double_as_longlong(b);
  if (!plain_range(bb)) return lib_div(1.0, b);
  const double r = rcp_seed(bb);
  return fma(fma(-b, r, 1.0), r, r);
#endif
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
  return mode_cbrt(v);
#else
  // 1e-290 < v < 1e290, compared on the bits (positive doubles order as integers)
  const long long bits = __double_as_longlong(v);
  if (!(bits > 0x03B8F2B061AEA072LL && bits < 0x7C2485CE9E7A065FLL)) return pow(v, 1.0 / 3.0);
#ifdef FIERRO_LIBRARY_ROOTS
  const double c0 = cbrt(v);
#else
  const double c0 = cbrt_newton(v, bits, (int)((bits >> 52) & 0x7FF));  // within an ulp: a starting value
#endif
  const double p = c0 * c0;
  const double pe = fma(c0, c0, -p);
  const double q = p * c0;
  const double qe = fma(p, c0, -q) + pe * c0;
  const double r = (v - q) - qe;  // v - q is exact (Sterbenz), qe carries the rest
  const float rf = (float)r;
  const float inv3p = __frcp_rn(3.0f * (float)p);
  const float step = rf * inv3p;  // (v - c0^3) / (3 c0^2)
  // ln v from the exponent and a single-precision log of the significand
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
