// Minimum squared node-pair distance of a hex (the CFL length of get_timestep,
// time_integration.cpp:93-128), exact, with most of the work off the FP64 pipe.
//
// The reference takes min over the 28 node pairs of sqrt(dx^2 + dy^2 + dz^2) with
// dx = x_b - x_a in FP64.  min of sqrt == sqrt of min (sqrt is monotone and
// correctly rounded), so only squared distances are compared.  Screening: each
// coordinate is cut to a single-precision image by integer operations (its top
// 20 significand bits, relative error < 2^-20), the 28 distances are estimated in
// FP32, and an error bound selects the pairs that can still be the minimum; only
// those are evaluated exactly in FP64, in the reference's operation order.  The
// result equals the full evaluation bit for bit.
//
// Bound: with M the largest |coordinate| of the element (of the images), every
// estimated distance d~ satisfies |d~ - d| <= 2^-21 d + E, E = 4e-6 M (covers
// sqrt(3) 2^-19 M for the truncation plus the FP32 roundings), so the true
// minimiser m has d~_m <= T = (min d~ + E)(1 + 2^-18) + E.  Elements whose
// coordinates are not all zero or within [2^-60, 2^60], or whose M < 2^-20, take
// the full FP64 path.
//
// Host compilation (tests) provides the CUDA intrinsics used below.
#pragma once

namespace cfl {

// Pairs (a, b), a < b, grouped by index gap (the reference's visiting order),
// packed 3 bits per node id: pairs 0..20 in the first word, 21..27 in the second.
constexpr unsigned long long pack3(const unsigned char (&t)[28], int from, int n) {
  unsigned long long w = 0;
  for (int i = 0; i < n; ++i) w |= (unsigned long long)t[from + i] << (3 * i);
  return w;
}
constexpr unsigned char kPairA[28] = {0, 1, 2, 3, 4, 5, 6, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 0, 1, 2, 3, 0, 1, 2, 0, 1, 0};
constexpr unsigned char kPairB[28] = {1, 2, 3, 4, 5, 6, 7, 2, 3, 4, 5, 6, 7, 3, 4, 5, 6, 7, 4, 5, 6, 7, 5, 6, 7, 6, 7, 7};
constexpr unsigned long long kA0 = pack3(kPairA, 0, 21), kA1 = pack3(kPairA, 21, 7);
constexpr unsigned long long kB0 = pack3(kPairB, 0, 21), kB1 = pack3(kPairB, 21, 7);

__device__ __forceinline__ int pair_a(int i) { return (int)((i < 21 ? kA0 >> (3 * i) : kA1 >> (3 * (i - 21))) & 7); }
__device__ __forceinline__ int pair_b(int i) { return (int)((i < 21 ? kB0 >> (3 * i) : kB1 >> (3 * (i - 21))) & 7); }

// Single-precision image of a double by truncating its significand; clears `ok`
// when the value is neither zero nor within [2^-60, 2^60] in magnitude.
__device__ __forceinline__ float image(double d, bool& ok) {
  const long long b = __double_as_longlong(d);
  const unsigned hi = (unsigned)((unsigned long long)b >> 32);
  const unsigned ahi = hi & 0x7FFFFFFFu;
  const unsigned e = ahi >> 20;
  const bool zero = (b & 0x7FFFFFFFFFFFFFFFLL) == 0;
  ok = ok && (zero || (e >= 1023u - 60u && e <= 1023u + 60u));
  return zero ? 0.0f : __uint_as_float((hi & 0x80000000u) | ((ahi - (896u << 20)) << 3));
}

__device__ __forceinline__ double exact_d2(const double* x, const double* y, const double* z, int a, int b) {
  const double dx = x[b] - x[a], dy = y[b] - y[a], dz = z[b] - z[a];
  return (dx * dx + dy * dy) + dz * dz;
}

__device__ __forceinline__ long long key_of(double d) {
  const long long b = __double_as_longlong(d);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}

__device__ __forceinline__ double key_decode(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}

// x, y, z: the element's node coordinates in registers; sx, sy, sz: the same
// values in per-thread memory (shared or local), indexed [lid * stride].
__device__ __forceinline__ double min_d2(const double* x, const double* y, const double* z,
                                         const double* sx, const double* sy, const double* sz, int stride) {
  bool ok = true;
  float fx[8], fy[8], fz[8];
  float M = 0.0f;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    fx[l] = image(x[l], ok);
    fy[l] = image(y[l], ok);
    fz[l] = image(z[l], ok);
    M = fmaxf(M, fmaxf(fabsf(fx[l]), fmaxf(fabsf(fy[l]), fabsf(fz[l]))));
  }
  long long kmin = 0x7FFFFFFFFFFFFFFFLL;
  if (ok && M >= 9.5367431640625e-07f) {  // 2^-20
    float e2[28];
    float e2min = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 28; ++i) {
      const int a = pair_a(i), b = pair_b(i);
      const float dx = fx[b] - fx[a], dy = fy[b] - fy[a], dz = fz[b] - fz[a];
      e2[i] = (dx * dx + dy * dy) + dz * dz;
      e2min = fminf(e2min, e2[i]);
    }
    const float E = 4.0e-6f * M;
    const float T = (sqrtf(e2min) + E) * (1.0f + 3.814697265625e-06f) + E;  // 2^-18
    const float T2 = T * T * (1.0f + 9.5367431640625e-07f);                 // 2^-20
    unsigned mask = 0;
#pragma unroll
    for (int i = 0; i < 28; ++i) mask |= (e2[i] <= T2 ? 1u : 0u) << i;
    while (mask) {
      const int i = __ffs((int)mask) - 1;
      mask &= mask - 1;
      const int a = pair_a(i) * stride, b = pair_b(i) * stride;
      const double dx = sx[b] - sx[a], dy = sy[b] - sy[a], dz = sz[b] - sz[a];
      const long long k = key_of((dx * dx + dy * dy) + dz * dz);
      kmin = k < kmin ? k : kmin;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 28; ++i) {
      const long long k = key_of(exact_d2(x, y, z, pair_a(i), pair_b(i)));
      kmin = k < kmin ? k : kmin;
    }
  }
  return key_decode(kmin);
}

}  // namespace cfl
