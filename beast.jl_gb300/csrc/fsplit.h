// An FP64 value split into two floats with integer operations only: a ~= hi + lo to about
// 2^-47 relative.  GB300 runs FP64 instructions, conversions included, at a small fraction of
// its FP32 rate, so the refinement matvec of a c128 matrix reads each entry as FP64 bits and
// works on the FP32 pipes.
//   hi: the sign, the exponent and the top 23 stored mantissa bits (a truncation, so
//       |lo| < 2^-23 |hi|);
//   lo: the remaining 29 mantissa bits times 2^(e - 1075), truncated to 24 significant bits,
//       with the sign of a, built from the bits with integer instructions only.
// |a| < 2^-97 gives 0 + 0, and lo is dropped below |a| = 2^-74: absolute errors below 1e-29,
// far under the FP64 rounding of a matvec of boundary-element entries.  |a| >= 2^128 (not a
// BEM matrix entry) overflows to +-inf, so the matvec reports it instead of hiding it.  No
// branch converts (a conversion instruction, even on a path not taken, would be if-converted
// into every call and run on the FP64 pipe).  Host and device builds give identical bits.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FS_HD __host__ __device__ __forceinline__
#else
#define FS_HD inline
#endif

namespace fsplit {

FS_HD uint64_t bits64(double a) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(a);
#else
  uint64_t u;
  memcpy(&u, &a, 8);
  return u;
#endif
}
FS_HD float from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
FS_HD uint32_t to_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

// leading zeros of a nonzero 32-bit word
FS_HD int clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __clz((int)x);
#else
  return __builtin_clz(x);
#endif
}

// (hi, lo) of a
FS_HD void split_f64(double a, float* hi, float* lo) {
  const uint64_t u = bits64(a);
  const uint32_t top = (uint32_t)(u >> 32);
  const int e = (int)((top >> 20) & 0x7FF);
  const uint32_t sgn = top & 0x80000000u;
  if (e > 1150) {  // beyond the float range: +-inf, NaN stays NaN (bits, not a conversion)
    const bool nan = e == 2047 && (u & 0x000FFFFFFFFFFFFFull) != 0;
    *hi = from_bits(sgn | 0x7F800000u | (nan ? 0x00400000u : 0u));
    *lo = 0.f;
    return;
  }
  if (e < 926) {
    *hi = 0.f;
    *lo = 0.f;
    return;
  }
  *hi = from_bits(sgn | ((uint32_t)(e - 896) << 23) | (uint32_t)((u >> 29) & 0x7FFFFFu));
  *lo = 0.f;
  const uint32_t m = (uint32_t)(u & 0x1FFFFFFFu);
  if (m != 0) {
    // m = 2^p (1 + f): biased float exponent p + (e - 1075) + 127, mantissa the 23 bits below
    // the leading one (truncated); results below the normal float range are dropped
    const int p = 31 - clz32(m);
    const int be = p + e - 948;
    if (be >= 1) *lo = from_bits(sgn | ((uint32_t)be << 23) | (((m << (31 - p)) >> 8) & 0x7FFFFFu));
  }
}

}  // namespace fsplit

namespace fsplit {

// a double rounded to the nearest float (ties to even) with integer operations only: the same
// bits as the conversion instruction for results in the normal float range; results below it
// (|a| < 2^-126) become 0, results above it +-inf, NaN stays NaN
FS_HD float to_float_rn(double a) {
  const uint64_t u = bits64(a);
  const uint32_t top = (uint32_t)(u >> 32);
  const int e = (int)((top >> 20) & 0x7FF);
  const uint32_t sgn = top & 0x80000000u;
  if (e > 1150) return from_bits(sgn | 0x7F800000u | (e == 2047 && (u & 0x000FFFFFFFFFFFFFull) ? 0x00400000u : 0u));
  if (e < 897) return from_bits(sgn);
  uint32_t f = ((uint32_t)(e - 896) << 23) | (uint32_t)((u >> 29) & 0x7FFFFFu);
  const uint32_t r = (uint32_t)(u & 0x1FFFFFFFu);
  f += (r > 0x10000000u || (r == 0x10000000u && (f & 1u))) ? 1u : 0u;  // a carry into the exponent is right
  return from_bits(sgn | f);
}

// a float as a double with integer operations only (exact; subnormal floats, below 1.2e-38,
// become 0; infinities and NaN keep their class)
FS_HD double f2d(float f) {
  const uint32_t u = to_bits(f);
  const uint32_t e = (u >> 23) & 0xFF;
  const uint64_t s = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t b = e == 0 ? s : s | ((uint64_t)(e == 0xFF ? 2047u : e + 896) << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29);
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}

}  // namespace fsplit
