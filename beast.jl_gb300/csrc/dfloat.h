// Double-float arithmetic on the FP32 pipes: a value is an unevaluated pair hi + lo of floats
// with |lo| <= ulp(hi) / 2 (about 48 significant bits).  GB300 runs FP64 at a small
// fraction of its FP32 rate, so the far-pair Green's function evaluations that need more than
// FP32 are written in this arithmetic instead of FP64.
//
// Methods: Knuth's TwoSum and the FMA form of Dekker's TwoProd as error-free transforms, the
// pair sum / product of Hida, Li and Bailey's QD library (2001), one Newton step for the square
// root and the reciprocal, Cody and Waite's (1980) argument reduction by pi/32 with a 64-entry
// table of sin / cos(m pi/32) (generated by gen_dftables.py) and short Taylor polynomials on
// |t| <= pi/64.
//
// Every product and sum that must be rounded on its own is written with the non-contracting
// intrinsics on the device and compiled with -ffp-contract=off on the host, so that the host
// build (used by the CPU tests) and the device build give identical results.
#pragma once
#include <math.h>

#include "dftables.h"

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace dfl {

struct df {
  float hi, lo;
};

// sin(m pi/32) hi, lo, cos(m pi/32) hi, lo (per translation unit)
#if defined(__CUDACC__)
static __constant__ float sincos_tab_dev[64][4] = DF_SINCOS_TABLE_INIT;
#endif
static const float sincos_tab_host[64][4] = DF_SINCOS_TABLE_INIT;

#if defined(__CUDA_ARCH__)
DF_HD float add_rn(float a, float b) { return __fadd_rn(a, b); }
DF_HD float sub_rn(float a, float b) { return __fsub_rn(a, b); }
DF_HD float mul_rn(float a, float b) { return __fmul_rn(a, b); }
#else
DF_HD float add_rn(float a, float b) { return a + b; }
DF_HD float sub_rn(float a, float b) { return a - b; }
DF_HD float mul_rn(float a, float b) { return a * b; }
#endif

// s + e = a + b exactly
DF_HD df two_sum(float a, float b) {
  const float s = add_rn(a, b);
  const float bb = sub_rn(s, a);
  const float e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
  return {s, e};
}
// as two_sum for |a| >= |b|
DF_HD df fast_two_sum(float a, float b) {
  const float s = add_rn(a, b);
  return {s, sub_rn(b, sub_rn(s, a))};
}
// p + e = a b exactly
DF_HD df two_prod(float a, float b) {
  const float p = mul_rn(a, b);
  return {p, fmaf(a, b, -p)};
}

DF_HD df make(float hi) { return {hi, 0.f}; }
DF_HD df neg(df a) { return {-a.hi, -a.lo}; }
DF_HD df add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, add_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, add_rn(s.lo, t.lo));
}
DF_HD df add(df a, float b) {
  const df s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, add_rn(s.lo, a.lo));
}
DF_HD df sub(df a, df b) { return add(a, neg(b)); }
// the "sloppy" pair sum of Hida, Li and Bailey: error below about 2^-44 (|a| + |b|) instead
// of 2^-44 |a + b| -- for sums whose terms do not cancel to far below their size
DF_HD df adds(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, add_rn(s.lo, add_rn(a.lo, b.lo)));
}
DF_HD df subs(df a, df b) { return adds(a, neg(b)); }
// the pair sum left unnormalised (the low part collects the TwoSum error and both low parts,
// a few ulp of the larger high part at most): for a sum whose consumer is a pair product, a
// running sum or another such sum, which add the low parts in anyway
DF_HD df addu(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return {s.hi, add_rn(s.lo, add_rn(a.lo, b.lo))};
}
DF_HD df subu(df a, df b) { return addu(a, neg(b)); }
DF_HD df mul(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}
DF_HD df mul(df a, float b) {
  const df p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, fmaf(a.lo, b, p.lo));
}
// the pair product left unnormalised (|lo| up to about 1.5 ulp(hi) instead of 0.5): for a
// product whose consumer is a pair sum, a running sum or another product -- they add the low
// parts in anyway -- the final fast two-sum of mul is three additions spent for nothing
DF_HD df mulu(df a, df b) {
  const float p = mul_rn(a.hi, b.hi);
  return {p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)))};
}
DF_HD df mulu(df a, float b) {
  const float p = mul_rn(a.hi, b);
  return {p, fmaf(a.lo, b, fmaf(a.hi, b, -p))};
}
// exact scaling by a power of two
DF_HD df scale(df a, float p2) { return {mul_rn(a.hi, p2), mul_rn(a.lo, p2)}; }

// sqrt(a), a >= 0: one Newton correction of the FP32 root
DF_HD df sqrt(df a) {
  if (!(a.hi > 0.f)) return {0.f, 0.f};
  const float s = sqrtf(a.hi);
  const float e = add_rn(fmaf(-s, s, a.hi), a.lo);  // a - s^2
  return fast_two_sum(s, e / mul_rn(2.f, s));
}
// 1 / sqrt(a), a > 0: one Newton correction of the FP32 reciprocal square root,
// y = y0 + y0 (1 - a y0^2) / 2 with a y0^2 formed exactly enough in pairs (about 2^-44).  The
// FP32 start is the hardware estimate on the device and 1 / sqrtf on the host, so the two
// builds agree to the pair accuracy here rather than bit for bit.
DF_HD df rsqrt(df a) {
#if defined(__CUDA_ARCH__)
  const float y0 = rsqrtf(a.hi);
#else
  const float y0 = 1.f / sqrtf(a.hi);
#endif
  const df y2 = two_prod(y0, y0);
  const df ay2 = mulu(a, y2);
  const float e = add_rn(sub_rn(1.f, ay2.hi), -ay2.lo);  // 1 - a y0^2, about 2^-22
  return fast_two_sum(y0, mul_rn(mul_rn(y0, e), 0.5f));
}
// the same left unnormalised: the correction y0 (1 - a y0^2) / 2 is at most about 2 ulp of y0,
// for consumers that take pair products
DF_HD df rsqrtu(df a) {
#if defined(__CUDA_ARCH__)
  const float y0 = rsqrtf(a.hi);
#else
  const float y0 = 1.f / sqrtf(a.hi);
#endif
  const df y2 = two_prod(y0, y0);
  const df ay2 = mulu(a, y2);
  const float e = add_rn(sub_rn(1.f, ay2.hi), -ay2.lo);
  return {y0, mul_rn(mul_rn(y0, e), 0.5f)};
}
// 1 / a: one Newton correction of the FP32 reciprocal
DF_HD df rcp(df a) {
  const float r = 1.f / a.hi;
  const float e = fmaf(-r, a.lo, fmaf(-r, a.hi, 1.f));  // 1 - r a
  return fast_two_sum(r, mul_rn(r, e));
}

// sin and cos of th (|th| < 2^20): th = n pi/32 + t, |t| <= pi/64, then the angle sum with
// the table entry of m = n mod 64.  Absolute error below 1e-11 (about 6e-12, set by the FP32
// cubic term), independent of |th| over that range.
DF_HD void sincos(df th, df* s, df* c) {
#if defined(__CUDA_ARCH__)
  const float(*tab)[4] = sincos_tab_dev;
#else
  const float(*tab)[4] = sincos_tab_host;
#endif
  const float n = rintf(mul_rn(th.hi, DF_32_OVER_PI));
  df t = add(th, neg(two_prod(n, DF_PI32_0)));
  t = add(t, neg(two_prod(n, DF_PI32_1)));
  t = add(t, -mul_rn(n, DF_PI32_2));
  const int m = ((int)n) & 63;
  // sin t = t + t^3 (-1/6 + t^2/120 - t^4/5040), the cubic part in FP32 (|t^3/6| < 2e-5)
  const float t2 = mul_rn(t.hi, t.hi);
  const float q = fmaf(t2, fmaf(t2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f);
  const df st = add(t, mul_rn(mul_rn(t.hi, t2), q));
  // cos t = 1 - t^2/2 + t^4 (1/24 - t^2/720), t^2/2 as a pair
  const float r4 = mul_rn(mul_rn(t2, t2), fmaf(t2, -1.f / 720.f, 1.f / 24.f));
  const df ct = add(add(make(1.f), neg(scale(mul(t, t), 0.5f))), r4);
  const df sm = {tab[m][0], tab[m][1]}, cm = {tab[m][2], tab[m][3]};
  *s = add(mul(sm, ct), mul(cm, st));
  *c = sub(mul(cm, ct), mul(sm, st));
}

// sincos with the table of m pi/32 passed in (shared memory in a kernel: lanes read different
// entries), on fewer FP32 additions than sincos: th.hi - n C0 is exact (Sterbenz: th.hi and
// n C0 lie within a factor 2 of each other, or n = 0), the small rest (th.lo, the low parts
// of n pi/32) is summed in FP32, and the sums with one dominant term (t + its cubic term,
// 1 - t^2/2) are fast two-sums.  Absolute error below 1e-11 for |th| < 2^10.
// NORM = false: the angle sum left unnormalised (addu) for consumers that take pair products
template <bool NORM = true>
DF_HD void sincos_tab(df th, const float (*tab)[4], df* s, df* c) {
  const float n = rintf(mul_rn(th.hi, DF_32_OVER_PI));
  const df p0 = two_prod(n, DF_PI32_0);
  const float s0 = sub_rn(th.hi, p0.hi);
  float e = sub_rn(th.lo, p0.lo);
  e = fmaf(-n, DF_PI32_1, e);
  e = fmaf(-n, DF_PI32_2, e);
  const df t = two_sum(s0, e);
  const int m = ((int)n) & 63;
  const float t2 = mul_rn(t.hi, t.hi);
  const float q = fmaf(t2, fmaf(t2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f);
  const df st = fast_two_sum(t.hi, add_rn(t.lo, mul_rn(mul_rn(t.hi, t2), q)));
  const float r4 = mul_rn(mul_rn(t2, t2), fmaf(t2, -1.f / 720.f, 1.f / 24.f));
  const df h = scale(mulu(t, t), 0.5f);  // t^2 / 2 < 1.2e-3
  const df c1 = fast_two_sum(1.f, -h.hi);
  // unnormalised: the low part (c1's, the quartic term and h's low part) is a few ulp of 1
  const df ct = NORM ? fast_two_sum(c1.hi, add_rn(c1.lo, sub_rn(r4, h.lo)))
                     : df{c1.hi, add_rn(c1.lo, sub_rn(r4, h.lo))};
  const df sm = {tab[m][0], tab[m][1]}, cm = {tab[m][2], tab[m][3]};
  if (NORM) {
    *s = adds(mulu(sm, ct), mulu(cm, st));
    *c = subs(mulu(cm, ct), mulu(sm, st));
  } else {
    *s = addu(mulu(sm, ct), mulu(cm, st));
    *c = subu(mulu(cm, ct), mulu(sm, st));
  }
}

// a += x for a running sum whose low part is normalised only at the end (norm): one TwoSum
// of the high parts and two plain additions instead of the sloppy sum's three more
DF_HD void acc(df& a, df x) {
  const df s = two_sum(a.hi, x.hi);
  a.hi = s.hi;
  a.lo = add_rn(a.lo, add_rn(s.lo, x.lo));
}
DF_HD df norm(df a) { return fast_two_sum(a.hi, a.lo); }

// Helmholtz / Maxwell Green's function exp(-i k R) / (4 pi R) for a real wavenumber k
DF_HD void green(df R, df k, df* re, df* im) {
  df s, c;
  sincos(mul(k, R), &s, &c);
  const df a = mul(rcp(R), df{DF_I4PI_HI, DF_I4PI_LO});
  *re = mul(a, c);
  *im = neg(mul(a, s));
}

// |x - y| for x - y = d + v given as pairs per component
DF_HD df norm3(df x, df y, df z) { return sqrt(add(add(mul(x, x), mul(y, y)), mul(z, z))); }

}  // namespace dfl
