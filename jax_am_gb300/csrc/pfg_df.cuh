// Double-float ("DF") arithmetic in FP32 operations (internal): a value is
// the unevaluated sum h + l of two floats with |l| <= ulp(h) / 2, about 48
// significant bits.  The compensated temperature of the fused step uses it
// so that a 2000-step run tracks a float64 run to ~1e-6 K at T ~ 1e4 K
// while every arithmetic operation stays float32.
//
// Methods (published): Knuth's TwoSum and Dekker's Fast2Sum for exact sums,
// TwoProd through a fused multiply-add for exact products, Dekker's
// double-length division, and the exponential by Cody-Waite range reduction
// (x = k ln 2 + r, ln 2 split into three parts) with a Taylor series of
// exp(r), |r| <= ln(2)/2, evaluated by Horner's rule in DF.
//
// The sums below must not be reassociated; nvcc keeps IEEE order for
// additions (contraction only fuses a product into an add, which none of
// the error-free sums contain).
#pragma once

#include <cuda_runtime.h>

namespace pfg {

struct DF {
  float h, l;
};

__device__ __forceinline__ DF df_from(float a) { return DF{a, 0.f}; }

// s + e == a + b exactly
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return DF{s, (a - (s - bb)) + (b - bb)};
}
// s + e == a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  const float s = a + b;
  return DF{s, b - (s - a)};
}
// p + e == a * b exactly
__device__ __forceinline__ DF two_prod(float a, float b) {
  const float p = a * b;
  return DF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = two_sum(x.h, y.h);
  const DF t = two_sum(x.l, y.l);
  s.l += t.h;
  s = fast_two_sum(s.h, s.l);
  s.l += t.l;
  return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ DF df_add_f(DF x, float b) {
  DF s = two_sum(x.h, b);
  s.l += x.l;
  return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ DF df_neg(DF x) { return DF{-x.h, -x.l}; }
__device__ __forceinline__ DF df_sub(DF x, DF y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ DF df_mul(DF x, DF y) {
  DF p = two_prod(x.h, y.h);
  p.l = fmaf(x.h, y.l, fmaf(x.l, y.h, p.l));
  return fast_two_sum(p.h, p.l);
}
__device__ __forceinline__ DF df_mul_f(DF x, float b) {
  DF p = two_prod(x.h, b);
  p.l = fmaf(x.l, b, p.l);
  return fast_two_sum(p.h, p.l);
}
// x / y (IEEE float32 quotients of the leading parts, one correction step)
__device__ __forceinline__ DF df_div(DF x, DF y) {
  const float q1 = __fdiv_rn(x.h, y.h);
  const DF r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fdiv_rn(r.h, y.h);
  const DF q = fast_two_sum(q1, q2);
  const DF r2 = df_sub(x, df_mul(y, q));
  return df_add_f(q, __fdiv_rn(r2.h, y.h));
}

// x > c and x < c for a float c (h + l compared exactly: |l| <= ulp(h) / 2)
__device__ __forceinline__ bool df_gt(DF x, float c) { return x.h > c || (x.h == c && x.l > 0.f); }
__device__ __forceinline__ bool df_lt(DF x, float c) { return x.h < c || (x.h == c && x.l < 0.f); }

// exp(x) for x <= 0 (the Gaussian beam's argument).  Below -100 the value
// (< 4e-44) is returned as 0, as float32 holds nothing there.
__device__ __forceinline__ DF df_exp_neg(DF x) {
  if (x.h < -100.f) return DF{0.f, 0.f};
  // ln 2 = L1 + L2 + L3: L1 has 12 significant bits, so k * L1 is exact
  // for |k| < 2^12; L2, L3 carry the next 24 bits each
  constexpr float L1 = 0.693145751953125f;
  constexpr float L2 = 1.428606765330187e-06f;
  constexpr float L3 = 5.497923148104107e-14f;
  const float k = rintf(x.h * 1.4426950408889634f);
  DF r = two_sum(x.h, -k * L1);  // exact difference of nearby values
  r.l += x.l;
  r = fast_two_sum(r.h, r.l);
  r = df_add(r, two_prod(-k, L2));
  r = df_add_f(r, -k * L3);
  // Taylor series of exp(r) to r^13 / 13!, |r| <= 0.347: truncation < 1e-16
  DF s = DF{1.f / 6227020800.f, 0.f};  // 1/13!
  constexpr double kInvFact[13] = {1.0 / 479001600.0, 1.0 / 39916800.0, 1.0 / 3628800.0,
                                   1.0 / 362880.0,    1.0 / 40320.0,    1.0 / 5040.0,
                                   1.0 / 720.0,       1.0 / 120.0,      1.0 / 24.0,
                                   1.0 / 6.0,         1.0 / 2.0,        1.0,
                                   1.0};
#pragma unroll
  for (int i = 0; i < 13; ++i) {
    const float ch = (float)kInvFact[i];
    const float cl = (float)(kInvFact[i] - (double)ch);
    s = df_add(df_mul(s, r), DF{ch, cl});
  }
  // 2^k, k in [-145, 0]: two exact power-of-two scalings keep it normal
  const int ki = (int)k;
  const int k1 = ki / 2, k2 = ki - k1;
  s.h = ldexpf(ldexpf(s.h, k1), k2);
  s.l = ldexpf(ldexpf(s.l, k1), k2);
  return s;
}

}  // namespace pfg
