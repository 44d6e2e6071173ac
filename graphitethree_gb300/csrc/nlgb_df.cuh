// nlgb_df.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)
// (about 48 significand bits, FP32's exponent range).  GB300 executes FP32
// at ~64x its FP64 rate, so a Krylov iteration written in double-float is
// bound by HBM instead of by the FP64 pipe, at 8 bytes per value like FP64.
//
// The algorithms are the classical error-free transformations: Knuth's
// TwoSum, Dekker's Fast2Sum, and the FMA TwoProduct, composed as Dekker's
// (1971) double-length addition and multiplication (the "sloppy" addition of
// Hida, Li & Bailey's QD library, 2001).  Each step is written with
// explicitly rounded operations so that the compiler can neither contract
// a*b + c into an FMA nor reassociate a sum: the error terms are exact only
// as written.  The same code compiles for the host (tests), built with
// -ffp-contract=off.
#pragma once
#include <vector_types.h>
#if defined(__CUDACC__)
#define NLGB_DF_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define NLGB_DF_HD inline
#endif

namespace nlgb {
namespace df {

NLGB_DF_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
NLGB_DF_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
NLGB_DF_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
NLGB_DF_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

NLGB_DF_HD float2 make(float hi, float lo) {
  float2 v;
  v.x = hi;
  v.y = lo;
  return v;
}

// s + e == a + b exactly (Knuth); commutative: the error of a rounded sum is
// unique, so two_sum(a, b) and two_sum(b, a) are identical.
NLGB_DF_HD float2 two_sum(float a, float b) {
  const float s = add(a, b);
  const float bb = sub(s, a);
  const float e = add(sub(a, sub(s, bb)), sub(b, bb));
  return make(s, e);
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker).
NLGB_DF_HD float2 fast_two_sum(float a, float b) {
  const float s = add(a, b);
  return make(s, sub(b, sub(s, a)));
}

// a + b (Dekker's double-length addition).  Commutative.
NLGB_DF_HD float2 dadd(float2 a, float2 b) {
  const float2 t = two_sum(a.x, b.x);
  return fast_two_sum(t.x, add(t.y, add(a.y, b.y)));
}

// a * b (TwoProduct of the heads plus the cross terms; lo * lo is below the
// format's precision).
NLGB_DF_HD float2 dmul(float2 a, float2 b) {
  const float p = mul(a.x, b.x);
  float e = fma(a.x, b.x, -p);
  e = fma(a.x, b.y, e);
  e = fma(a.y, b.x, e);
  return fast_two_sum(p, e);
}

// acc + a * b: the product's (head, tail) enters the addition unnormalised.
NLGB_DF_HD float2 mac(float2 acc, float2 a, float2 b) {
  const float p = mul(a.x, b.x);
  float e = fma(a.x, b.x, -p);
  e = fma(a.x, b.y, e);
  e = fma(a.y, b.x, e);
  const float2 t = two_sum(acc.x, p);
  return fast_two_sum(t.x, add(t.y, add(acc.y, e)));
}

NLGB_DF_HD float2 neg(float2 a) { return make(-a.x, -a.y); }

// Nearest float head, then the rounded remainder (exact when d's
// significand fits in 48 bits and both parts are normal floats).
NLGB_DF_HD float2 from_double(double d) {
  const float hi = (float)d;
  return make(hi, (float)(d - (double)hi));
}

NLGB_DF_HD double to_double(float2 a) { return (double)a.x + (double)a.y; }

}  // namespace df
}  // namespace nlgb
