// Double-float ("double-word") arithmetic on the FP32 pipes: a value is an unevaluated sum h + l of two
// floats with |l| <= ulp(h) / 2, about 48 significant bits.
//
// The building blocks are the classical error-free transformations: TwoSum (Knuth), Fast2Sum (Dekker
// 1971) and the FMA-based exact product; the sum, product and quotient follow Joldes, Muller & Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word arithmetic" (ACM TOMS 2017):
// relative errors of a few units of 2^-48 each.  Every operation is written with the _rn intrinsics so
// that the compiler cannot contract a product and a sum into one FMA, which would break the error terms.
#pragma once

#include <cuda_runtime.h>

struct F2 {
  float h, l;
};

__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// Requires |a| >= |b| (or a == 0).
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ F2 df_from_double(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - double(h))};
}

__device__ __forceinline__ F2 df_neg(F2 x) { return {-x.h, -x.l}; }

// Accurate sum (Joldes et al., Algorithm 6).
__device__ __forceinline__ F2 df_add(F2 x, F2 y) {
  F2 s = two_sum(x.h, y.h);
  const F2 t = two_sum(x.l, y.l);
  s = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}

// Product: the exact FP32 product of the high parts by FMA plus the cross terms (Joldes et al., Algorithm 11).
__device__ __forceinline__ F2 df_mul(F2 x, F2 y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, e));
  return fast_two_sum(p, e);
}

// Product by a float.
__device__ __forceinline__ F2 df_mul_f(F2 x, float c) {
  const float p = __fmul_rn(x.h, c);
  const float e = __fmaf_rn(x.l, c, __fmaf_rn(x.h, c, -p));
  return fast_two_sum(p, e);
}

__device__ __forceinline__ F2 df_sqr(F2 x) {
  const float p = __fmul_rn(x.h, x.h);
  const float e = __fmaf_rn(__fadd_rn(x.h, x.h), x.l, __fmaf_rn(x.h, x.h, -p));
  return fast_two_sum(p, e);
}

// Square root of x > 0: the correctly rounded FP32 root and one Newton correction, (x - h^2) / (2h), whose
// residual the FMA gives exactly.
__device__ __forceinline__ F2 df_sqrt(F2 x) {
  const float h = __fsqrt_rn(x.h);
  const float e = __fadd_rn(__fmaf_rn(-h, h, x.h), x.l);
  return fast_two_sum(h, __fdiv_rn(e, __fadd_rn(h, h)));
}

// Quotient x / y: an FP32 quotient, the double-float remainder x - q y, and its FP32 quotient as correction.
__device__ __forceinline__ F2 df_div(F2 x, F2 y) {
  const float q1 = __fdiv_rn(x.h, y.h);
  const F2 r = df_add(x, df_neg(df_mul_f(y, q1)));
  return fast_two_sum(q1, __fdiv_rn(r.h, y.h));
}

// a - c for triple-float expansions (a0 + a1 + a2, c0 + c1 + c2), rounded once to double-float: the two
// leading differences are exact (TwoSum), so the result carries no absolute error from the operands'
// magnitude, only a few units of 2^-48 relative to the difference itself.
__device__ __forceinline__ F2 diff3(float a0, float a1, float a2, float c0, float c1, float c2) {
  const F2 s = two_sum(a0, -c0);
  const F2 t = two_sum(a1, -c1);
  const F2 p = two_sum(s.h, t.h);
  const float q = __fadd_rn(__fadd_rn(s.l, p.l), __fadd_rn(t.l, __fsub_rn(a2, c2)));
  return fast_two_sum(p.h, q);
}
