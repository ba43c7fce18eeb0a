// Double-float arithmetic: a value is the unevaluated sum h + l of two floats (about 48
// significant bits). GB300 runs FP64 at 1/64 of its FP32 rate, so FP64-accuracy arithmetic in
// hot loops is done this way on the FP32 pipes. The building blocks are the published
// error-free transformations -- Knuth's TwoSum, Dekker's FastTwoSum, the FMA form of TwoProduct
// -- combined as in the double-double algorithms of Hida, Li and Bailey (accurate addition,
// multiplication with cross terms, division by long division). All operations use the
// explicitly rounded intrinsics so that the compiler cannot contract or reassociate them.
#pragma once

namespace gmm {

struct dfloat {
  float h, l;
};

__device__ __forceinline__ dfloat df_make(float h) { return {h, 0.0f}; }

__device__ __forceinline__ dfloat df_from_double(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to_double(dfloat a) { return (double)a.h + (double)a.l; }

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
  float s1, s2, t1, t2;
  df_two_sum(a.h, b.h, s1, s2);
  df_two_sum(a.l, b.l, t1, t2);
  s2 = __fadd_rn(s2, t1);
  df_fast_two_sum(s1, s2, s1, s2);
  s2 = __fadd_rn(s2, t2);
  df_fast_two_sum(s1, s2, s1, s2);
  return {s1, s2};
}

__device__ __forceinline__ dfloat df_neg(dfloat a) { return {-a.h, -a.l}; }

__device__ __forceinline__ dfloat df_sub(dfloat a, dfloat b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);  // exact low part of a.h * b.h
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  dfloat r;
  df_fast_two_sum(p, e, r.h, r.l);
  return r;
}

// a - f * b, the update of an elimination step
__device__ __forceinline__ dfloat df_sub_mul(dfloat a, dfloat f, dfloat b) { return df_sub(a, df_mul(f, b)); }

// a / b by long division: three float quotient digits, each from the remainder of the last
__device__ __forceinline__ dfloat df_div(dfloat a, dfloat b) {
  const float q1 = __fdiv_rn(a.h, b.h);
  dfloat r = df_sub(a, df_mul(df_make(q1), b));
  const float q2 = __fdiv_rn(r.h, b.h);
  r = df_sub(r, df_mul(df_make(q2), b));
  const float q3 = __fdiv_rn(r.h, b.h);
  dfloat q;
  df_fast_two_sum(q1, q2, q.h, q.l);
  return df_add(q, df_make(q3));
}

}  // namespace gmm
