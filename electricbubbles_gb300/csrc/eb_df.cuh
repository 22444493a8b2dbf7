// Double-float arithmetic: a value is an unevaluated sum hi + lo of two floats
// (|lo| <= ulp(hi)/2), about 48 significant bits. On GB300 the FP32 pipes issue ~60x
// more operations per cycle than the FP64 pipe, so double-float work of ~10 FP32
// operations per FP64 operation runs several times faster than native FP64.
//
// Error-free transformations (Knuth's two-sum, Dekker's fast two-sum, the FMA two-
// product) written with the explicitly rounded intrinsics so that the compiler can
// neither contract a multiply into a later add nor reassociate.
#pragma once

#include <cuda_runtime.h>

struct dfl {
  float hi, lo;
};

// accumulator: running float sum s plus the collected low-order parts c
struct dfacc {
  float s, c;
};

__device__ __forceinline__ dfl dfl_make(float h, float l) { return dfl{h, l}; }

__device__ __forceinline__ dfl dfl_from_double(double x) {
  float h = __double2float_rn(x);
  return dfl{h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double dfl_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly
__device__ __forceinline__ dfl two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dfl{s, e};
}

// s + e = a + b exactly when |a| >= |b| (or a = 0)
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  return dfl{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl dfl_neg(dfl a) { return dfl{-a.hi, -a.lo}; }

__device__ __forceinline__ dfl dfl_add(dfl a, dfl b) {
  dfl s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dfl dfl_sub(dfl a, dfl b) { return dfl_add(a, dfl_neg(b)); }

__device__ __forceinline__ dfl dfl_mul(dfl a, dfl b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ dfl dfl_mul_f(dfl a, float b) {
  float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ dfl dfl_sqr(dfl a) {
  float p = __fmul_rn(a.hi, a.hi);
  float e = __fmaf_rn(a.hi, a.hi, -p);
  e = __fmaf_rn(__fmul_rn(2.0f, a.hi), a.lo, e);
  return fast_two_sum(p, e);
}

// 1/a: hardware reciprocal estimate (about 23 bits) and one Newton step in double-float
__device__ __forceinline__ dfl dfl_rcp(dfl a) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a.hi));
  float t = __fmaf_rn(-a.hi, r, 1.0f);  // 1 - a.hi r, exact to ~2^-47
  t = __fmaf_rn(-a.lo, r, t);
  return fast_two_sum(r, __fmul_rn(r, t));
}

__device__ __forceinline__ void acc_add(dfacc& a, float v) {
  dfl t = two_sum(a.s, v);
  a.s = t.hi;
  a.c = __fadd_rn(a.c, t.lo);
}

// a += x y
__device__ __forceinline__ void acc_prod(dfacc& a, dfl x, dfl y) {
  float p = __fmul_rn(x.hi, y.hi);
  float pe = __fmaf_rn(x.hi, y.hi, -p);
  pe = __fmaf_rn(x.hi, y.lo, pe);
  pe = __fmaf_rn(x.lo, y.hi, pe);
  acc_add(a, p);
  a.c = __fadd_rn(a.c, pe);
}

__device__ __forceinline__ void acc_dfl(dfacc& a, dfl x) {
  acc_add(a, x.hi);
  a.c = __fadd_rn(a.c, x.lo);
}

__device__ __forceinline__ dfl acc_value(dfacc a) { return fast_two_sum(a.s, a.c); }

// complex double-float
struct cdf {
  dfl x, y;
};

__device__ __forceinline__ cdf cdf_from_float4(float4 v) { return cdf{{v.x, v.y}, {v.z, v.w}}; }

__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
  return cdf{dfl_sub(dfl_mul(a.x, b.x), dfl_mul(a.y, b.y)), dfl_add(dfl_mul(a.x, b.y), dfl_mul(a.y, b.x))};
}

__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return cdf{dfl_add(a.x, b.x), dfl_add(a.y, b.y)}; }
