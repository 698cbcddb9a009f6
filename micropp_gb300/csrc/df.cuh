// df.cuh -- double-float arithmetic: a value held as the unevaluated sum hi + lo of two FP32 numbers.
//
// The FP64 pipe of sm_103a issues 2 operations per SM and cycle, the FP32 pipe 128.  Where a kernel needs more
// than FP32 accuracy but its operands are FP32 (the FP32 tangent times a double-float vector), the error-free
// transformations below keep about 48 bits with FP32 operations only:
//   two_sum  -- Knuth's TwoSum: s = fl(a + b) and the exact error e, a + b = s + e, for any a, b;
//   two_prod -- p = fl(a b) and e = a b - p exactly, by one fused multiply-add.
// The explicit-rounding intrinsics keep the compiler from contracting or reordering the steps.
#pragma once

#include <cuda_runtime.h>

namespace mgb {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (h, l) -= k (xh + xl): the product k xh is split exactly, its high part enters h by TwoSum, and every
// error term (the TwoSum error, the product's low part, k xl) collects in l.
__device__ __forceinline__ void df_sub_prod(float &h, float &l, float k, float xh, float xl) {
  const float p = __fmul_rn(k, xh);
  const float pe = __fmaf_rn(k, xh, -p);
  float s, t;
  two_sum(h, -p, s, t);
  h = s;
  l = __fmaf_rn(-k, xl, __fadd_rn(l, __fsub_rn(t, pe)));
}

// (h, l) += d, renormalised so that h = fl(h + l).
__device__ __forceinline__ void df_add(float &h, float &l, float d) {
  float s, t;
  two_sum(h, d, s, t);
  two_sum(s, __fadd_rn(t, l), h, l);
}

// A double as a double-float pair (hi = the nearest float, lo = the nearest float to the rest).
__device__ __forceinline__ void df_split(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// A double-float value and its arithmetic (Dekker; the "sloppy" addition: the error of a + b stays below about
// 2^-44 (|a| + |b|), which is what an FP64 sum of inexact terms guarantees too).
struct dfl {
  float h, l;
};

__device__ __forceinline__ dfl df_of(double v) {
  dfl r;
  df_split(v, r.h, r.l);
  return r;
}
__device__ __forceinline__ dfl df_of(float v) { return dfl{v, 0.f}; }
__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.h + (double)a.l; }

// s = fl(a + b), e = the exact error, for |a| >= |b| (or a = 0).
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfl{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl{-a.h, -a.l}; }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl operator*(dfl a, float b) {
  const float p = __fmul_rn(a.h, b);
  return fast_two_sum(p, __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p)));
}
// a / b: the FP32 quotient, corrected by one Newton step on the double-float remainder a - q b.
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q = __fdiv_rn(a.h, b.h);
  const dfl r = a - b * q;
  return fast_two_sum(q, __fdiv_rn(r.h, b.h));
}
// sqrt(a) for a >= 0 (0 otherwise): the FP32 root, corrected by one Newton step.
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.h > 0.f)) return dfl{0.f, 0.f};
  const float x = __fsqrt_rn(a.h);
  const float p = __fmul_rn(x, x);
  const float pe = __fmaf_rn(x, x, -p);
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.h, p), pe), a.l);
  return fast_two_sum(x, __fdiv_rn(d, __fadd_rn(x, x)));
}
__device__ __forceinline__ bool operator<(dfl a, dfl b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool operator<=(dfl a, dfl b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
__device__ __forceinline__ bool df_nonneg(dfl a) { return a.h > 0.f || (a.h == 0.f && a.l >= 0.f); }

}  // namespace mgb
