// df.cuh -- double-float arithmetic: a value held as the unevaluated sum hi + lo of two FP32 numbers.
//
// The FP64 pipe of sm_103a issues 2 operations per SM and cycle, the FP32 pipe 128.  Where a kernel needs more
// than FP32 accuracy but its operands are FP32 (the FP32 tangent times a double-float vector), the error-free
// transformations below keep about 46 bits (2^-44 relative) with FP32 operations only:
//   two_sum  -- Knuth's TwoSum: s = fl(a + b) and the exact error e, a + b = s + e, for any a, b;
//   two_prod -- p = fl(a b) and e = a b - p exactly, by one fused multiply-add.
// Every step is a correctly rounded FP32 operation that the compiler may neither contract nor reorder: the
// explicit-rounding intrinsics on the device.  The header also compiles as plain C++ (the CPU test of these
// operators, built without floating-point contraction), where the same steps are the plain operators.
#pragma once

#ifdef __CUDACC__
#include <cuda_runtime.h>
#define MGB_DF __host__ __device__ __forceinline__
#else
#include <cmath>
#define MGB_DF inline
#endif

namespace mgb {

MGB_DF float rn_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
MGB_DF float rn_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
MGB_DF float rn_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
MGB_DF float rn_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
MGB_DF float rn_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
MGB_DF float rn_sqrt(float a) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}

MGB_DF void two_sum(float a, float b, float &s, float &e) {
  s = rn_add(a, b);
  const float bb = rn_sub(s, a);
  e = rn_add(rn_sub(a, rn_sub(s, bb)), rn_sub(b, bb));
}

// (h, l) -= k (xh + xl): the product k xh is split exactly, its high part enters h by TwoSum, and every
// error term (the TwoSum error, the product's low part, k xl) collects in l.
MGB_DF void df_sub_prod(float &h, float &l, float k, float xh, float xl) {
  const float p = rn_mul(k, xh);
  const float pe = rn_fma(k, xh, -p);
  float s, t;
  two_sum(h, -p, s, t);
  h = s;
  l = rn_fma(-k, xl, rn_add(l, rn_sub(t, pe)));
}

// (h, l) += d, renormalised so that h = fl(h + l).
MGB_DF void df_add(float &h, float &l, float d) {
  float s, t;
  two_sum(h, d, s, t);
  two_sum(s, rn_add(t, l), h, l);
}

// A double as a double-float pair (hi = the nearest float, lo = the nearest float to the rest).
MGB_DF void df_split(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// A double-float value and its arithmetic (Dekker; the "sloppy" addition: the error of a + b stays below about
// 2^-44 (|a| + |b|), which is what an FP64 sum of inexact terms guarantees too).
struct dfl {
  float h, l;
};

MGB_DF dfl df_of(double v) {
  dfl r;
  df_split(v, r.h, r.l);
  return r;
}
MGB_DF dfl df_of(float v) { return dfl{v, 0.f}; }
MGB_DF double df_to_double(dfl a) { return (double)a.h + (double)a.l; }

// s = fl(a + b), e = the exact error, for |a| >= |b| (or a = 0).
MGB_DF dfl fast_two_sum(float a, float b) {
  const float s = rn_add(a, b);
  return dfl{s, rn_sub(b, rn_sub(s, a))};
}

MGB_DF dfl operator+(dfl a, dfl b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return fast_two_sum(s, rn_add(e, rn_add(a.l, b.l)));
}
MGB_DF dfl operator-(dfl a) { return dfl{-a.h, -a.l}; }
MGB_DF dfl operator-(dfl a, dfl b) { return a + (-b); }
MGB_DF dfl operator*(dfl a, dfl b) {
  const float p = rn_mul(a.h, b.h);
  float e = rn_fma(a.h, b.h, -p);
  e = rn_fma(a.h, b.l, rn_fma(a.l, b.h, e));
  return fast_two_sum(p, e);
}
MGB_DF dfl operator*(dfl a, float b) {
  const float p = rn_mul(a.h, b);
  return fast_two_sum(p, rn_fma(a.l, b, rn_fma(a.h, b, -p)));
}
// a / b: the FP32 quotient, corrected by one Newton step on the double-float remainder a - q b.
MGB_DF dfl operator/(dfl a, dfl b) {
  const float q = rn_div(a.h, b.h);
  const dfl r = a - b * q;
  return fast_two_sum(q, rn_div(r.h, b.h));
}
// sqrt(a) for a >= 0 (0 otherwise): the FP32 root, corrected by one Newton step.
MGB_DF dfl df_sqrt(dfl a) {
  if (!(a.h > 0.f)) return dfl{0.f, 0.f};
  const float x = rn_sqrt(a.h);
  const float p = rn_mul(x, x);
  const float pe = rn_fma(x, x, -p);
  const float d = rn_add(rn_sub(rn_sub(a.h, p), pe), a.l);
  return fast_two_sum(x, rn_div(d, rn_add(x, x)));
}
MGB_DF bool operator<(dfl a, dfl b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
MGB_DF bool operator<=(dfl a, dfl b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
MGB_DF bool df_nonneg(dfl a) { return a.h > 0.f || (a.h == 0.f && a.l >= 0.f); }

}  // namespace mgb
