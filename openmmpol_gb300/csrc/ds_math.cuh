// Double-single (float-float) arithmetic for the FP32-pipe kernels that must
// deliver FP64-level accuracy (ds_kernels.cu, grad_ds.cu).
//
// A value is the unevaluated sum h + l of two floats (~48-bit significand).
// Error-free transformations: Knuth's TwoSum, Dekker's FastTwoSum and the
// FMA-based TwoProd; the double-word algorithms follow the analysis of
// Joldes, Muller and Popescu (ACM TOMS 44(4), 2017).  Files using these
// functions are compiled with --fmad=false (every intended FMA is an
// explicit fmaf, no product is fused into a later addition) and -ftz=true.
#pragma once

#include <cuda_runtime.h>

namespace ommp {
namespace gpu {

struct dsf {
  float h, l;
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ dsf two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// s + e = a + b exactly when |a| >= |b| or a = 0 (Dekker)
__device__ __forceinline__ dsf fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
// x * y, double-single operands
__device__ __forceinline__ dsf ds_mul(dsf x, dsf y) {
  float p = x.h * y.h;
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dsf ds_sqr(dsf x) {
  float p = x.h * x.h;
  float e = fmaf(x.h, x.h, -p);
  e = fmaf(x.h + x.h, x.l, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dsf ds_mulf(dsf x, float y) {
  float p = x.h * y;
  float e = fmaf(x.h, y, -p);
  e = fmaf(x.l, y, e);
  return fast_two_sum(p, e);
}
// (ah + al) - (bh + bl): the hi difference is exact, the lo difference
// rounds once; absolute error ~2^-48 of the operands (coordinates)
__device__ __forceinline__ dsf ds_diff(float ah, float al, float bh, float bl) {
  dsf s = two_sum(ah, -bh);
  return fast_two_sum(s.h, s.l + (al - bl));
}
// 1/sqrt(a): FP32 estimate y, one Newton step y (1 + (1 - a y^2) / 2) with
// 1 - a y^2 formed in double-single (the estimate's 2^-22 error squares)
__device__ __forceinline__ dsf ds_rsqrt(dsf a) {
  float y = rsqrtf(a.h);
  float p = y * y;
  dsf y2{p, fmaf(y, y, -p)};
  dsf t = ds_mul(a, y2);
  float e = (1.0f - t.h) - t.l;  // 1 - t.h is exact: t.h is within 2^-21 of 1
  float c = (0.5f * y) * e;
  return fast_two_sum(y, c);
}
// acc += p_exact(x * y) with x, y double-single, lazily (acc.l collects the
// low-order parts; the caller renormalises)
__device__ __forceinline__ void acc_mul(float &ah, float &al, dsf x, dsf y) {
  float p = x.h * y.h;
  float q = fmaf(x.h, y.h, -p);
  q = fmaf(x.h, y.l, q);
  q = fmaf(x.l, y.h, q);
  dsf s = two_sum(ah, p);
  ah = s.h;
  al += s.l + q;
}

__device__ __forceinline__ dsf to_ds(double v) {
  float h = (float)v;
  return {h, (float)(v - (double)h)};
}

// sum of three double-single products a.b (a, b given as hi/lo floats)
__device__ __forceinline__ dsf ds_dot3(float ah0, float al0, float ah1, float al1, float ah2, float al2, dsf b0,
                                       dsf b1, dsf b2) {
  float q0 = ah0 * b0.h, q1 = ah1 * b1.h, q2 = ah2 * b2.h;
  float f0 = fmaf(al0, b0.h, fmaf(ah0, b0.l, fmaf(ah0, b0.h, -q0)));
  float f1 = fmaf(al1, b1.h, fmaf(ah1, b1.l, fmaf(ah1, b1.h, -q1)));
  float f2 = fmaf(al2, b2.h, fmaf(ah2, b2.l, fmaf(ah2, b2.h, -q2)));
  const dsf u1 = two_sum(q0, q1);
  const dsf u2 = two_sum(u1.h, q2);
  return fast_two_sum(u2.h, ((f0 + f1) + f2) + (u1.l + u2.l));
}
__device__ __forceinline__ dsf ds_add(dsf x, dsf y) {
  const dsf s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, s.l + (x.l + y.l));
}

// operators for generic formulas (every result renormalised)
__device__ __forceinline__ dsf operator+(dsf x, dsf y) { return ds_add(x, y); }
__device__ __forceinline__ dsf operator-(dsf x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dsf operator-(dsf x, dsf y) { return ds_add(x, -y); }
__device__ __forceinline__ dsf operator*(dsf x, dsf y) { return ds_mul(x, y); }
__device__ __forceinline__ dsf operator*(dsf x, float y) { return ds_mulf(x, y); }
__device__ __forceinline__ dsf operator*(float y, dsf x) { return ds_mulf(x, y); }
__device__ __forceinline__ dsf &operator+=(dsf &x, dsf y) { return x = ds_add(x, y); }
__device__ __forceinline__ dsf &operator-=(dsf &x, dsf y) { return x = ds_add(x, -y); }

}  // namespace gpu
}  // namespace ommp
