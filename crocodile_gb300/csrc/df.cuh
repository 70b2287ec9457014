// Double-float ("double-word") arithmetic on the FP32 units: a value is the
// unevaluated sum hi + lo of two floats (about 48 significant bits).  The
// building blocks are error-free transformations (two_sum after Knuth, the
// product error by FMA) and the pair sum and product of Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic" (ACM TOMS 2017): AccurateDWPlusDW and DWTimesDW
// with FMA.  Complex values carry two such pairs; in memory a float4
// (re.hi, re.lo, im.hi, im.lo), 16 bytes like a complex128.
#pragma once

#include <cuda_runtime.h>

#include "df_convert.h"

namespace cg {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  const df v = fast_two_sum(s.hi, s.lo + t.hi);
  return fast_two_sum(v.hi, t.lo + v.lo);
}

// Sloppy pair sum (SloppyDWPlusDW in the same paper): one two_sum of the
// high parts, the low parts added in single precision.  Its error is about
// 2u^2 (|x| + |y|), bounded normwise rather than relative to |x + y|, which is
// what an FFT's error analysis uses; 11 operations against 20.
__device__ __forceinline__ df df_add_fast(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}

__device__ __forceinline__ df df_neg(df x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}

struct cdf {
  df re, im;
};

__device__ __forceinline__ cdf cdf_add(const cdf &a, const cdf &b) {
  return {df_add(a.re, b.re), df_add(a.im, b.im)};
}
__device__ __forceinline__ cdf cdf_sub(const cdf &a, const cdf &b) {
  return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))};
}
__device__ __forceinline__ cdf cdf_mul(const cdf &a, const cdf &w) {
  return {df_add(df_mul(a.re, w.re), df_neg(df_mul(a.im, w.im))),
          df_add(df_mul(a.re, w.im), df_mul(a.im, w.re))};
}
// the butterfly forms: sloppy sums (normwise error bounds)
__device__ __forceinline__ cdf cdf_add_f(const cdf &a, const cdf &b) {
  return {df_add_fast(a.re, b.re), df_add_fast(a.im, b.im)};
}
__device__ __forceinline__ cdf cdf_sub_f(const cdf &a, const cdf &b) {
  return {df_add_fast(a.re, df_neg(b.re)), df_add_fast(a.im, df_neg(b.im))};
}
// x.hi y.hi + sg z.hi t.hi as an exact two_sum of the two rounded products,
// their rounding errors (FMA) and the four cross terms accumulated in one
// float, then one renormalisation: 19 operations against 25 for two df_mul
// and a sloppy sum, with the same kind of normwise bound
__device__ __forceinline__ df df_dot2(df x, df y, df z, df t, float sg) {
  const float p1 = x.hi * y.hi, p2 = sg * z.hi * t.hi;
  const float e1 = fmaf(x.hi, y.hi, -p1), e2 = fmaf(sg * z.hi, t.hi, -p2);
  const df s = two_sum(p1, p2);
  float c = s.lo + (e1 + e2);
  c = fmaf(x.hi, y.lo, c);
  c = fmaf(x.lo, y.hi, c);
  c = fmaf(sg * z.hi, t.lo, c);
  c = fmaf(sg * z.lo, t.hi, c);
  return fast_two_sum(s.hi, c);
}
__device__ __forceinline__ cdf cdf_mul_f(const cdf &a, const cdf &w) {
  return {df_dot2(a.re, w.re, a.im, w.im, -1.f), df_dot2(a.re, w.im, a.im, w.re, 1.f)};
}
// a times a real double-float
__device__ __forceinline__ cdf cdf_scale(const cdf &a, df w) {
  return {df_mul(a.re, w), df_mul(a.im, w)};
}

// FP64 <-> double-float at the edges of a pipeline, by integer operations on
// the bit patterns (df_convert.h): the same results as the FP64 forms
// (float)v, (float)(v - hi) and (double)hi + (double)lo without the FP64 pipe
__device__ __forceinline__ df df_split(double v) {
  df r;
  f64_split(v, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ double df_join(df v) { return f64_join(v.hi, v.lo); }

__device__ __forceinline__ cdf cdf_from(double2 v) { return {df_split(v.x), df_split(v.y)}; }
__device__ __forceinline__ double2 cdf_to(const cdf &v) {
  return make_double2(df_join(v.re), df_join(v.im));
}
__device__ __forceinline__ cdf cdf_load(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ float4 cdf_store(const cdf &v) {
  return make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
}

}  // namespace cg
