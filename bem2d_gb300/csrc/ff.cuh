// Compensated single-single ("float-float") arithmetic: a value is the
// unevaluated sum hi + lo of two floats, |lo| <= ulp(hi)/2, about 48
// significant bits.  It runs on the FP32 pipe, which on GB300 issues 64x the
// FMA lanes of the FP64 pipe.  Error-free transformations after Knuth
// (two-sum), Dekker (fast two-sum) and the FMA-based two-product; the
// operation set follows Dekker, "A floating-point technique for extending the
// available precision" (1971) and Hida, Li & Bailey's double-double library
// (2001), written here for float pairs.
#pragma once

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#include <cmath>
using std::fmaf;
#endif

namespace bem2d_gpu {

struct ff {
  float hi, lo;
};

__host__ __device__ __forceinline__ ff ff_make(float h, float l) {
  ff r;
  r.hi = h;
  r.lo = l;
  return r;
}

// Round-to-nearest product that the compiler may not contract into a later
// add (an error-free transformation needs the rounded product itself).
__host__ __device__ __forceinline__ float f_mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// s + e = a + b exactly (any magnitudes)
__host__ __device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return ff_make(s, e);
}

// s + e = a + b exactly, requires |a| >= |b| (or a == 0)
__host__ __device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return ff_make(s, e);
}

// p + e = a * b exactly
__host__ __device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = f_mul_rn(a, b);
  const float e = fmaf(a, b, -p);
  return ff_make(p, e);
}

__host__ __device__ __forceinline__ ff ff_from_double(double d) {
  const float h = (float)d;
  return ff_make(h, (float)(d - (double)h));
}

__host__ __device__ __forceinline__ double ff_to_double(ff a) {
  return (double)a.hi + (double)a.lo;
}

__host__ __device__ __forceinline__ ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }

// accurate addition (relative error ~2^-46 even under cancellation)
__host__ __device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const ff t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}

// addition without the low-part two-sum: accurate unless a and b nearly cancel
__host__ __device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ ff ff_add_f(ff a, float b) {
  ff s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = f_mul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// a b + c d: both hi products exact (FMA residuals), their sum by a two-sum,
// the residuals and cross terms into the low part, one normalisation.  The
// error is ~2^-47 max(|a b|, |c d|), as ff_add_fast(ff_mul(a, b), ff_mul(c,
// d)), in fewer operations.
__host__ __device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d) {
  const float p = f_mul_rn(a.hi, b.hi);
  const float q = f_mul_rn(c.hi, d.hi);
  float e1 = fmaf(a.hi, b.hi, -p);
  e1 = fmaf(a.hi, b.lo, e1);
  e1 = fmaf(a.lo, b.hi, e1);
  float e2 = fmaf(c.hi, d.hi, -q);
  e2 = fmaf(c.hi, d.lo, e2);
  e2 = fmaf(c.lo, d.hi, e2);
  const ff s = two_sum(p, q);
  return fast_two_sum(s.hi, s.lo + (e1 + e2));
}

__host__ __device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const float p = f_mul_rn(a.hi, b);
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ ff ff_sqr(ff a) {
  const float p = f_mul_rn(a.hi, a.hi);
  float e = fmaf(a.hi, a.hi, -p);
  e = fmaf(a.hi + a.hi, a.lo, e);
  return fast_two_sum(p, e);
}

// One Horner step c + t y when |c.hi| >= |t y| is known in advance (the
// polynomial generator checks |c_k| >= sum_{j>k} |c_j| for |t| <= 1): the
// product is left unnormalised and c.hi + p is split by a fast two-sum.
// Same accuracy as ff_add_fast(c, ff_mul(t, y)), fewer operations.
__host__ __device__ __forceinline__ ff ff_horner_fast(ff c, ff t, ff y) {
  const float p = f_mul_rn(t.hi, y.hi);
  float e = fmaf(t.hi, y.hi, -p);
  e = fmaf(t.hi, y.lo, e);
  e = fmaf(t.lo, y.hi, e);
  const float s = c.hi + p;
  const float err = p - (s - c.hi);
  return fast_two_sum(s, err + (e + c.lo));
}

// exact scaling by a power of two
__host__ __device__ __forceinline__ ff ff_scale2(ff a, float p2) {
  return ff_make(a.hi * p2, a.lo * p2);
}

__host__ __device__ __forceinline__ float f_rsqrt(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.0f / std::sqrt(x);
#endif
}

// 1/sqrt(a): single-precision seed and one Newton step carried in ff
// (y1 = y + y (1 - a y^2) / 2; quadratic convergence from ~1e-7).
__host__ __device__ __forceinline__ ff ff_rsqrt(ff a) {
  const float y = f_rsqrt(a.hi);
  const ff y2 = two_prod(y, y);
  const ff ay2 = ff_mul(a, y2);
  const float e = (1.0f - ay2.hi) - ay2.lo;  // 1 - a y^2, small
  return fast_two_sum(y, 0.5f * y * e);
}

// 1/a: single-precision seed, one Newton step in ff
__host__ __device__ __forceinline__ ff ff_rcp(ff a) {
  const float y = 1.0f / a.hi;
  const ff ay = ff_mul_f(a, y);
  const float e = (1.0f - ay.hi) - ay.lo;
  return fast_two_sum(y, y * e);
}

// Natural logarithm of a > 0 (normal hi part).  a = 2^e m with m in
// [sqrt(1/2), sqrt(2)); log m = 2 atanh(u) = 2 (u + u^3/3 + u^5/5 + ...),
// u = (m - 1)/(m + 1), |u| <= 0.172, so u^2 <= 0.0295.  m - 1 is exact
// (Sterbenz), which keeps the relative accuracy of log m near m = 1.  The
// series terms through u^8/9 are carried in ff (each coefficient bounds the
// rest of the series, so the fast Horner step applies), the rest (below
// 2e-9) in FP32; log 2 is the ff pair nearest to it.
__host__ __device__ __forceinline__ ff ff_log(ff a) {
  int e;
  float m = frexpf(a.hi, &e);  // a.hi = m 2^e, m in [1/2, 1)
  if (m < 0.70710678f) {
    m *= 2.0f;
    --e;
  }
  const float ml = ldexpf(a.lo, -e);
  const ff num = two_sum(m - 1.0f, ml);
  const ff den = ff_add_f(two_sum(m, 1.0f), ml);
  const ff u = ff_mul(num, ff_rcp(den));
  const ff u2 = ff_sqr(u);
  const float v = u2.hi;
  const float tail =
      v * fmaf(v, fmaf(v, fmaf(v, fmaf(v, fmaf(v, fmaf(v, 1.0f / 25.0f, 1.0f / 23.0f),
                                                 1.0f / 21.0f), 1.0f / 19.0f), 1.0f / 17.0f),
                         1.0f / 15.0f), 1.0f / 13.0f) + 1.0f / 11.0f;
  ff s = ff_add_f(ff_make(0.1111111119389534f, -8.278422947149977e-10f), v * tail);  // 1/9
  s = ff_horner_fast(ff_make(0.1428571492433548f, -6.38621200366174e-09f), u2, s);  // 1/7
  s = ff_horner_fast(ff_make(0.20000000298023224f, -2.9802322831784522e-09f), u2, s);  // 1/5
  s = ff_horner_fast(ff_make(0.3333333432674408f, -9.934107758624577e-09f), u2, s);     // 1/3
  s = ff_horner_fast(ff_make(1.0f, 0.0f), u2, s);
  const ff lm = ff_mul(ff_scale2(u, 2.0f), s);
  const ff l2 = ff_mul_f(ff_make(0.6931471824645996f, -1.9046542121259336e-09f), (float)e);
  return ff_add(l2, lm);
}

}  // namespace bem2d_gpu
