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
  const float p = a * b;
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

__host__ __device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

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
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}

__host__ __device__ __forceinline__ ff ff_sqr(ff a) {
  const float p = a.hi * a.hi;
  float e = fmaf(a.hi, a.hi, -p);
  e = fmaf(a.hi + a.hi, a.lo, e);
  return fast_two_sum(p, e);
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

// sqrt(a) = a * rsqrt(a)
__host__ __device__ __forceinline__ ff ff_sqrt(ff a) {
  const float y = sqrtf(a.hi);
  const ff y2 = two_prod(y, y);
  const ff d = ff_sub(a, y2);  // a - y^2, small
  return fast_two_sum(y, d.hi / (2.0f * y));
}

// 1/a: single-precision seed, one Newton step in ff
__host__ __device__ __forceinline__ ff ff_rcp(ff a) {
  const float y = 1.0f / a.hi;
  const ff ay = ff_mul_f(a, y);
  const float e = (1.0f - ay.hi) - ay.lo;
  return fast_two_sum(y, y * e);
}

}  // namespace bem2d_gpu
