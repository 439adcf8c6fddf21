// Complex arithmetic on double2 (complex128) and float2 (complex64).
#pragma once
#include <cuda_runtime.h>

namespace bem2d_gpu {

template <typename T>
struct CTraits;
template <>
struct CTraits<double2> {
  typedef double R;
  static __device__ __forceinline__ double2 make(double a, double b) { return make_double2(a, b); }
};
template <>
struct CTraits<float2> {
  typedef float R;
  static __device__ __forceinline__ float2 make(float a, float b) { return make_float2(a, b); }
};

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
  return CTraits<T>::make(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c - a*b
template <typename T>
__device__ __forceinline__ T cfms(T c, T a, T b) {
  T r;
  r.x = fma(-a.x, b.x, fma(a.y, b.y, c.x));
  r.y = fma(-a.x, b.y, fma(-a.y, b.x, c.y));
  return r;
}
// c + a*b
template <typename T>
__device__ __forceinline__ T cfma(T a, T b, T c) {
  T r;
  r.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
  r.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
  return r;
}
template <typename T>
__device__ __forceinline__ T crcp(T a) {
  typedef typename CTraits<T>::R R;
  // 1/a with scaling against overflow/underflow of |a|^2
  const R s = fabs(a.x) + fabs(a.y);
  const R ar = a.x / s, ai = a.y / s;
  const R d = (ar * ar + ai * ai) * s;
  return CTraits<T>::make(ar / d, -ai / d);
}
template <typename T>
__device__ __forceinline__ typename CTraits<T>::R cabs1(T a) {
  return fabs(a.x) + fabs(a.y);
}

}  // namespace bem2d_gpu
