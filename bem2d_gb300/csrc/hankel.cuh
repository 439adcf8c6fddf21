// Hankel functions of the first kind H0(x) = J0 + i Y0 and H1(x) = J1 + i Y1
// for a real argument x > 0: the evaluator behind every kernel evaluation of
// the assembly (it replaces the reference's GSL J0/Y0/J1/Y1 calls,
// lib/bem2d_mathroutines.cpp:20-42).
//
// Three pieces (polynomial tables generated by gen_hankel.py with mpmath):
//   x <= 4      ascending-series form of the regular parts (A&S 9.1.10-13)
//   4 < x <= 8  modulus-phase form H_nu = sqrt(2/(pi x)) (P + iQ) e^{i(x-(2nu+1)pi/4)}
//   x > 8       same form, second interval (A&S 9.2.5-9.2.6)
// FP64 tables reach |error| <~ 2e-16 |H|; the FP32 tables ~ 1e-7 |H|.
// The same source compiles for the host (accuracy tests) and the device.
#pragma once

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#include <cmath>
using std::fma;
#endif

#include "hankel_coeffs.h"

namespace bem2d_gpu {

constexpr double kTwoOverPi = 0.63661977236758134308;
constexpr double kSqrtHalf = 0.70710678118654752440;

__host__ __device__ __forceinline__ void sincos_d(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
  sincos(x, s, c);
#else
  *s = std::sin(x);
  *c = std::cos(x);
#endif
}

// J0, Y0, J1, Y1 at x > 0 in FP64.
__host__ __device__ __forceinline__ void hankel01_d(double x, double* j0,
                                                    double* y0, double* j1,
                                                    double* y1) {
  if (x <= 4.0) {
    const double t = x * x * 0.125 - 1.0;
    const double a0 = hk_small_d_0(t), a1 = hk_small_d_1(t);
    const double b0 = hk_small_d_2(t), b1 = hk_small_d_3(t);
    const double lx = kTwoOverPi * log(x);
    const double jj1 = x * a1;
    *j0 = a0;
    *j1 = jj1;
    *y0 = fma(lx, a0, b0);
    *y1 = fma(lx, jj1, fma(x, b1, -kTwoOverPi / x));
    return;
  }
  const double ix = 1.0 / x;
  double p0, q0, p1, q1;
  if (x <= 8.0) {
    const double s = 16.0 * ix * ix;                   // (4/x)^2 in [1/4, 1]
    const double t = fma(s, 8.0 / 3.0, -5.0 / 3.0);    // 2 (s - 1/4)/(3/4) - 1
    const double q = 4.0 * ix;
    p0 = hk_mid_d_0(t);
    q0 = hk_mid_d_1(t) * q;
    p1 = hk_mid_d_2(t);
    q1 = hk_mid_d_3(t) * q;
  } else {
    const double s = 64.0 * ix * ix;                   // (8/x)^2 in (0, 1)
    const double t = fma(s, 2.0, -1.0);
    const double q = 8.0 * ix;
    p0 = hk_far_d_0(t);
    q0 = hk_far_d_1(t) * q;
    p1 = hk_far_d_2(t);
    q1 = hk_far_d_3(t) * q;
  }
  const double amp = sqrt(kTwoOverPi * ix);
  double sx, cx;
  sincos_d(x, &sx, &cx);
  // e^{i(x - pi/4)} = c + i s
  const double c = (cx + sx) * kSqrtHalf;
  const double s = (sx - cx) * kSqrtHalf;
  *j0 = amp * fma(p0, c, -q0 * s);
  *y0 = amp * fma(p0, s, q0 * c);
  // e^{i(x - 3pi/4)} = s - i c
  *j1 = amp * fma(p1, s, q1 * c);
  *y1 = amp * fma(q1, s, -p1 * c);
}

}  // namespace bem2d_gpu
