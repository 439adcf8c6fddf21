// Hankel functions of the first kind H0(z), H1(z) for a complex argument z:
// the evaluator behind complex wavenumbers, where the reference calls AMOS
// zbesh (lib/bem2d_mathroutines.cpp:44-75; kode = 1, unscaled).  The kernels
// evaluate z = k |x - y|, so z lies on the ray of arg k.
//
// Domain: Re z > 0 and -pi/3 <= arg z <= pi/2 (Im k >= -sqrt(3) Re k).
// Two pieces, FP64:
//   |z| <= 1.5   ascending series of J0, J1 and of the regular parts of Y0,
//                Y1 (A&S 9.1.10-9.1.13, complex principal logarithm);
//   |z| > 1.5    the Laplace-type integral behind Hankel's asymptotic
//                expansion (Watson, Theory of Bessel Functions, sec. 7.2)
//                  H_nu(z) = sqrt(2/(pi z)) e^{i(z - nu pi/2 - pi/4)}
//                            / Gamma(nu + 1/2)
//                            * int_0^inf e^{-u} u^{nu-1/2} (1 + iu/(2z))^{nu-1/2} du,
//                with u = v^2 written as an integral over the whole real
//                line of e^{-v^2} times an analytic function, evaluated by
//                the trapezoidal rule (geometric convergence in 1/h; the
//                step shrinks as |z| falls because the integrand's branch
//                point v^2 = 2iz approaches the real axis).
// H0 and H1 come out directly, not as J + iY, so there is no cancellation
// where H decays (Im z > 0).  Relative error against mpmath and against
// scipy.special.hankel1 (AMOS) <= 4e-15 (1 + |z|/50) over the domain (the
// |z| term is the conditioning of e^{iz} itself).
// The same source compiles for the host (accuracy tests) and the device.
#pragma once

#include "hankel.cuh"

namespace bem2d_gpu {

struct cd {
  double re, im;
};

__host__ __device__ __forceinline__ cd cd_mul(cd a, cd b) {
  return cd{fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re)};
}

__host__ __device__ __forceinline__ double exp_d(double x) {
#ifdef __CUDA_ARCH__
  return exp(x);
#else
  return std::exp(x);
#endif
}

// Principal square root of w (w not on the negative real axis).
__host__ __device__ __forceinline__ cd cd_sqrt(cd w) {
  const double m = sqrt(fma(w.re, w.re, w.im * w.im));
  if (w.re >= 0) {
    const double s = sqrt(0.5 * (m + w.re));
    return cd{s, w.im / (2 * s)};
  }
  const double t = sqrt(0.5 * (m - w.re));
  return cd{fabs(w.im) / (2 * t), w.im >= 0 ? t : -t};
}

constexpr double kEulerGamma = 0.57721566490153286061;
constexpr double kInvPi = 0.31830988618379067154;
constexpr double kSqrt2OverPi = 0.45015815807855303478;  // sqrt(2) / pi

// |z| <= 1.5: series.  q = z^2/4, t_m = (-q)^m / (m!)^2.
//   J0 = sum t_m                     J1 = (z/2) sum t_m / (m+1)
//   Y0 = (2/pi) [(ln(z/2) + gamma) J0 - sum_{m>=1} H_m t_m]
//   Y1 = -2/(pi z) + (2/pi) ln(z/2) J1
//        - (1/pi)(z/2) sum (H_m + H_{m+1} - 2 gamma) t_m / (m+1)
// (H_m the harmonic numbers).
__host__ __device__ __forceinline__ void hankel01_c_series(cd z, cd* h0, cd* h1) {
  const cd q = cd{0.25 * (z.re * z.re - z.im * z.im), 0.5 * z.re * z.im};
  cd t{1.0, 0.0};
  cd j0{0, 0}, j1{0, 0}, s0{0, 0}, s1{0, 0};
  double hm = 0.0;
#pragma unroll 1
  for (int m = 0; m < 12; ++m) {
    if (m > 0) hm += 1.0 / m;
    const double inv = 1.0 / (m + 1);
    const cd t1{t.re * inv, t.im * inv};
    j0.re += t.re;
    j0.im += t.im;
    j1.re += t1.re;
    j1.im += t1.im;
    s0.re -= hm * t.re;
    s0.im -= hm * t.im;
    const double c = 2 * hm + inv - 2 * kEulerGamma;
    s1.re = fma(c, t1.re, s1.re);
    s1.im = fma(c, t1.im, s1.im);
    // t <- t * (-q) / (m+1)^2
    const cd nt = cd_mul(t, q);
    t = cd{-nt.re * inv * inv, -nt.im * inv * inv};
  }
  const cd zh{0.5 * z.re, 0.5 * z.im};
  j1 = cd_mul(j1, zh);
  // ln(z/2) = ln|z/2| + i arg z
  const cd lz{log(sqrt(fma(zh.re, zh.re, zh.im * zh.im))), atan2(z.im, z.re)};
  const cd lg{lz.re + kEulerGamma, lz.im};
  const cd a0 = cd_mul(lg, j0);
  const cd y0{2 * kInvPi * (a0.re + s0.re), 2 * kInvPi * (a0.im + s0.im)};
  // -2/(pi z) = -2 conj(z) / (pi |z|^2)
  const double iz2 = 1.0 / fma(z.re, z.re, z.im * z.im);
  const cd a1 = cd_mul(lz, j1);
  const cd b1 = cd_mul(zh, s1);
  const cd y1{-2 * kInvPi * z.re * iz2 + 2 * kInvPi * a1.re - kInvPi * b1.re,
              2 * kInvPi * z.im * iz2 + 2 * kInvPi * a1.im - kInvPi * b1.im};
  // H = J + iY
  *h0 = cd{j0.re - y0.im, j0.im + y0.re};
  *h1 = cd{j1.re - y1.im, j1.im + y1.re};
}

// |z| > 1.5: trapezoidal rule with step h over v in [-6.5, 6.5] (e^{-v^2}
// below 5e-19 outside).  With c = i / (2z), s(v) = sqrt(1 + c v^2):
//   T0 = h sum e^{-v^2} / s(v),   T1 = h sum e^{-v^2} v^2 s(v)
//   H0 = (sqrt2/pi) e^{iz} z^{-1/2} e^{-i pi/4} T0
//   H1 = 2 (sqrt2/pi) e^{iz} z^{-1/2} e^{-3i pi/4} T1
__host__ __device__ __forceinline__ void hankel01_c_integral(cd z, double r, cd* h0, cd* h1) {
  const double h = r <= 3.0 ? 0.0625 : r <= 7.0 ? 0.125 : r <= 14.0 ? 0.25 : 0.5;
  const int nv = (int)(6.5 / h);
  const double iz2 = 1.0 / fma(z.re, z.re, z.im * z.im);
  // c = i/(2z) = i conj(z) / (2|z|^2) = (z.im, z.re) / (2|z|^2)
  const double cr = 0.5 * z.im * iz2, ci = 0.5 * z.re * iz2;
  double t0r = 0, t0i = 0, t1r = 0, t1i = 0;
#pragma unroll 1
  for (int j = 0; j <= nv; ++j) {
    const double v = j * h;
    const double t = v * v;
    const cd w{fma(t, cr, 1.0), t * ci};
    const cd s = cd_sqrt(w);
    const double e = exp_d(-t) * (j == 0 ? h : 2 * h);
    const double em = e / sqrt(fma(w.re, w.re, w.im * w.im));  // e / |s|^2
    t0r = fma(em, s.re, t0r);  // e conj(s) / |s|^2 = e / s
    t0i = fma(-em, s.im, t0i);
    const double et = e * t;
    t1r = fma(et, s.re, t1r);
    t1i = fma(et, s.im, t1i);
  }
  // p = (sqrt2/pi) e^{iz} / sqrt(z)
  const cd sz = cd_sqrt(z);
  double sn, cs;
  sincos_d(z.re, &sn, &cs);
  const double ez = exp_d(-z.im);
  const cd eiz{ez * cs, ez * sn};
  const double isz = 1.0 / fma(sz.re, sz.re, sz.im * sz.im);
  const cd rz{sz.re * isz, -sz.im * isz};  // 1 / sqrt(z)
  cd p = cd_mul(eiz, rz);
  p.re *= kSqrt2OverPi;
  p.im *= kSqrt2OverPi;
  // e^{-i pi/4} = (1 - i)/sqrt2, e^{-3i pi/4} = -(1 + i)/sqrt2
  const cd p0{kSqrtHalf * (p.re + p.im), kSqrtHalf * (p.im - p.re)};
  const cd p1{2 * kSqrtHalf * (p.im - p.re), -2 * kSqrtHalf * (p.re + p.im)};
  *h0 = cd_mul(p0, cd{t0r, t0i});
  *h1 = cd_mul(p1, cd{t1r, t1i});
}

// H0(z), H1(z) for Re z > 0, -pi/3 <= arg z <= pi/2.
__host__ __device__ __forceinline__ void hankel01_c(cd z, cd* h0, cd* h1) {
  const double r = sqrt(fma(z.re, z.re, z.im * z.im));
  if (r <= 1.5)
    hankel01_c_series(z, h0, h1);
  else
    hankel01_c_integral(z, r, h0, h1);
}

}  // namespace bem2d_gpu
