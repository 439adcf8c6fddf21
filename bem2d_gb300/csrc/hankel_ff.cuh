// Kernel evaluation in float-float arithmetic (FP32 pipe).  For arguments
// x = k d >= 4: H0 and H1 in modulus-phase form
//   H_nu(x) = sqrt(2/(pi x)) (P_nu + i Q_nu) e^{i(x - (2 nu + 1) pi/4)}
// with P, Q from hankel_ff_coeffs.h (four intervals of x), and e^{i(x-pi/4)}
// from a Cody-Waite reduction modulo 2 pi/64 plus short Taylor polynomials
// around a 64-entry table of e^{i(2 pi j/64 - pi/4)}.  Accuracy ~1e-14
// relative to |H|.  bessel01_ff adds the small arguments (x <= 4) from the
// power-series form.  The same source builds on the host for accuracy tests.
#pragma once

#include "ff.cuh"
#include "hankel_ff_coeffs.h"

namespace bem2d_gpu {

struct ffc {
  ff re, im;
};

// 2 pi / 64 = C1 + C2 + C3 (C1, C2 single-precision, C3 the rest)
constexpr float kRedC1 = 0.09817477315664291f;
constexpr float kRedC2 = -2.7319617679211206e-09f;
constexpr float kRedC3 = -1.0719528187536762e-16f;
constexpr float kRedInv = 10.18591594696045f;  // 64 / (2 pi)

// 1 - a and 1/2 - a for |a| <= 1/4: the head by a fast two-sum (exact), the
// low part left unnormalised (|lo| stays a few ulps of hi, which the ff
// products that consume these values accept)
__host__ __device__ __forceinline__ ff ff_one_minus(ff a) {
  const ff s = fast_two_sum(1.0f, -a.hi);
  return ff_make(s.hi, s.lo - a.lo);
}
__host__ __device__ __forceinline__ ff ff_half_minus(ff a) {
  const ff s = fast_two_sum(0.5f, -a.hi);
  return ff_make(s.hi, s.lo - a.lo);
}

// e^{i(x - pi/4)} for x > 0 (ff), table tab[j] = (cos, sin)(2 pi j/64 - pi/4)
// as ff pairs: tab[4 j] = cos.hi, tab[4 j + 1] = cos.lo, [+2], [+3] = sin.
// Only the absolute error matters (|E| = 1): ~1e-16 plus x 2^-48 from x
// itself.
__host__ __device__ __forceinline__ ffc expi_ff(ff x, const float* tab) {
  const float j = rintf(x.hi * kRedInv);
  const float r1 = fmaf(-j, kRedC1, x.hi);  // exact
  // r = r1 + x.lo - j C2 - j C3: the two larger small terms by two-sums,
  // the rounding errors, j C2's low part and j C3 into the low part
  const ff p = two_prod(j, kRedC2);
  const ff s1 = two_sum(r1, x.lo);
  const ff s2 = two_sum(s1.hi, -p.hi);
  const ff r = fast_two_sum(s2.hi, fmaf(-j, kRedC3, (s1.lo + s2.lo) - p.lo));
  const int idx = ((int)j) & 63;
  const ff r2 = ff_sqr(r);  // |r| <= pi/64, r^2 <= 2.5e-3
  // sin r = r (1 - r^2 S), S = 1/6 - r^2/120 + r^4/5040
  const float st = r2.hi * fmaf(r2.hi, 1.0f / 5040.0f, -1.0f / 120.0f);
  const ff S = ff_add_f(ff_make(0.1666666716337204f, -4.967053879312289e-09f), st);
  const ff sinr = ff_mul(r, ff_one_minus(ff_mul(r2, S)));
  // cos r = 1 - r^2 C, C = 1/2 - r^2 D, D = 1/24 - r^2/720 + r^4/40320
  const float dt = r2.hi * fmaf(r2.hi, 1.0f / 40320.0f, -1.0f / 720.0f);
  const ff D = ff_add_f(ff_make(0.0416666679084301f, -1.2417634698280722e-09f), dt);
  const ff cosr = ff_one_minus(ff_mul(r2, ff_half_minus(ff_mul(r2, D))));
  const ff ca = ff_make(tab[4 * idx], tab[4 * idx + 1]);
  const ff sa = ff_make(tab[4 * idx + 2], tab[4 * idx + 3]);
  ffc e;
  e.re = ff_dot2(ca, cosr, ff_neg(sa), sinr);
  e.im = ff_dot2(sa, cosr, ca, sinr);
  return e;
}

// P0, Q0, P1, Q1 at x >= 4 given ix = 1/x.
__host__ __device__ __forceinline__ void pq_ff(float xhi, ff ix, ff* p0, ff* q0, ff* p1,
                                               ff* q1) {
  const ff ix2 = ff_sqr(ix);
  if (xhi < 8.0f) {
    const ff s = ff_scale2(ix2, 16.0f);  // (4/x)^2 in (1/4, 1]
    const ff tt = ff_add_fast(ff_mul(s, ff_make(2.6666667461395264f, -7.947286206899662e-08f)),
                              ff_make(-1.6666666269302368f, -3.973643103449831e-08f));
    const ff q = ff_scale2(ix, 4.0f);
    *p0 = hkff_3_0(tt);
    *q0 = ff_mul(hkff_3_1(tt), q);
    *p1 = hkff_3_2(tt);
    *q1 = ff_mul(hkff_3_3(tt), q);
  } else if (xhi < 16.0f) {
    const ff s = ff_scale2(ix2, 64.0f);  // (8/x)^2 in [1/4, 1]
    // t = 2 (s - 1/4) / (3/4) - 1 = (8/3) s - 5/3
    const ff tt = ff_add_fast(ff_mul(s, ff_make(2.6666667461395264f, -7.947286206899662e-08f)),
                              ff_make(-1.6666666269302368f, -3.973643103449831e-08f));
    const ff q = ff_scale2(ix, 8.0f);
    *p0 = hkff_0_0(tt);
    *q0 = ff_mul(hkff_0_1(tt), q);
    *p1 = hkff_0_2(tt);
    *q1 = ff_mul(hkff_0_3(tt), q);
  } else if (xhi < 64.0f) {
    const ff s = ff_scale2(ix2, 256.0f);  // (16/x)^2 in [1/16, 1]
    // t = (32 s - 17) / 15
    const ff t = ff_mul(ff_add_f(ff_scale2(s, 32.0f), -17.0f),
                        ff_make(0.06666667014360428f, -3.47693762670076e-09f));
    const ff q = ff_scale2(ix, 16.0f);
    *p0 = hkff_1_0(t);
    *q0 = ff_mul(hkff_1_1(t), q);
    *p1 = hkff_1_2(t);
    *q1 = ff_mul(hkff_1_3(t), q);
  } else {
    const ff s = ff_scale2(ix2, 4096.0f);  // (64/x)^2 in (0, 1]
    const ff t = ff_add_f(ff_scale2(s, 2.0f), -1.0f);
    const ff q = ff_scale2(ix, 64.0f);
    *p0 = hkff_2_0(t);
    *q0 = ff_mul(hkff_2_1(t), q);
    *p1 = hkff_2_2(t);
    *q1 = ff_mul(hkff_2_3(t), q);
  }
}

struct BesselFF {
  ff j0, y0, j1, y1;
};

// J0, Y0, J1, Y1 at any x > 0 given x and ix = 1/x.  x <= 4: the
// power-series form (A&S 9.1.10-9.1.13) with the regular parts A0, A1, B0,
// B1 as polynomials in t = x^2/8 - 1 and the logarithm from ff_log; x > 4:
// the modulus-phase form above.  Absolute accuracy ~1e-14 of max(1, |H|).
__host__ __device__ __forceinline__ BesselFF bessel01_ff(ff x, ff ix, const float* tab) {
  BesselFF r;
  if (x.hi <= 4.0f) {
    const ff t = ff_add_f(ff_scale2(ff_sqr(x), 0.125f), -1.0f);
    const ff a0 = hkff_4_0(t), a1 = hkff_4_1(t), b0 = hkff_4_2(t), b1 = hkff_4_3(t);
    const ff two_pi = ff_make(0.6366197466850281f, 2.5682552973194106e-08f);  // 2/pi
    const ff lx = ff_mul(two_pi, ff_log(x));
    r.j0 = a0;
    r.j1 = ff_mul(x, a1);
    r.y0 = ff_add_fast(ff_mul(lx, a0), b0);
    r.y1 = ff_add_fast(ff_add_fast(ff_mul(lx, r.j1), ff_mul(x, b1)), ff_neg(ff_mul(two_pi, ix)));
  } else {
    ff p0, q0, p1, q1;
    pq_ff(x.hi, ix, &p0, &q0, &p1, &q1);
    // sqrt(2/pi) / sqrt(x)
    const ff amp = ff_mul(ff_make(0.7978845834732056f, -2.2670340271702116e-08f), ff_rsqrt(x));
    const ffc e = expi_ff(x, tab);  // c + i s = e^{i(x - pi/4)}
    // J0 + i Y0 = amp (P0 + i Q0)(c + i s);  J1 + i Y1 = amp (P1 + i Q1)(s - i c)
    r.j0 = ff_mul(amp, ff_add_fast(ff_mul(p0, e.re), ff_neg(ff_mul(q0, e.im))));
    r.y0 = ff_mul(amp, ff_add_fast(ff_mul(p0, e.im), ff_mul(q0, e.re)));
    r.j1 = ff_mul(amp, ff_add_fast(ff_mul(p1, e.im), ff_mul(q1, e.re)));
    r.y1 = ff_mul(amp, ff_add_fast(ff_mul(q1, e.im), ff_neg(ff_mul(p1, e.re))));
  }
  return r;
}

// Host-side table of e^{i(2 pi j/64 - pi/4)} as ff pairs (4 floats per j).
inline void expi_table(float* tab) {
  for (int j = 0; j < 64; ++j) {
    const long double a = 2.0L * 3.14159265358979323846264338327950288L * j / 64.0L -
                          3.14159265358979323846264338327950288L / 4.0L;
    const long double c = cosl(a), s = sinl(a);
    const float ch = (float)c, sh = (float)s;
    tab[4 * j] = ch;
    tab[4 * j + 1] = (float)(c - (long double)ch);
    tab[4 * j + 2] = sh;
    tab[4 * j + 3] = (float)(s - (long double)sh);
  }
}

}  // namespace bem2d_gpu
