/*
 * H0^(1)(z), H1^(1)(z) of a complex argument in 113-bit binary128 arithmetic
 * (TEST INFRASTRUCTURE ONLY): the reference for complex wavenumbers.  Used by
 * the zbesh stand-in of the reference build (shim/shim_support.c) and by the
 * oracle's complex-k kernels (bem2d_oracle.c).
 *
 * Ascending series of J and Y where |z| + max(Im z, 0) <= 40 (the series
 * loses about e^{|z| + Im z} of the 1e-34 unit roundoff to cancellation),
 * Hankel's asymptotic expansion elsewhere (|z| > 20: its smallest term,
 * about e^{-2|z|}, is below 1e-17).  Results agree with mpmath to double
 * rounding and with scipy.special.hankel1 (AMOS) to its own accuracy.
 */
#ifndef ORC_HANKEL_Q_H
#define ORC_HANKEL_Q_H

#include <math.h>

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 qreal;
#define Q_LOG logq
#define Q_ATAN2 atan2q
#define Q_SQRT sqrtq
#define Q_EXP expq
#define Q_SIN sinq
#define Q_COS cosq
#define Q_C(x) x##Q
#else /* aarch64: long double is IEEE binary128 */
typedef long double qreal;
#define Q_LOG logl
#define Q_ATAN2 atan2l
#define Q_SQRT sqrtl
#define Q_EXP expl
#define Q_SIN sinl
#define Q_COS cosl
#define Q_C(x) x##L
#endif

typedef struct {
  qreal re, im;
} qcplx;

static qcplx qmul(qcplx a, qcplx b) {
  qcplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}

/* H_nu^(1)(z), nu = 0 or 1, z = zr + i zi with zr > 0 or zi != 0. */
static qcplx hankel1_q(int nu, qreal zr, qreal zi) {
  const qreal pi = Q_C(3.14159265358979323846264338327950288);
  const qreal gam = Q_C(0.57721566490153286060651209008240243);
  const qreal r = Q_SQRT(zr * zr + zi * zi);
  qcplx h;
  if (r + (zi > 0 ? zi : 0) <= 40) {
    /* q = z^2/4, t_m = (-q)^m/(m!)^2; J0 = sum t_m, J1 = (z/2) sum t_m/(m+1),
       Y0 = (2/pi)[(ln(z/2)+gamma) J0 - sum H_m t_m],
       Y1 = -2/(pi z) + (2/pi) ln(z/2) J1 - (1/pi)(z/2) sum (2H_m + 1/(m+1) - 2gamma) t_m/(m+1) */
    qcplx q = {(zr * zr - zi * zi) / 4, zr * zi / 2};
    qcplx t = {1, 0}, j0 = {0, 0}, j1 = {0, 0}, s0 = {0, 0}, s1 = {0, 0};
    qreal hm = 0;
    for (int m = 0; m < 400; ++m) {
      if (m > 0) hm += Q_C(1.0) / m;
      const qreal inv = Q_C(1.0) / (m + 1);
      j0.re += t.re; j0.im += t.im;
      j1.re += t.re * inv; j1.im += t.im * inv;
      s0.re -= hm * t.re; s0.im -= hm * t.im;
      const qreal c = (2 * hm + inv - 2 * gam) * inv;
      s1.re += c * t.re; s1.im += c * t.im;
      qcplx nt = qmul(t, q);
      t.re = -nt.re * inv * inv;
      t.im = -nt.im * inv * inv;
      if (m > r && Q_SQRT(t.re * t.re + t.im * t.im) < Q_C(1e-40)) break;
    }
    const qcplx zh = {zr / 2, zi / 2};
    const qcplx lz = {Q_LOG(r / 2), Q_ATAN2(zi, zr)};
    if (nu == 0) {
      const qcplx lg = {lz.re + gam, lz.im};
      const qcplx a = qmul(lg, j0);
      const qcplx y = {2 / pi * (a.re + s0.re), 2 / pi * (a.im + s0.im)};
      h.re = j0.re - y.im;
      h.im = j0.im + y.re;
    } else {
      j1 = qmul(j1, zh);
      const qreal iz2 = 1 / (zr * zr + zi * zi);
      const qcplx a = qmul(lz, j1), b = qmul(zh, s1);
      const qcplx y = {-2 / pi * zr * iz2 + 2 / pi * a.re - b.re / pi,
                       2 / pi * zi * iz2 + 2 / pi * a.im - b.im / pi};
      h.re = j1.re - y.im;
      h.im = j1.im + y.re;
    }
    return h;
  }
  /* Hankel's expansion: H = sqrt(2/(pi z)) e^{i(z - nu pi/2 - pi/4)}
     sum_m i^m a_m(nu) / z^m, a_m = prod_{j=1..m} (4nu^2 - (2j-1)^2) / (8^m m!),
     summed while the terms decrease. */
  qcplx iz = {zr / (r * r), -zi / (r * r)}; /* 1/z */
  qcplx term = {1, 0}, sum = {1, 0};
  qreal prev = 1;
  for (int m = 1; m < 200; ++m) {
    const qreal f = (4 * nu * nu - (qreal)(2 * m - 1) * (2 * m - 1)) / (8 * (qreal)m);
    qcplx tt = qmul(term, iz);
    /* times i * f */
    term.re = -tt.im * f;
    term.im = tt.re * f;
    const qreal mag = Q_SQRT(term.re * term.re + term.im * term.im);
    if (mag > prev) break;
    sum.re += term.re;
    sum.im += term.im;
    prev = mag;
    if (mag < Q_C(1e-40)) break;
  }
  /* sqrt(2/(pi z)) = sqrt(2/pi) / sqrt(z) */
  const qreal sr = Q_SQRT((r + zr) / 2), si = (zi >= 0 ? 1 : -1) * Q_SQRT((r - zr) / 2);
  const qreal sn = sr * sr + si * si;
  const qcplx isz = {sr / sn, -si / sn};
  const qreal ph = zr - nu * pi / 2 - pi / 4;
  const qreal ez = Q_EXP(-zi);
  const qcplx e = {ez * Q_COS(ph), ez * Q_SIN(ph)};
  qcplx p = qmul(qmul(e, isz), sum);
  const qreal a = Q_SQRT(2 / pi);
  h.re = a * p.re;
  h.im = a * p.im;
  return h;
}

/* H0, H1 at z = zr + i zi, rounded to double. */
static void orc_hankel01_q(double zr, double zi, double* h0r, double* h0i, double* h1r,
                           double* h1i) {
  const qcplx a = hankel1_q(0, (qreal)zr, (qreal)zi);
  const qcplx b = hankel1_q(1, (qreal)zr, (qreal)zi);
  *h0r = (double)a.re;
  *h0i = (double)a.im;
  *h1r = (double)b.re;
  *h1i = (double)b.im;
}

#endif
