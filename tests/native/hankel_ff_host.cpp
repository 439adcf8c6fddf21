// Host build of the float-float far-field Hankel pieces
// (bem2d_gb300/csrc/hankel_ff.cuh), exported for accuracy tests.
#include <cmath>

#include "hankel_ff.cuh"

using namespace bem2d_gpu;

static ffc cmul_ff(ffc a, ffc b) {
  ffc r;
  r.re = ff_add_fast(ff_mul(a.re, b.re), ff_neg(ff_mul(a.im, b.im)));
  r.im = ff_add_fast(ff_mul(a.re, b.im), ff_mul(a.im, b.re));
  return r;
}

// out[4i..4i+3] = J0, Y0, J1, Y1 at x[i] > 8 (x given as a double, rounded
// to float-float first)
extern "C" void hankel01_ff_host(int n, const double* x, double* out) {
  float tab[256];
  expi_table(tab);
  for (int i = 0; i < n; ++i) {
    const ff xf = ff_from_double(x[i]);
    const ff ix = ff_rcp(xf);
    ff p0, q0, p1, q1;
    pq_ff(xf.hi, ix, &p0, &q0, &p1, &q1);
    const ff amp = ff_mul(ff_make(0.7978845834732056f, -2.2670340271702116e-08f), ff_rsqrt(xf));
    const ffc e = expi_ff(xf, tab);
    ffc h0 = cmul_ff(ffc{p0, q0}, e);
    ffc h1 = cmul_ff(ffc{p1, q1}, e);  // times -i below
    out[4 * i] = ff_to_double(ff_mul(amp, h0.re));
    out[4 * i + 1] = ff_to_double(ff_mul(amp, h0.im));
    out[4 * i + 2] = ff_to_double(ff_mul(amp, h1.im));
    out[4 * i + 3] = -ff_to_double(ff_mul(amp, h1.re));
  }
}

// out[4i..4i+3] = J0, Y0, J1, Y1 at x[i] > 0 through bessel01_ff (both the
// small-argument and the modulus-phase branch)
extern "C" void bessel01_ff_host(int n, const double* x, double* out) {
  float tab[256];
  expi_table(tab);
  for (int i = 0; i < n; ++i) {
    const ff xf = ff_from_double(x[i]);
    const BesselFF b = bessel01_ff(xf, ff_rcp(xf), tab);
    out[4 * i] = ff_to_double(b.j0);
    out[4 * i + 1] = ff_to_double(b.y0);
    out[4 * i + 2] = ff_to_double(b.j1);
    out[4 * i + 3] = ff_to_double(b.y1);
  }
}

// out[i] = log(x[i]) through ff_log
extern "C" void log_ff_host(int n, const double* x, double* out) {
  for (int i = 0; i < n; ++i) out[i] = ff_to_double(ff_log(ff_from_double(x[i])));
}

// out[2i], out[2i+1] = ff_dot2(a, b, c, d) for in[8i..8i+7] = a.hi, a.lo,
// b.hi, b.lo, c.hi, c.lo, d.hi, d.lo
extern "C" void dot2_ff_host(int n, const float* in, float* out) {
  for (int i = 0; i < n; ++i) {
    const float* v = in + 8 * i;
    const ff r = ff_dot2(ff_make(v[0], v[1]), ff_make(v[2], v[3]), ff_make(v[4], v[5]),
                         ff_make(v[6], v[7]));
    out[2 * i] = r.hi;
    out[2 * i + 1] = r.lo;
  }
}
