// bem2d C++ API (GB300 build): single kernel values on the host, with the
// same Hankel evaluators as the GPU (bem2d_gb300/csrc/hankel.cuh, real
// argument; hankel_c.cuh, complex argument).
#include <cmath>

#include "../csrc/hankel_c.cuh"
#include "bem2d_exceptions.h"
#include "bem2d_kernel.h"
#include "bem2d_mathroutines.h"

namespace bem2d {

complex BesselH0(double x) {
  double j0, y0, j1, y1;
  bem2d_gpu::hankel01_d(x, &j0, &y0, &j1, &y1);
  return complex(j0, y0);
}
complex BesselH1(double x) {
  double j0, y0, j1, y1;
  bem2d_gpu::hankel01_d(x, &j0, &y0, &j1, &y1);
  return complex(j1, y1);
}
// Complex argument (the reference's AMOS zbesh branch): the GPU's
// complex-argument evaluator, domain Re z > 0, arg z >= -pi/3.
static void check_complex_arg(complex x) {
  if (!(x.real() > 0.0 && x.imag() >= -std::sqrt(3.0) * x.real()))
    throw UnsupportedError("Hankel functions of complex argument: Re z > 0, arg z >= -pi/3");
}
complex BesselH0(complex x) {
  check_complex_arg(x);
  bem2d_gpu::cd h0, h1;
  bem2d_gpu::hankel01_c(bem2d_gpu::cd{x.real(), x.imag()}, &h0, &h1);
  return complex(h0.re, h0.im);
}
complex BesselH1(complex x) {
  check_complex_arg(x);
  bem2d_gpu::cd h0, h1;
  bem2d_gpu::hankel01_c(bem2d_gpu::cd{x.real(), x.imag()}, &h0, &h1);
  return complex(h1.re, h1.im);
}

// H0(k d), H1(k d) for a real or complex wavenumber (lib/bem2d_kernel.cpp:15-112)
static void hankel_kd(const freqtype& k, double d, complex* h0, complex* h1) {
  if (k.im == 0) {
    *h0 = BesselH0(k.re * d);
    *h1 = BesselH1(k.re * d);
  } else {
    const complex z = complex(k.re, k.im) * d;
    *h0 = BesselH0(z);
    *h1 = BesselH1(z);
  }
}

complex SingleLayer::operator()(Point x, Point y) const {
  complex h0, h1;
  hankel_kd(k_, length(x - y), &h0, &h1);
  return complex(0, 1) / 4.0 * h0;
}

complex DoubleLayer::operator()(Point x, Point y) const {
  const Point w = y - x;
  const double d = length(w);
  complex h0, h1;
  hankel_kd(k_, d, &h0, &h1);
  return -complex(0, 1) * complex(k_.re, k_.im) / 4.0 * (h1 / d * (n2_.x * w.x + n2_.y * w.y));
}

complex ConjDoubleLayer::operator()(Point x, Point y) const {
  const Point w = x - y;
  const double d = length(w);
  complex h0, h1;
  hankel_kd(k_, d, &h0, &h1);
  return -complex(0, 1) * complex(k_.re, k_.im) / 4.0 * (h1 / d * (n1_.x * w.x + n1_.y * w.y));
}

complex CombinedSingleConjDouble::operator()(Point x, Point y) const {
  const Point w = x - y;
  const double d = length(w);
  const complex i(0, 1);
  complex h0, h1;
  hankel_kd(k_, d, &h0, &h1);
  const complex s = i / 4.0 * h0;
  const complex cd = -i * complex(k_.re, k_.im) / 4.0 * (h1 / d * (n1_.x * w.x + n1_.y * w.y));
  return cd - i * eta_ * s;
}

}  // namespace bem2d
