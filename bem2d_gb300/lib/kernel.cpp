// bem2d C++ API (GB300 build): single kernel values on the host, with the
// same Hankel evaluator as the GPU (bem2d_gb300/csrc/hankel.cuh).
#include <cmath>

#include "../csrc/hankel.cuh"
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
complex BesselH0(complex) {
  throw UnsupportedError("Hankel functions of complex argument are not built (complex wavenumbers)");
}
complex BesselH1(complex) {
  throw UnsupportedError("Hankel functions of complex argument are not built (complex wavenumbers)");
}

static void real_k(const freqtype& k) {
  if (k.im != 0) throw UnsupportedError("complex wavenumbers are not supported in this build");
}

complex SingleLayer::operator()(Point x, Point y) const {
  real_k(k_);
  return complex(0, 1) / 4.0 * BesselH0(k_.re * length(x - y));
}

complex DoubleLayer::operator()(Point x, Point y) const {
  real_k(k_);
  const Point w = y - x;
  const double d = length(w);
  return -complex(0, 1) * k_.re / 4.0 * (BesselH1(k_.re * d) / d * (n2_.x * w.x + n2_.y * w.y));
}

complex ConjDoubleLayer::operator()(Point x, Point y) const {
  real_k(k_);
  const Point w = x - y;
  const double d = length(w);
  return -complex(0, 1) * k_.re / 4.0 * (BesselH1(k_.re * d) / d * (n1_.x * w.x + n1_.y * w.y));
}

complex CombinedSingleConjDouble::operator()(Point x, Point y) const {
  real_k(k_);
  const Point w = x - y;
  const double d = length(w);
  const complex i(0, 1);
  const complex s = i / 4.0 * BesselH0(k_.re * d);
  const complex cd = -i * k_.re / 4.0 * (BesselH1(k_.re * d) / d * (n1_.x * w.x + n1_.y * w.y));
  return cd - i * eta_ * s;
}

}  // namespace bem2d
