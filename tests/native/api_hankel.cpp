// Host-side Hankel functions of the bem2d C++ API with a complex argument
// (BesselH0 / BesselH1(complex), the reference's AMOS branch) and the
// SingleLayer functor at a complex wavenumber.  Reads "zr zi" lines and
// prints "H0 H1 S" per line (re im pairs), where S = SingleLayer(z)(x, y)
// for |x - y| = 1, i.e. i/4 H0(z).  No GPU is used.
#include <cstdio>

#include "bem2d.h"

int main() {
  double zr, zi;
  while (std::scanf("%lf %lf", &zr, &zi) == 2) {
    const bem2d::complex z(zr, zi);
    const bem2d::complex h0 = bem2d::BesselH0(z), h1 = bem2d::BesselH1(z);
    bem2d::freqtype k = {zr, zi};
    bem2d::SingleLayer sl(k);
    const bem2d::complex s = sl(bem2d::Point(0.25, -0.5), bem2d::Point(1.25, -0.5));
    std::printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", h0.real(), h0.imag(), h1.real(),
                h1.imag(), s.real(), s.imag());
  }
  return 0;
}
