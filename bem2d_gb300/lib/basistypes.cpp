// bem2d C++ API (GB300 build): basis families.
#include <cmath>

#include "bem2d_basistypes.h"

namespace bem2d {

ConstBasis::ConstBasis() {}

PolBasis::PolBasis(int degree) : degree_(degree) {}
void PolBasis::AddBasis(int degree, pGeometry pgeom) {
  for (int i = 0; i <= degree; ++i) pgeom->AddBasis(pBasis(new PolBasis(i)));
}

LinBasis::LinBasis(int sign) : sign_(sign) {}
void LinBasis::AddBasis(pGeometry pgeom) {
  pgeom->AddBasis(pBasis(new LinBasis(1)));
  pgeom->AddBasis(pBasis(new LinBasis(-1)));
}

WaveBasis::WaveBasis(double direction, freqtype k) : direction_(direction), k_(k) {}
complex WaveBasis::operator()(double t) const {
  return std::exp(complex(0, 1) * complex(k_.re, k_.im) * direction_ * t);
}
void WaveBasis::AddBasis(freqtype k, pGeometry pgeom) {
  pgeom->AddBasis(pBasis(new WaveBasis(1.0, k)));
  pgeom->AddBasis(pBasis(new WaveBasis(-1.0, k)));
}

WavePolBasis::WavePolBasis(int degree, double direction, freqtype k)
    : direction_(direction), k_(k), degree_(degree) {}
complex WavePolBasis::operator()(double t) const {
  double r = 1;
  for (int i = 0; i < degree_; ++i) r *= t;
  return std::exp(complex(0, 1) * complex(k_.re, k_.im) * direction_ * t) * r;
}
void WavePolBasis::AddBasis(int degree, freqtype k, pGeometry pgeom) {
  for (int i = 0; i <= degree; ++i) {
    pgeom->AddBasis(pBasis(new WavePolBasis(i, 1.0, k)));
    pgeom->AddBasis(pBasis(new WavePolBasis(i, -1.0, k)));
  }
}

}  // namespace bem2d
