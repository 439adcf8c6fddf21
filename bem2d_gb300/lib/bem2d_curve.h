// bem2d C++ API (GB300 build): parametrised curves t in [0,1] -> R^2.
#ifndef BEM2D_CURVE_H
#define BEM2D_CURVE_H

#include <cmath>

#include "bem2d_defs.h"
#include "bem2d_point.h"

namespace bem2d {

class Curve {
 public:
  virtual Point Map(double t) const = 0;
  virtual Point Deriv(double t) const = 0;
  // Arc length over [0,1] / [t1,t2] (composite 20-point Gauss-Legendre on
  // 64 panels; the reference uses GSL's adaptive QAG).
  double Length();
  double Length(double t1, double t2);
  virtual ~Curve() {}
};

typedef std::shared_ptr<Curve> pCurve;

double AbsDerivative(double t, void* c);

}  // namespace bem2d

#endif
