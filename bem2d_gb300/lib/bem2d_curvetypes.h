// bem2d C++ API (GB300 build): the library's curves.  The GPU evaluates these
// six shapes itself (same formulas); other Curve subclasses cannot be
// assembled on the GPU and raise UnsupportedError.
#ifndef BEM2D_CURVETYPES_H
#define BEM2D_CURVETYPES_H

#include <cmath>

#include "bem2d_curve.h"

namespace bem2d {

// unit circle
class Circle : public Curve {
 public:
  Point Map(double t) const { return Point(std::cos(2 * PI * t), std::sin(2 * PI * t)); }
  Point Deriv(double t) const {
    return 2 * PI * Point(-1.0 * std::sin(2 * PI * t), std::cos(2 * PI * t));
  }
};

// r(t) = 1 + 0.3 cos(6 pi t)
class Trefoil : public Curve {
 public:
  Point Map(double t) const;
  Point Deriv(double t) const;
};

// (cos 2 pi t + 0.65 cos 4 pi t - 0.65, 1.5 sin 2 pi t)
class Kite : public Curve {
 public:
  Point Map(double t) const;
  Point Deriv(double t) const;
};

// semi-axes rho and 1/rho
class Ellipse : public Curve {
 public:
  explicit Ellipse(double rho) : rho_(rho) {}
  Point Map(double t) const;
  Point Deriv(double t) const;
  double rho() const { return rho_; }

 private:
  double rho_;
};

// (a cos th, b sin th), th = theta1 + t (theta2 - theta1)
class EllipseArc : public Curve {
 public:
  EllipseArc(double a, double b, double theta1, double theta2)
      : theta1_(theta1), theta2_(theta2), a_(a), b_(b) {}
  Point Map(double t) const;
  Point Deriv(double t) const;
  double a() const { return a_; }
  double b() const { return b_; }
  double theta1() const { return theta1_; }
  double theta2() const { return theta2_; }

 private:
  double theta1_, theta2_, a_, b_;
};

// z(t) = e^{2 pi i t} / (1 + alpha e^{4 pi i t})
class InvEllipse : public Curve {
 public:
  explicit InvEllipse(double alpha) : alpha_(alpha) {}
  Point Map(double t) const;
  Point Deriv(double t) const;
  double alpha() const { return alpha_; }

 private:
  double alpha_;
};

}  // namespace bem2d

#endif
