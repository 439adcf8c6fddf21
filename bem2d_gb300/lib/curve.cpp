// bem2d C++ API (GB300 build): curve lengths and the library curve types.
#include <cmath>
#include <complex>

#include "bem2d_curve.h"
#include "bem2d_curvetypes.h"

namespace bem2d {

double AbsDerivative(double t, void* c) { return length(static_cast<Curve*>(c)->Deriv(t)); }

// composite 20-point Gauss-Legendre on 64 panels (nodes by Newton on P_20)
static const std::vector<std::pair<double, double> >& gl20() {
  static std::vector<std::pair<double, double> > r;
  if (r.empty()) {
    const int n = 20;
    for (int i = 0; i < n; ++i) {
      double z = std::cos(PI * (i + 0.75) / (n + 0.5)), dp = 0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1, p1 = z;
        for (int k = 2; k <= n; ++k) {
          const double p2 = ((2.0 * k - 1) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1);
        const double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) break;
      }
      r.push_back(std::make_pair(z, 2.0 / ((1 - z * z) * dp * dp)));
    }
  }
  return r;
}

double Curve::Length() { return Length(0, 1); }

double Curve::Length(double t1, double t2) {
  const int panels = 64;
  const double h = (t2 - t1) / panels;
  double s = 0;
  for (int p = 0; p < panels; ++p) {
    const double c = t1 + (p + 0.5) * h;
    for (const auto& q : gl20()) s += q.second * 0.5 * h * length(Deriv(c + 0.5 * h * q.first));
  }
  return s;
}

Point Trefoil::Map(double t) const {
  const double r = 1 + 0.3 * std::cos(3 * 2 * PI * t);
  return Point(r * std::cos(2 * PI * t), r * std::sin(2 * PI * t));
}
Point Trefoil::Deriv(double t) const {
  const double r = 1 + 0.3 * std::cos(3 * 2 * PI * t);
  const double rp = -0.3 * 3 * 2 * PI * std::sin(3 * 2 * PI * t);
  return Point(rp * std::cos(2 * PI * t) - r * 2 * PI * std::sin(2 * PI * t),
               rp * std::sin(2 * PI * t) + r * 2 * PI * std::cos(2 * PI * t));
}

Point Kite::Map(double t) const {
  return Point(std::cos(2 * PI * t) + 0.65 * std::cos(4 * PI * t) - 0.65, 1.5 * std::sin(2 * PI * t));
}
Point Kite::Deriv(double t) const {
  return Point(-2 * PI * std::sin(2 * PI * t) - 0.65 * 4 * PI * std::sin(4 * PI * t),
               1.5 * 2 * PI * std::cos(2 * PI * t));
}

Point Ellipse::Map(double t) const {
  return Point(rho_ * std::cos(2 * PI * t), 1 / rho_ * std::sin(2 * PI * t));
}
Point Ellipse::Deriv(double t) const {
  return Point(-rho_ * 2 * PI * std::sin(2 * PI * t), 2 * PI / rho_ * std::cos(2 * PI * t));
}

Point EllipseArc::Map(double t) const {
  const double th = theta1_ + t * (theta2_ - theta1_);
  return Point(a_ * std::cos(th), b_ * std::sin(th));
}
Point EllipseArc::Deriv(double t) const {
  const double th = theta1_ + t * (theta2_ - theta1_);
  return Point(-a_ * (theta2_ - theta1_) * std::sin(th), b_ * (theta2_ - theta1_) * std::cos(th));
}

Point InvEllipse::Map(double t) const {
  const std::complex<double> e = std::polar(1.0, 2 * PI * t), e2 = std::polar(1.0, 4 * PI * t);
  const std::complex<double> z = e / (1.0 + alpha_ * e2);
  return Point(z.real(), z.imag());
}
Point InvEllipse::Deriv(double t) const {
  const std::complex<double> i(0, 1);
  const std::complex<double> e = std::polar(1.0, 2 * PI * t), e2 = std::polar(1.0, 4 * PI * t);
  const std::complex<double> q = 1.0 + alpha_ * e2;
  const std::complex<double> d = 2.0 * PI * i * e * (1.0 - alpha_ * e2) / (q * q);
  return Point(d.real(), d.imag());
}

}  // namespace bem2d
