// bem2d C++ API (GB300 build): incident fields and right-hand-side functionals.
#ifndef BEM2D_FUN_H
#define BEM2D_FUN_H

#include <cmath>

#include "bem2d_defs.h"
#include "bem2d_kernel.h"
#include "bem2d_point.h"

namespace bem2d {

// exp(i k d.x)
class PlaneWave {
 public:
  PlaneWave() {}
  PlaneWave(Point direction, freqtype k) : direction_(direction), k_(k) {}
  complex operator()(Point p) const {
    return std::exp(complex(k_.re, k_.im) * complex(0, 1) * (direction_.x * p.x + direction_.y * p.y));
  }
  void SetNormal(Point) {}
  freqtype k() const { return k_; }
  Point direction() const { return direction_; }

 private:
  Point direction_;
  freqtype k_{0, 0};
};

// i k (n.d) exp(i k d.x)
class NormalPlaneWave {
 public:
  NormalPlaneWave() {}
  NormalPlaneWave(Point direction, freqtype k) : direction_(direction), k_(k) {}
  complex operator()(Point p) const {
    const complex i(0, 1);
    const complex f = std::exp(complex(k_.re, k_.im) * i * (direction_.x * p.x + direction_.y * p.y));
    return i * complex(k_.re, k_.im) * f * (n_.x * direction_.x + n_.y * direction_.y);
  }
  void SetNormal(Point normal) { n_ = normal; }
  freqtype k() const { return k_; }
  Point direction() const { return direction_; }

 private:
  Point direction_;
  freqtype k_{0, 0};
  Point n_;
};

// i k (n.d) exp(i k d.x) - i eta exp(i k d.x)   (eta defaults to k.re)
class CombinedPlaneWave {
 public:
  CombinedPlaneWave(Point direction, freqtype k, double eta) : direction_(direction), k_(k), eta_(eta) {}
  CombinedPlaneWave(Point direction, freqtype k) : direction_(direction), k_(k), eta_(k.re) {}
  complex operator()(Point p) const {
    const complex i(0, 1);
    const complex f = std::exp(complex(k_.re, k_.im) * i * (direction_.x * p.x + direction_.y * p.y));
    return i * complex(k_.re, k_.im) * f * (n_.x * direction_.x + n_.y * direction_.y) - i * eta_ * f;
  }
  void SetNormal(Point normal) { n_ = normal; }
  freqtype k() const { return k_; }
  Point direction() const { return direction_; }
  double eta() const { return eta_; }

 private:
  Point direction_;
  freqtype k_;
  Point n_;
  double eta_;
};

// outgoing wave i/4 H0(k |x|)
class OutWave {
 public:
  explicit OutWave(freqtype k) : k_(k), s_(k) {}
  complex operator()(Point x) const { return s_(Point(0, 0), x); }
  void SetNormal(Point) {}
  freqtype k() const { return k_; }

 private:
  freqtype k_;
  SingleLayer s_;
};

class IdFun {
 public:
  complex operator()(Point) const { return 1.0; }
  void SetNormal(Point) {}
};

}  // namespace bem2d

#endif
