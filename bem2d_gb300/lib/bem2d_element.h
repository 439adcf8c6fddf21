// bem2d C++ API (GB300 build): boundary elements.  An element maps t in [0,1]
// onto a piece of the boundary and carries the links (index, next, prev) that
// select the graded quadrature for identical and adjacent pairs.
#ifndef BEM2D_ELEMENT_H
#define BEM2D_ELEMENT_H

#include <cstddef>

#include "bem2d_curve.h"
#include "bem2d_defs.h"
#include "bem2d_point.h"

namespace bem2d {

class Element {
 public:
  Element() = default;
  Element(const Element&) = delete;
  Element& operator=(const Element&) = delete;
  virtual ~Element() {}

  virtual const Point Map(double t) const = 0;
  virtual const Point Deriv(double t) const = 0;
  virtual const double Length() const = 0;

  const Point First() { return Map(0); }
  const Point Last() { return Map(1); }
  // outward normal for counter-clockwise boundaries: (d.y, -d.x) / |d|
  const Point Normal(double t) const {
    const Point p(Deriv(t));
    return normalize(Point(p.y, -p.x));
  }

  void set_index(std::size_t i) { index_ = i; }
  std::size_t index() const { return index_; }
  void set_next(std::size_t i) { next_ = i; }
  std::size_t next() const { return next_; }
  void set_prev(std::size_t i) { prev_ = i; }
  std::size_t prev() const { return prev_; }

 private:
  // unset links compare unequal to every index
  std::size_t index_ = static_cast<std::size_t>(-1);
  std::size_t next_ = static_cast<std::size_t>(-1);
  std::size_t prev_ = static_cast<std::size_t>(-1);
};

typedef std::shared_ptr<Element> pElement;

// straight segment p1 -> p2
class ConstElement : public Element {
 public:
  ConstElement(const Point& p1, const Point& p2, std::size_t index);
  const Point Map(double t) const { return p1_ + d_ * t; }
  const Point Deriv(double) const { return d_; }
  const double Length() const { return length(d_); }
  const Point& p1() const { return p1_; }
  const Point& p2() const { return p2_; }

 private:
  const Point p1_, p2_, d_;
};

// curve(t1 + t (t2 - t1))
class AnalyticCurveElement : public Element {
 public:
  AnalyticCurveElement(double t1, double t2, pCurve curve, std::size_t index);
  const Point Map(double t) const { return curve_->Map(tstart_ + t * (tend_ - tstart_)); }
  const Point Deriv(double t) const {
    return (tend_ - tstart_) * curve_->Deriv(tstart_ + t * (tend_ - tstart_));
  }
  const double Length() const { return curve_->Length(tstart_, tend_); }
  const pCurve& curve() const { return curve_; }
  double tstart() const { return tstart_; }
  double tend() const { return tend_; }

 private:
  pCurve curve_;
  double tstart_, tend_;
};

}  // namespace bem2d

#endif
