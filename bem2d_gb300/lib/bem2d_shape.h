// bem2d C++ API (GB300 build): boundary builders.
#ifndef BEM2D_SHAPE_H
#define BEM2D_SHAPE_H

#include <vector>

#include "bem2d_defs.h"
#include "bem2d_element.h"
#include "bem2d_exceptions.h"
#include "bem2d_geometry.h"
#include "bem2d_point.h"

namespace bem2d {

// n chords of the circle of the given radius
class DiskShapePiecewiseConst {
 public:
  DiskShapePiecewiseConst(int n, double radius);
  pGeometry GetGeometry();

 private:
  std::vector<pElement> elements_;
};

// closed polygon; ppw/k version: n = max(150, ceil(ppw k |side| / 2 pi))
// cells per side, the end cells split geometrically (L levels, ratio sigma)
class Polygon {
 public:
  Polygon(const std::vector<Point>& points, int ppw, freqtype k, int L = 0, double sigma = 0.15);
  Polygon(const std::vector<Point>& points, int n);
  pGeometry GetGeometry();

 private:
  std::vector<pElement> elements_;
};

// open segment p0 -> p1 (same grading rule, at least 10 cells)
class Line {
 public:
  Line(Point p0, Point p1, int ppw, freqtype k, int L = 0, double sigma = 0.15);
  Line(Point p0, Point p1, int n);
  pGeometry GetGeometry();

 private:
  std::vector<pElement> elements_;
};

// elements of equal arc length on a curve (arc length by composite
// Gauss-Legendre quadrature, inverted by Newton's method)
class AnalyticCurve {
 public:
  AnalyticCurve(int n, pCurve curve, int closed = 1);
  AnalyticCurve(int ppw, freqtype k, pCurve curve, int closed = 1, int L = 0,
                double sigma = 0.15);
  pGeometry GetGeometry();
  void ParameterizeArc(dvector& partition);

 private:
  void Build(int closed);
  std::vector<pElement> elements_;
  pCurve curve_;
  dvector arclengthparam;
};

}  // namespace bem2d

#endif
