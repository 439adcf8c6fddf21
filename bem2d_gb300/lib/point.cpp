// bem2d C++ API (GB300 build): Point arithmetic.
#include <cmath>

#include "bem2d_point.h"

namespace bem2d {

std::ostream& operator<<(std::ostream& s, const Point& z) { return s << "(" << z.x << "," << z.y << ")"; }
Point operator+(const Point& a, const Point& b) { return Point(a.x + b.x, a.y + b.y); }
Point operator-(const Point& a, const Point& b) { return Point(a.x - b.x, a.y - b.y); }
Point operator*(const Point& p, double t) { return Point(t * p.x, t * p.y); }
Point operator*(double t, const Point& p) { return Point(t * p.x, t * p.y); }
double length(const Point& p) { return std::sqrt(p.x * p.x + p.y * p.y); }
Point normalize(const Point& p) {
  const double l = length(p);
  return Point(p.x / l, p.y / l);
}

}  // namespace bem2d
