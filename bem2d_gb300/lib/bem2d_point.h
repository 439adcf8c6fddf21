// bem2d C++ API (GB300 build): points in the plane.
#ifndef BEM2D_POINT_H
#define BEM2D_POINT_H

#include <iostream>

#include "bem2d_defs.h"

namespace bem2d {

struct Point {
  double x;
  double y;
  Point(double xx, double yy) : x(xx), y(yy) {}
  Point() : x(0), y(0) {}
  Point(const Point& p) = default;
  Point& operator=(const Point& p) = default;
};

std::ostream& operator<<(std::ostream& s, const Point& z);
Point operator+(const Point& p1, const Point& p2);
Point operator-(const Point& p1, const Point& p2);
Point operator*(const Point& p, double t);
Point operator*(double t, const Point& p);
double length(const Point& p);     // Euclidean norm
Point normalize(const Point& p);   // p / length(p)

typedef std::vector<Point> PointVector;
typedef std::shared_ptr<PointVector> pPointVector;

}  // namespace bem2d

#endif
