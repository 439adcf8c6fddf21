// bem2d C++ API (GB300 build): boundary builders.  Polygon / Line / Disk
// follow the reference's construction rules point for point (same element
// end points); AnalyticCurve parametrises by arc length with its own method
// (Gauss-Legendre arc length + Newton), not the reference's GSL ODE solver.
#include <algorithm>
#include <cmath>

#include "bem2d_curvetypes.h"
#include "bem2d_shape.h"

namespace bem2d {

static void link_closed(std::vector<pElement>& e) {
  const int n = (int)e.size();
  for (int i = 0; i < n; ++i) {
    e[i]->set_next(i + 1 < n ? i + 1 : 0);
    e[i]->set_prev(i > 0 ? i - 1 : n - 1);
  }
}

DiskShapePiecewiseConst::DiskShapePiecewiseConst(int n, double radius) {
  const double angle = 2 * PI / n;
  std::vector<Point> pts;
  for (int i = 0; i < n; ++i) pts.push_back(Point(radius * std::cos(i * angle), radius * std::sin(i * angle)));
  for (int i = 0; i < n; ++i) elements_.push_back(pElement(new ConstElement(pts[i], pts[(i + 1) % n], i)));
  link_closed(elements_);
}
pGeometry DiskShapePiecewiseConst::GetGeometry() { return pGeometry(new Geometry(elements_)); }

// One side p0 -> p1 with n coarse cells; the first and last cell split into
// 1 + L geometric cells (ratio sigma) when L > 0.
static void graded_side(std::vector<pElement>& out, const Point& p0, const Point& p1, int n, int L,
                        double sigma, int& count) {
  const Point dir = p1 - p0;
  if (L == 0) {
    out.push_back(pElement(new ConstElement(p0, p0 + (1.0 / n) * dir, count++)));
  } else {
    double ts = 1;
    for (int m = 0; m < L; ++m) ts = ts * sigma;
    out.push_back(pElement(new ConstElement(p0, p0 + (ts / n) * dir, count++)));
    for (int j = 0; j < L; ++j) {
      const Point q1 = p0 + ts / n * dir;
      ts = ts / sigma;
      const Point q2 = p0 + ts / n * dir;
      out.push_back(pElement(new ConstElement(q1, q2, count++)));
    }
  }
  for (int j = 1; j < n - 1; ++j) {
    const Point q1 = p0 + (1.0 * j) / n * dir;
    const Point q2 = p0 + (1.0 * (j + 1)) / n * dir;
    out.push_back(pElement(new ConstElement(q1, q2, count++)));
  }
  const Point base = p0 + (1.0 * (n - 1)) / n * dir;
  if (L == 0) {
    out.push_back(pElement(new ConstElement(base, p1, count++)));
  } else {
    double ts = 1;
    for (int j = 0; j < L; ++j) {
      const Point q1 = base + (1 - ts) / n * dir;
      ts *= sigma;
      const Point q2 = base + (1 - ts) / n * dir;
      out.push_back(pElement(new ConstElement(q1, q2, count++)));
    }
    out.push_back(pElement(new ConstElement(base + (1 - ts) / n * dir, p1, count++)));
  }
}

Polygon::Polygon(const std::vector<Point>& points, int ppw, freqtype k, int L, double sigma) {
  std::vector<Point> p(points);
  p.push_back(p[0]);
  int count = 0;
  for (std::size_t i = 0; i < points.size(); ++i) {
    const Point dir = p[i + 1] - p[i];
    int n = (int)std::ceil(ppw * (double)k.re * length(dir) / 2.0 / PI);
    n = std::max(150, n);
    graded_side(elements_, p[i], p[i + 1], n, L, sigma, count);
  }
  link_closed(elements_);
}

Polygon::Polygon(const std::vector<Point>& points, int n) {
  std::vector<Point> p(points);
  p.push_back(p[0]);
  for (std::size_t i = 0; i < points.size(); ++i) {
    const Point dir = p[i + 1] - p[i];
    for (int j = 0; j < n; ++j) {
      const Point q1 = p[i] + (1.0 * j) / n * dir;
      const Point q2 = p[i] + (1.0 * (j + 1)) / n * dir;
      elements_.push_back(pElement(new ConstElement(q1, q2, n * i + j)));
    }
  }
  link_closed(elements_);
}
pGeometry Polygon::GetGeometry() { return pGeometry(new Geometry(elements_)); }

Line::Line(Point p0, Point p1, int ppw, freqtype k, int L, double sigma) {
  int n = (int)std::ceil(ppw * (double)k.re * length(p1 - p0) / 2.0 / PI);
  n = std::max(10, n);
  int count = 0;
  graded_side(elements_, p0, p1, n, L, sigma, count);
  // linked as a closed chain, as the reference's graded Line is
  link_closed(elements_);
}

Line::Line(Point p0, Point p1, int n) {
  const Point dir = p1 - p0;
  for (int j = 0; j < n; ++j)
    elements_.push_back(pElement(new ConstElement(p0 + (1.0 * j) / n * dir, p0 + (1.0 * (j + 1)) / n * dir, j)));
  for (int i = 0; i < n; ++i) {
    if (i + 1 < n) elements_[i]->set_next(i + 1);
    if (i > 0) elements_[i]->set_prev(i - 1);
  }
}
pGeometry Line::GetGeometry() { return pGeometry(new Geometry(elements_)); }

// ---- arc length -------------------------------------------------------------
static double arc(const Curve& c, double a, double b) {
  // 20-point Gauss-Legendre on [a,b] (intervals are short here)
  static double x[20], w[20];
  static bool init = false;
  if (!init) {
    const int n = 20;
    for (int i = 0; i < n; ++i) {
      double z = std::cos(PI * (i + 0.75) / (n + 0.5)), dp = 0;
      for (int it = 0; it < 100; ++it) {
        double q0 = 1, q1 = z;
        for (int k = 2; k <= n; ++k) {
          const double q2 = ((2.0 * k - 1) * z * q1 - (k - 1.0) * q0) / k;
          q0 = q1;
          q1 = q2;
        }
        dp = n * (z * q1 - q0) / (z * z - 1);
        const double dz = q1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) break;
      }
      x[i] = z;
      w[i] = 2.0 / ((1 - z * z) * dp * dp);
    }
    init = true;
  }
  double s = 0;
  for (int i = 0; i < 20; ++i) s += w[i] * length(c.Deriv(0.5 * (a + b) + 0.5 * (b - a) * x[i]));
  return 0.5 * (b - a) * s;
}

void AnalyticCurve::ParameterizeArc(dvector& partition) {
  const int n = (int)partition.size() - 1;
  arclengthparam.assign(n + 1, 0.0);
  // tabulate s(t) on a fine grid, then Newton from the bracketing node
  const int M = 4096;
  dvector s(M + 1, 0.0);
  for (int i = 0; i < M; ++i) s[i + 1] = s[i] + arc(*curve_, (double)i / M, (double)(i + 1) / M);
  int j = 0;
  for (int i = 1; i < n; ++i) {
    const double target = partition[i];
    while (j < M - 1 && s[j + 1] < target) ++j;
    double t = (double)j / M;
    double st = s[j];
    for (int it = 0; it < 50; ++it) {
      const double f = st - target;
      const double dt = -f / length(curve_->Deriv(t));
      const double tn = t + dt;
      st += arc(*curve_, t, tn);
      t = tn;
      if (std::fabs(dt) < 1e-16) break;
    }
    arclengthparam[i] = t;
  }
  arclengthparam[n] = 1;
}

void AnalyticCurve::Build(int closed) {
  const int n = (int)arclengthparam.size() - 1;
  for (int i = 0; i < n; ++i)
    elements_.push_back(pElement(new AnalyticCurveElement(arclengthparam[i], i == n - 1 ? 1.0 : arclengthparam[i + 1], curve_, i)));
  for (int i = 0; i < n; ++i) {
    if (i + 1 < n) elements_[i]->set_next(i + 1);
    if (i > 0) elements_[i]->set_prev(i - 1);
  }
  if (closed) {
    elements_[0]->set_prev(n - 1);
    elements_[n - 1]->set_next(0);
  }
}

AnalyticCurve::AnalyticCurve(int n, pCurve curve, int closed) : curve_(curve) {
  const double len = curve_->Length();
  dvector partition(n + 1);
  for (int i = 0; i <= n; ++i) partition[i] = i * len / n;
  ParameterizeArc(partition);
  Build(closed);
}

AnalyticCurve::AnalyticCurve(int ppw, freqtype k, pCurve curve, int closed, int L, double sigma)
    : curve_(curve) {
  const double len = curve_->Length();
  dvector partition;
  partition.push_back(0);
  int c = (int)std::ceil(ppw * (double)k.re * len / 2.0 / PI);
  c = std::max(c, 10);
  if (L == 0) {
    partition.push_back(len / c);
  } else {
    double ts = 1;
    for (int m = 0; m < L; ++m) ts = ts * sigma;
    partition.push_back(ts * len / c);
    for (int m = 0; m < L; ++m) {
      ts = ts / sigma;
      partition.push_back(ts * len / c);
    }
  }
  for (int j = 2; j < c; ++j) partition.push_back(len / c * j);
  if (L == 0) {
    partition.push_back(len);
  } else {
    const double td = len / c * (c - 1);
    double ts = 1;
    for (int m = 0; m < L; ++m) {
      ts = ts * sigma;
      partition.push_back(td + len / c * (1 - ts));
    }
    partition.push_back(len);
  }
  ParameterizeArc(partition);
  Build(closed);
}

pGeometry AnalyticCurve::GetGeometry() { return pGeometry(new Geometry(elements_)); }

}  // namespace bem2d
