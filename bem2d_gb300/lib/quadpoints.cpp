// bem2d C++ API (GB300 build): quadrature rule objects (host).  Nodes and
// weights from the library's own Gauss-Legendre routine (bem2d_gauss).
#include <cmath>

#include "../../include/bem2d_gpu.h"
#include "bem2d_quadpoints.h"
#include "bem2d_quadrature.h"

namespace bem2d {

void Gauss(dvector& x, dvector& w, int N) {
  if (N < 1) throw ParameterException();
  x.assign(N, 0.0);
  w.assign(N, 0.0);
  if (bem2d_gauss(N, &x[0], &w[0]) != BEM2D_OK) throw LapackError();
}

void MapPoints(dvector& x, dvector& w, double a, double b) {
  for (std::size_t i = 0; i < x.size(); ++i) {
    x[i] = a + (b - a) * x[i];
    w[i] = (b - a) * w[i];
  }
}

void MapPoints2d(dvector& x, dvector& y, dvector& w, double a, double b, double c, double d) {
  for (std::size_t i = 0; i < x.size(); ++i) {
    x[i] = a + (b - a) * x[i];
    y[i] = c + (d - c) * y[i];
    w[i] = (b - a) * (d - c) * w[i];
  }
}

Gauss1D::Gauss1D(int N) : N_(N) {
  if (N < 1) throw ParameterException();
  Gauss(x_, w_, N);
}

QuadPoints1D Gauss1D::Rescale(double a, double b) const {
  if (a >= b) throw IntervalException();
  QuadPoints1D p;
  p.a = a;
  p.b = b;
  p.x = x_;
  p.w = w_;
  MapPoints(p.x, p.w, a, b);
  return p;
}

Gauss2D::Gauss2D(int N) : N_(N * N) {
  if (N < 1) throw ParameterException();
  dvector xt, wt;
  Gauss(xt, wt, N);
  x_.resize(N_);
  y_.resize(N_);
  w_.resize(N_);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      x_[i * N + j] = xt[i];
      y_[i * N + j] = xt[j];
      w_[i * N + j] = wt[i] * wt[j];
    }
}

QuadPoints2D Gauss2D::Rescale(double a, double b, double c, double d) const {
  if (a >= b || c >= d) throw IntervalException();
  QuadPoints2D p;
  p.a = a;
  p.b = b;
  p.c = c;
  p.d = d;
  p.x = x_;
  p.y = y_;
  p.w = w_;
  MapPoints2d(p.x, p.y, p.w, a, b, c, d);
  return p;
}

static void append(dvector& x, dvector& y, dvector& w, const QuadPoints2D& q) {
  x.insert(x.end(), q.x.begin(), q.x.end());
  y.insert(y.end(), q.y.begin(), q.y.end());
  w.insert(w.end(), q.w.begin(), q.w.end());
}

AdaptedGauss1::AdaptedGauss1(int N, int L, double sigma) : N_(N * N * L * L), L_(L), sigma_(sigma) {
  dvector xl;
  for (int i = 0; i < L; ++i) xl.push_back(std::pow(sigma, L - i));
  xl.push_back(1.0);
  Gauss2D g(N);
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) append(x_, y_, w_, g.Rescale(xl[i], xl[i + 1], xl[j], xl[j + 1]));
}

AdaptedGauss2::AdaptedGauss2(int N, int L, double sigma) : N_(3 * N * N * L), L_(L), sigma_(sigma) {
  Gauss2D g(N);
  double a = sigma, b = 1;
  for (int l = L; l > 0; --l) {
    append(x_, y_, w_, g.Rescale(0, a, 1 - b, 1 - a));
    append(x_, y_, w_, g.Rescale(a, b, 1 - b, 1 - a));
    append(x_, y_, w_, g.Rescale(a, b, 1 - a, 1));
    a *= sigma;
    b *= sigma;
  }
}

AdaptedGauss3::AdaptedGauss3(int N, int L, double sigma) : N_(3 * N * N * L), L_(L), sigma_(sigma) {
  Gauss2D g(N);
  double a = 1, b = sigma;
  for (int l = L; l > 0; --l) {
    append(x_, y_, w_, g.Rescale(1 - a, 1 - b, 0, b));
    append(x_, y_, w_, g.Rescale(1 - a, 1 - b, b, a));
    append(x_, y_, w_, g.Rescale(1 - b, 1, b, a));
    a *= sigma;
    b *= sigma;
  }
}

}  // namespace bem2d
