// bem2d C++ API (GB300 build): quadrature rules on [0,1] and [0,1]^2 (host
// objects; the GPU builds the same rules itself).
#ifndef BEM2D_QUADPOINTS_H
#define BEM2D_QUADPOINTS_H

#include "bem2d_defs.h"
#include "bem2d_exceptions.h"

namespace bem2d {

struct QuadPoints1D {
  dvector x, w;
  double a, b;
};

struct QuadPoints2D {
  dvector x, y, w;
  double a, b, c, d;
};

// N-point Gauss-Legendre rule on [0,1]
class Gauss1D {
 public:
  explicit Gauss1D(int N);
  QuadPoints1D Rescale(double a, double b) const;
  const dvector& x() const { return x_; }
  const dvector& w() const { return w_; }
  int Size() const { return N_; }

 private:
  dvector x_, w_;
  int N_;
};

// N x N tensor rule on [0,1]^2, point i*N+j = (x_i, x_j)
class Gauss2D {
 public:
  explicit Gauss2D(int N);
  QuadPoints2D Rescale(double a, double b, double c, double d) const;
  const dvector& x() const { return x_; }
  const dvector& y() const { return y_; }
  const dvector& w() const { return w_; }
  int Size() const { return N_; }

 private:
  dvector x_, y_, w_;
  int N_;
};

// graded rule toward the corner (0,0): L x L geometric boxes
class AdaptedGauss1 {
 public:
  AdaptedGauss1(int N, int L, double sigma);
  const dvector& x() const { return x_; }
  const dvector& y() const { return y_; }
  const dvector& w() const { return w_; }
  int Size() const { return N_; }

 private:
  dvector x_, y_, w_;
  int N_, L_;
  double sigma_;
};

// graded rule toward the corner (0,1): three boxes per level
class AdaptedGauss2 {
 public:
  AdaptedGauss2(int N, int L, double sigma);
  const dvector& x() const { return x_; }
  const dvector& y() const { return y_; }
  const dvector& w() const { return w_; }
  int Size() const { return N_; }

 private:
  dvector x_, y_, w_;
  int N_, L_;
  double sigma_;
};

// graded rule toward the corner (1,0): three boxes per level
class AdaptedGauss3 {
 public:
  AdaptedGauss3(int N, int L, double sigma);
  const dvector& x() const { return x_; }
  const dvector& y() const { return y_; }
  const dvector& w() const { return w_; }
  int Size() const { return N_; }

 private:
  dvector x_, y_, w_;
  int N_, L_;
  double sigma_;
};

}  // namespace bem2d

#endif
