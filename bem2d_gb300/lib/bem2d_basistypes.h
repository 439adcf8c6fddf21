// bem2d C++ API (GB300 build): basis families.  PolBasis and LinBasis are
// assembled on the GPU; WaveBasis / WavePolBasis (complex valued) are
// declared for source compatibility and raise UnsupportedError in assembly.
#ifndef BEM2D_BASISTYPES_H
#define BEM2D_BASISTYPES_H

#include "bem2d_basis.h"
#include "bem2d_defs.h"
#include "bem2d_geometry.h"

namespace bem2d {

// Declared like the reference's: its operator() is not const, so the class
// stays abstract and cannot be instantiated.
class ConstBasis : public Basis {
 public:
  ConstBasis();
  complex operator()(double t) { return 1.0; }
};
typedef std::shared_ptr<ConstBasis> pConstBasis;

// t^degree
class PolBasis : public Basis {
 public:
  // adds PolBasis(0), ..., PolBasis(deg) to every element of pgeom
  static void AddBasis(int deg, pGeometry pgeom);
  explicit PolBasis(int degree);
  complex operator()(double t) const {
    double r = 1;
    for (int i = 0; i < degree_; ++i) r = r * t;
    return r;
  }
  int degree() const { return degree_; }

 private:
  int degree_;
};
typedef std::shared_ptr<PolBasis> pPolBasis;

// t (sign 1) or 1 - t (sign -1)
class LinBasis : public Basis {
 public:
  // adds LinBasis(1) then LinBasis(-1) to every element
  static void AddBasis(pGeometry pgeom);
  explicit LinBasis(int sign);
  complex operator()(double t) const { return sign_ == -1 ? 1 - t : t; }
  int sign() const { return sign_; }

 private:
  int sign_;
};
typedef std::shared_ptr<LinBasis> pLinBasis;

// exp(i k direction t)
class WaveBasis : public Basis {
 public:
  static void AddBasis(freqtype k, pGeometry pgeom);
  WaveBasis(double direction, freqtype k);
  complex operator()(double t) const;

 private:
  double direction_;
  freqtype k_;
};
typedef std::shared_ptr<WaveBasis> pWaveBasis;

// t^degree exp(i k direction t)
class WavePolBasis : public Basis {
 public:
  static void AddBasis(int degree, freqtype k, pGeometry pgeom);
  WavePolBasis(int degree, double direction, freqtype k);
  complex operator()(double t) const;

 private:
  double direction_;
  freqtype k_;
  int degree_;
};
typedef std::shared_ptr<WavePolBasis> pWavePolBasis;

}  // namespace bem2d

#endif
