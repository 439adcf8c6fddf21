// bem2d C++ API (GB300 build): Helmholtz kernels (functor objects).  Passed to
// DiscreteKernel they select the GPU kernel; operator() evaluates one value on
// the host with the same Hankel evaluator the GPU uses.
#ifndef BEM2D_KERNEL_H
#define BEM2D_KERNEL_H

#include "bem2d_defs.h"
#include "bem2d_point.h"

namespace bem2d {

// i/4 H0(k |x - y|)
class SingleLayer {
 public:
  explicit SingleLayer(freqtype k) : k_(k) {}
  SingleLayer(const SingleLayer& s) = default;
  complex operator()(Point x, Point y) const;
  void SetNormal(Point normal1, Point normal2) {
    n1_ = normal1;
    n2_ = normal2;
  }
  freqtype k() const { return k_; }

 private:
  freqtype k_;
  Point n1_, n2_;
};

// -(i k/4) H1(k d)/d n2.(y - x)
class DoubleLayer {
 public:
  explicit DoubleLayer(freqtype k) : k_(k) {}
  DoubleLayer(const DoubleLayer& d) = default;
  complex operator()(Point x, Point y) const;
  void SetNormal(Point normal1, Point normal2) {
    n1_ = normal1;
    n2_ = normal2;
  }
  freqtype k() const { return k_; }

 private:
  freqtype k_;
  Point n1_, n2_;
};

// -(i k/4) H1(k d)/d n1.(x - y)
class ConjDoubleLayer {
 public:
  explicit ConjDoubleLayer(freqtype k) : k_(k) {}
  ConjDoubleLayer(const ConjDoubleLayer& d) = default;
  complex operator()(Point x, Point y) const;
  void SetNormal(Point normal1, Point normal2) {
    n1_ = normal1;
    n2_ = normal2;
  }
  freqtype k() const { return k_; }

 private:
  freqtype k_;
  Point n1_, n2_;
};

// ConjDoubleLayer - i eta SingleLayer (eta defaults to k.re)
class CombinedSingleConjDouble {
 public:
  CombinedSingleConjDouble(freqtype k, double eta) : k_(k), eta_(eta) {}
  explicit CombinedSingleConjDouble(freqtype k) : k_(k), eta_(k.re) {}
  CombinedSingleConjDouble(const CombinedSingleConjDouble& s) = default;
  complex operator()(Point x, Point y) const;
  void SetNormal(Point normal1, Point normal2) {
    n1_ = normal1;
    n2_ = normal2;
  }
  freqtype getk() const { return k_; }
  double eta() const { return eta_; }

 private:
  freqtype k_;
  Point n1_, n2_;
  double eta_;
};

class IdKernel {
 public:
  void SetNormal(Point, Point) {}
  complex operator()(Point, Point) const { return 1.0; }
};

}  // namespace bem2d

#endif
