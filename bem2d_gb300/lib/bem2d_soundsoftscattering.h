// bem2d C++ API (GB300 build): sound-soft scattering problem,
//   (1/2 I + D' - i eta S) phi = 1/2 (du_inc/dn - i eta u_inc)
// discretised as A = Id + 2 K_combined, b = 2 <f, phi_i>; assembly, solve and
// field evaluation on the GPU.
#ifndef BEM2D_SOUNDSOFTSCATTERING_H
#define BEM2D_SOUNDSOFTSCATTERING_H

#include <limits>
#include <vector>

#include "bem2d_defs.h"
#include "bem2d_fun.h"
#include "bem2d_geometry.h"
#include "bem2d_mathroutines.h"
#include "bem2d_outputhandler.h"
#include "bem2d_quadrature.h"

namespace bem2d {

namespace detail {
// A = Id + 2 K_combined(k, eta) on the GPU
pMatrix CombinedSystemMatrix(const Geometry& g, QuadOption q, freqtype k, double eta);
}

template <typename T1, typename T2>
class SoundSoftScattering {
 public:
  SoundSoftScattering(pGeometry geom, freqtype kvalue, T1 inc, T2 rhs)
      : pgeom_(geom), k_(kvalue), incident_(inc), frhs_(rhs), plotInterior_(false) {
    quadopts_.L = 3;
    quadopts_.N = 5;
    quadopts_.sigma = 0.15;
  }
  virtual ~SoundSoftScattering() {}

  void SetQuadOption(int L, int N, double sigma) {
    quadopts_.L = L;
    quadopts_.N = N;
    quadopts_.sigma = sigma;
  }
  virtual void DiscretizeMatrix() {
    pA_ = detail::CombinedSystemMatrix(*pgeom_, quadopts_, k_, frhs_.eta());
    pId_ = EvalIdent(*pgeom_, quadopts_);
  }
  virtual void DiscretizeRhs() {
    prhs_ = DotProdBasFuns(*pgeom_, quadopts_, frhs_);
    (*prhs_) = 2.0 * (*prhs_);
  }
  void Discretize() {
    DiscretizeMatrix();
    DiscretizeRhs();
  }
  void Solve() { psol_ = SolveSystem(*pA_, *prhs_); }
  pMatrix GetMatrix() const { return pA_; }
  pMatrix GetIdent() const { return pId_; }

  pcvector EvalIncident(const std::vector<Point>& points) {
    pcvector pz(new cvector(points.size()));
    std::vector<int> inpoly(points.size(), 0);
    if (plotInterior_ && !polygons_.empty()) InPolygon(polygons_, points, inpoly);
    for (std::size_t i = 0; i < points.size(); ++i)
      (*pz)[i] = inpoly[i] == 0 ? incident_(points[i])
                                : complex(std::numeric_limits<double>::quiet_NaN());
    return pz;
  }
  // u_inc - S phi at the points
  pcvector EvalSol(const std::vector<Point>& points) {
    std::shared_ptr<Geometry::flat_basis_map> bfuns = pgeom_->FlatMap();
    SingleLayer sl(k_);
    pcvector kerneleval(new cvector(points.size()));
    Gauss1D g1d(quadopts_.N);
    EvalKernel(*bfuns, points, *kerneleval, *psol_, sl, g1d);
    pcvector result = EvalIncident(points);
    for (std::size_t i = 0; i < points.size(); ++i) (*result)[i] -= (*kerneleval)[i];
    return result;
  }
  void NormCond(double& norm, double& cond) const {
    Matrix k = ChangeBasis(*pA_, *pId_);
    L2NormCond(k, norm, cond);
  }
  void SetOutput(pOutputHandler output) { pout_ = output; }
  void WriteIncident() { pout_->WriteIncident(*EvalIncident(pout_->mesh())); }
  void WriteScattered() {
    pcvector full = EvalSol(pout_->mesh()), inc = EvalIncident(pout_->mesh());
    cvector sc(*full);
    for (std::size_t i = 0; i < sc.size(); ++i) sc[i] -= (*inc)[i];
    pout_->WriteScattered(sc);
  }
  void WriteFull() { pout_->WriteFull(*EvalSol(pout_->mesh())); }
  void WriteAll() {
    pcvector inc = EvalIncident(pout_->mesh()), full = EvalSol(pout_->mesh());
    cvector sc(*full);
    for (std::size_t i = 0; i < sc.size(); ++i) sc[i] -= (*inc)[i];
    pout_->WriteAll(*inc, sc, *full);
  }
  void set_polygons(std::vector<pGeometry>& polygons) { polygons_ = polygons; }
  void set_polygons(pGeometry polygon) { polygons_.push_back(polygon); }
  void set_plotInterior() { plotInterior_ = true; }

 private:
  pGeometry pgeom_;
  freqtype k_;
  T1 incident_;
  T2 frhs_;
  pOutputHandler pout_;
  QuadOption quadopts_;
  pMatrix pA_, pId_, prhs_, psol_;
  std::vector<pGeometry> polygons_;
  bool plotInterior_;
};

}  // namespace bem2d

#endif
