// bem2d C++ API (GB300 build): Galerkin discretisation.  DiscreteKernel,
// EvalIdent, DotProdBasFuns and EvalKernel assemble on the GPU through the C
// ABI of include/bem2d_gpu.h (see bem2d_gpu_glue.cpp); the results come back
// as host matrices in the reference's layout.
#ifndef BEM2D_QUADRATURE_H
#define BEM2D_QUADRATURE_H

#include <type_traits>
#include <utility>
#include <vector>

#include "bem2d_defs.h"
#include "bem2d_exceptions.h"
#include "bem2d_fun.h"
#include "bem2d_geometry.h"
#include "bem2d_kernel.h"
#include "bem2d_mathroutines.h"
#include "bem2d_point.h"
#include "bem2d_quadpoints.h"

namespace bem2d {

// L graded levels and sigma for the singular pairs, N Gauss points per
// element direction
struct QuadOption {
  int L;
  int N;
  double sigma;
};

// Gauss-Legendre nodes / weights on [0,1]
void Gauss(dvector& x, dvector& w, int N);
void MapPoints(dvector& x, dvector& w, double a, double b);
void MapPoints2d(dvector& x, dvector& y, dvector& w, double a, double b, double c, double d);

// Galerkin matrix of a kernel over the geometry's basis functions
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, SingleLayer g);
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, DoubleLayer g);
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, ConjDoubleLayer g);
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, CombinedSingleConjDouble g);

template <typename kernel>
pMatrix DiscreteKernel(const Geometry&, QuadOption, kernel) {
  static_assert(!std::is_same<kernel, kernel>::value,
                "DiscreteKernel: only the library kernels (SingleLayer, DoubleLayer, "
                "ConjDoubleLayer, CombinedSingleConjDouble) are assembled on the GPU");
  return pMatrix();
}

// mass matrix <phi_i, phi_j>
pMatrix EvalIdent(const Geometry& geom, QuadOption opts);

// right-hand side <f, phi_i> for the plane-wave functionals
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, PlaneWave fun);
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, NormalPlaneWave fun);
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, CombinedPlaneWave fun);
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, IdFun fun);

template <typename Bem2dfun>
pMatrix DotProdBasFuns(const Geometry&, QuadOption, Bem2dfun) {
  static_assert(!std::is_same<Bem2dfun, Bem2dfun>::value,
                "DotProdBasFuns: only PlaneWave, NormalPlaneWave, CombinedPlaneWave and "
                "IdFun are evaluated on the GPU");
  return pMatrix();
}

// vals[j] += sum_u alpha_u sum_q g(points[j], y_uq) |J| phi_u(y_uq) w_q
// (the potential of the density alpha at the points; field evaluation)
namespace detail {
void EvalKernelGpu(const Geometry::flat_basis_map& basfuns, const std::vector<Point>& points,
                   cvector& vals, const complex* alpha, int kernel, freqtype k, double eta,
                   int N);
}

template <typename kernel>
void EvalKernel(const Geometry::flat_basis_map&, const std::vector<Point>&, cvector&, Matrix&,
                kernel, const Gauss1D&) {
  static_assert(!std::is_same<kernel, kernel>::value,
                "EvalKernel: only the library kernels are evaluated on the GPU");
}
inline void EvalKernel(const Geometry::flat_basis_map& basfuns,
                       const std::vector<Point>& points, cvector& vals, Matrix& alpha,
                       SingleLayer g, const Gauss1D& g1d) {
  detail::EvalKernelGpu(basfuns, points, vals, &(*alpha.data)[0], 0, g.k(), 0.0, g1d.Size());
}
inline void EvalKernel(const Geometry::flat_basis_map& basfuns,
                       const std::vector<Point>& points, cvector& vals, Matrix& alpha,
                       DoubleLayer g, const Gauss1D& g1d) {
  detail::EvalKernelGpu(basfuns, points, vals, &(*alpha.data)[0], 1, g.k(), 0.0, g1d.Size());
}
inline void EvalKernel(const Geometry::flat_basis_map& basfuns,
                       const std::vector<Point>& points, cvector& vals, Matrix& alpha,
                       ConjDoubleLayer g, const Gauss1D& g1d) {
  detail::EvalKernelGpu(basfuns, points, vals, &(*alpha.data)[0], 2, g.k(), 0.0, g1d.Size());
}
inline void EvalKernel(const Geometry::flat_basis_map& basfuns,
                       const std::vector<Point>& points, cvector& vals, Matrix& alpha,
                       CombinedSingleConjDouble g, const Gauss1D& g1d) {
  detail::EvalKernelGpu(basfuns, points, vals, &(*alpha.data)[0], 3, g.getk(), g.eta(),
                        g1d.Size());
}

// single basis function with coefficient alpha
template <typename kernel>
void EvalKernel(std::pair<pElement, pBasis>& basfun, const std::vector<Point>& points,
                cvector& vals, complex alpha, kernel g, Gauss1D& g1d) {
  if (points.size() != vals.size()) throw SizeError();
  Geometry::flat_basis_map one(1, basfun);
  Matrix a(1, 1);
  (*a.data)[0] = alpha;
  EvalKernel(one, points, vals, a, g, g1d);
}

}  // namespace bem2d

#endif
