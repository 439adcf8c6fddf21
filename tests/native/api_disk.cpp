// A program written against the bem2d C++ API as the reference's drivers are
// (only "bem2d.h" and the public classes): the unit disk with 160 equal-arc
// elements, k = 10, plane wave along x.  Prints the solution, the field at
// four points and norm / condition number, one number per line, for
// tests/test_cpp_api_gpu.py.
#include <cstdio>
#include <vector>

#include "bem2d.h"

int main() {
  bem2d::freqtype k = {10, 0};
  bem2d::pCurve circle(new bem2d::Circle);
  std::vector<bem2d::pElement> elems;
  const int n = 160;
  for (int i = 0; i < n; ++i) {
    bem2d::pElement e(new bem2d::AnalyticCurveElement(1.0 * i / n, 1.0 * (i + 1) / n, circle, i));
    e->set_next((i + 1) % n);
    e->set_prev((i + n - 1) % n);
    elems.push_back(e);
  }
  bem2d::pGeometry g(new bem2d::Geometry(elems));
  bem2d::PolBasis::AddBasis(0, g);
  bem2d::Point dir(1, 0);
  bem2d::PlaneWave pw(dir, k);
  bem2d::CombinedPlaneWave cpw(dir, k);
  bem2d::SoundSoftScattering<bem2d::PlaneWave, bem2d::CombinedPlaneWave> s(g, k, pw, cpw);
  s.Discretize();
  s.Solve();
  std::vector<bem2d::Point> pts;
  pts.push_back(bem2d::Point(-1.5, 0.0));
  pts.push_back(bem2d::Point(2.0, 1.0));
  pts.push_back(bem2d::Point(0.0, -3.0));
  pts.push_back(bem2d::Point(1.2, 0.4));
  bem2d::pcvector u = s.EvalSol(pts);
  double norm = 0, cond = 0;
  s.NormCond(norm, cond);
  // the combined operator's single and conjugate double layer, by the drivers' recipe
  bem2d::QuadOption q;
  q.L = 3;
  q.N = 5;
  q.sigma = 0.15;
  bem2d::Matrix dsl = *bem2d::DiscreteKernel(*g, q, bem2d::SingleLayer(k));
  bem2d::Matrix dcdl = *bem2d::DiscreteKernel(*g, q, bem2d::ConjDoubleLayer(k));
  bem2d::Matrix id = *bem2d::EvalIdent(*g, q);
  bem2d::Matrix comb = id + 2.0 * dcdl - bem2d::complex(0, 2.0) * k.re * dsl;
  bem2d::Matrix cb = bem2d::ChangeBasis(comb, id);
  double n2 = 0, c2 = 0;
  bem2d::L2NormCond(cb, n2, c2);
  std::printf("%.17g %.17g\n", norm, cond);
  std::printf("%.17g %.17g\n", n2, c2);
  for (std::size_t i = 0; i < u->size(); ++i) std::printf("%.17g %.17g\n", (*u)[i].real(), (*u)[i].imag());
  bem2d::Matrix a = *s.GetMatrix();
  std::printf("%.17g %.17g\n", (*a.data)[0].real(), (*a.data)[0].imag());
  return 0;
}
