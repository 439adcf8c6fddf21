// Golden-vector generator: a small driver written against the reference
// library's public C++ API (the reference sources are compiled in place into
// oracle/_ref, never copied).  Test infrastructure only.
//
// It reads a case description (the same element table the GPU C-ABI takes),
// runs the reference's own assembly / solve / norm routines and writes raw
// little-endian complex128 (column-major) or float64 outputs.
//
// Input format, one directive per line ('#' starts a comment):
//   quad L N sigma
//   seg  p1x p1y p2x p2y index next prev          (ConstElement)
//   curve KIND t1 t2 c0 c1 c2 c3 index next prev   (AnalyticCurveElement)
//        KIND: circle trefoil kite ellipse(c0=rho) ellipsearc(c0..c3=a,b,th1,th2)
//              invellipse(c0=alpha)
//   basis poly DEG | basis lin SIGN                (Geometry::AddBasis to all)
//   op kernel single|double|conjdouble|combined KRE KIM ETA OUTFILE
//   op ident OUTFILE
//   op scattering KRE KIM DX DY ETA PREFIX   -> PREFIX_A.bin PREFIX_rhs.bin
//                                               PREFIX_x.bin PREFIX_normcond.bin
//   op numrange KRE KIM ETA NANG OUTFILE     (NumRange of ChangeBasis(A,Id))
//   op singvals KRE KIM ETA OUTFILE          (SingularValues of ChangeBasis(A,Id))
//   op timing KRE KIM DX DY ETA OUTFILE      (wall-clock seconds: assemble, solve)
//   op evalsol KRE KIM DX DY ETA OUTFILE X0 Y0 X1 Y1 ...  (EvalSol at the points)
//   op hankel OUTFILE ZR0 ZI0 ZR1 ZI1 ...    (BesselH0, BesselH1 of complex z:
//                                             H0(z0) H1(z0) H0(z1) ... complex128)
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "bem2d.h"

using namespace bem2d;

namespace {

void WriteComplex(const std::string& path, const Matrix& m) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(&(*m.data)[0], sizeof(complex), m.data->size(), f);
  std::fclose(f);
}

void WriteDoubles(const std::string& path, const std::vector<double>& v) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

pCurve MakeCurve(const std::string& kind, double c0, double c1, double c2,
                 double c3) {
  if (kind == "circle") return pCurve(new Circle);
  if (kind == "trefoil") return pCurve(new Trefoil);
  if (kind == "kite") return pCurve(new Kite);
  if (kind == "ellipse") return pCurve(new Ellipse(c0));
  if (kind == "ellipsearc") return pCurve(new EllipseArc(c0, c1, c2, c3));
  if (kind == "invellipse") return pCurve(new InvEllipse(c0));
  throw std::runtime_error("unknown curve " + kind);
}

struct Case {
  QuadOption quad;
  std::vector<pElement> elems;
  std::vector<std::pair<std::string, double> > bases;
  pGeometry geom;
};

pGeometry BuildGeometry(Case& c) {
  pGeometry g(new Geometry(c.elems));
  for (size_t b = 0; b < c.bases.size(); ++b) {
    if (c.bases[b].first == "poly")
      g->AddBasis(pBasis(new PolBasis((int)c.bases[b].second)));
    else
      g->AddBasis(pBasis(new LinBasis((int)c.bases[b].second)));
  }
  return g;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    std::cerr << "usage: ref_dump CASEFILE" << std::endl;
    return 2;
  }
  std::ifstream in(argv[1]);
  Case c;
  c.quad.L = 3;
  c.quad.N = 5;
  c.quad.sigma = 0.15;
  std::string line;
  std::vector<std::string> ops;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    std::string key;
    ss >> key;
    if (key == "quad") {
      ss >> c.quad.L >> c.quad.N >> c.quad.sigma;
    } else if (key == "seg") {
      double x1, y1, x2, y2;
      long idx, nxt, prv;
      ss >> x1 >> y1 >> x2 >> y2 >> idx >> nxt >> prv;
      pElement e(new ConstElement(Point(x1, y1), Point(x2, y2), idx));
      e->set_next(nxt);
      e->set_prev(prv);
      c.elems.push_back(e);
    } else if (key == "curve") {
      std::string kind;
      double t1, t2, c0, c1, c2, c3;
      long idx, nxt, prv;
      ss >> kind >> t1 >> t2 >> c0 >> c1 >> c2 >> c3 >> idx >> nxt >> prv;
      pElement e(new AnalyticCurveElement(t1, t2, MakeCurve(kind, c0, c1, c2, c3), idx));
      e->set_next(nxt);
      e->set_prev(prv);
      c.elems.push_back(e);
    } else if (key == "basis") {
      std::string kind;
      double p;
      ss >> kind >> p;
      c.bases.push_back(std::make_pair(kind, p));
    } else if (key == "op") {
      ops.push_back(line);
    }
  }
  c.geom = BuildGeometry(c);
  const Geometry& g = *c.geom;

  for (size_t o = 0; o < ops.size(); ++o) {
    std::istringstream ss(ops[o]);
    std::string key, what;
    ss >> key >> what;
    if (what == "kernel") {
      std::string kname, out;
      double kre, kim, eta;
      ss >> kname >> kre >> kim >> eta >> out;
      freqtype k = {kre, kim};
      pMatrix m;
      if (kname == "single") m = DiscreteKernel(g, c.quad, SingleLayer(k));
      else if (kname == "double") m = DiscreteKernel(g, c.quad, DoubleLayer(k));
      else if (kname == "conjdouble") m = DiscreteKernel(g, c.quad, ConjDoubleLayer(k));
      else m = DiscreteKernel(g, c.quad, CombinedSingleConjDouble(k, eta));
      WriteComplex(out, *m);
    } else if (what == "hankel") {
      std::string out;
      ss >> out;
      double zr, zi;
      Matrix m(1);
      m.data->clear();
      while (ss >> zr >> zi) {
        m.data->push_back(BesselH0(complex(zr, zi)));
        m.data->push_back(BesselH1(complex(zr, zi)));
      }
      WriteComplex(out, m);
    } else if (what == "ident") {
      std::string out;
      ss >> out;
      WriteComplex(out, *EvalIdent(g, c.quad));
    } else if (what == "scattering" || what == "timing") {
      double kre, kim, dx, dy, eta;
      std::string prefix;
      ss >> kre >> kim >> dx >> dy >> eta >> prefix;
      freqtype k = {kre, kim};
      Point dir(dx, dy);
      PlaneWave pw(dir, k);
      CombinedPlaneWave cpw(dir, k, eta);
      SoundSoftScattering<PlaneWave, CombinedPlaneWave> ss3(c.geom, k, pw, cpw);
      ss3.SetQuadOption(c.quad.L, c.quad.N, c.quad.sigma);
      auto t0 = std::chrono::steady_clock::now();
      ss3.DiscretizeMatrix();
      // DiscretizeRhs keeps its result private; recompute it the same way
      // (lib/bem2d_soundsoftscattering.h:105-110).
      pMatrix rhs = DotProdBasFuns(g, c.quad, cpw);
      *rhs = 2.0 * (*rhs);
      auto t1 = std::chrono::steady_clock::now();
      pMatrix x = SolveSystem(*ss3.GetMatrix(), *rhs);
      auto t2 = std::chrono::steady_clock::now();
      if (what == "timing") {
        std::vector<double> t;
        t.push_back(std::chrono::duration<double>(t1 - t0).count());
        t.push_back(std::chrono::duration<double>(t2 - t1).count());
        WriteDoubles(prefix, t);
        continue;
      }
      WriteComplex(prefix + "_A.bin", *ss3.GetMatrix());
      WriteComplex(prefix + "_rhs.bin", *rhs);
      WriteComplex(prefix + "_x.bin", *x);
      double norm = 0, cond = 0;
      ss3.NormCond(norm, cond);
      std::vector<double> nc;
      nc.push_back(norm);
      nc.push_back(cond);
      WriteDoubles(prefix + "_normcond.bin", nc);
    } else if (what == "evalsol") {
      double kre, kim, dx, dy, eta;
      std::string out;
      ss >> kre >> kim >> dx >> dy >> eta >> out;
      std::vector<Point> pts;
      double px, py;
      while (ss >> px >> py) pts.push_back(Point(px, py));
      freqtype k = {kre, kim};
      Point dir(dx, dy);
      PlaneWave pw(dir, k);
      CombinedPlaneWave cpw(dir, k, eta);
      SoundSoftScattering<PlaneWave, CombinedPlaneWave> s3(c.geom, k, pw, cpw);
      s3.SetQuadOption(c.quad.L, c.quad.N, c.quad.sigma);
      s3.Discretize();
      s3.Solve();
      pcvector v = s3.EvalSol(pts);
      Matrix m((int)pts.size(), 1);
      *m.data = *v;
      WriteComplex(out, m);
    } else if (what == "numrange" || what == "singvals") {
      double kre, kim, eta;
      int nang = 0;
      std::string out;
      ss >> kre >> kim >> eta;
      if (what == "numrange") ss >> nang;
      ss >> out;
      freqtype k = {kre, kim};
      Matrix kmat = *DiscreteKernel(g, c.quad, CombinedSingleConjDouble(k, eta));
      Matrix id = *EvalIdent(g, c.quad);
      Matrix a = id + 2.0 * kmat;
      Matrix b = ChangeBasis(a, id);
      if (what == "numrange") {
        NumRange(b, nang, out);
      } else {
        pdvector sv;
        SingularValues(b, sv);
        WriteDoubles(out, *sv);
      }
    } else {
      std::cerr << "unknown op " << what << std::endl;
      return 3;
    }
  }
  return 0;
}
