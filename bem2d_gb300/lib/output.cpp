// bem2d C++ API (GB300 build): text output (plot grids, matrices, densities).
#include <fstream>
#include <map>

#include "bem2d_outputhandler.h"
#include "bem2d_outputroutines.h"

namespace bem2d {

// The text formats below are the reference library's
// (lib/bem2d_outputroutines.cpp): same file names, point order, sampling and
// column layout, default stream formatting, so drivers write the same files.

void Abrange(dvector& xx, double a, double b, int n) {
  xx.resize(n);
  const double h = 1.0 / (n - 1);
  for (int i = 0; i < n; ++i) xx[i] = a + h * i * (b - a);
}

// x outer, y inner: point (i, j) at index i * ypts + j
std::shared_ptr<std::vector<Point> > MeshGrid(double ax, double bx, double ay, double by, int xpts,
                                              int ypts) {
  dvector xs, ys;
  Abrange(xs, ax, bx, xpts);
  Abrange(ys, ay, by, ypts);
  std::shared_ptr<std::vector<Point> > p(new std::vector<Point>);
  p->reserve((std::size_t)xpts * ypts);
  for (int i = 0; i < xpts; ++i)
    for (int j = 0; j < ypts; ++j) p->push_back(Point(xs[i], ys[j]));
  return p;
}

// data file `name` (a blank line after each x column) and gnuplot script
// `name`_gplot
void GplotOut(std::string name, const std::vector<Point>& points, const dvector& z, int xpts,
              int ypts) {
  {
    std::ofstream d(name.c_str());
    for (int i = 0; i < xpts; ++i) {
      for (int j = 0; j < ypts; ++j) {
        const std::size_t k = (std::size_t)i * ypts + j;
        d << points[k].x << " " << points[k].y << " " << z[k] << "\n";
      }
      d << "\n";
    }
  }
  std::ofstream s((name + "_gplot").c_str());
  s << "set pm3d map\n"
    << "set hidden3d\n"
    << "set datafile missing \"nan\"\n"
    << "set palette rgbformulae 33,13,10\n"
    << "set size ratio -1\n"
    << "set size square\n"
    << "set cbrange [-1:1]\n"
    << "splot '" << name << "'\n"
    << "pause -1\n";
}

// `fname`_real and `fname`_imag: row i holds entries (i, j) of the leading
// dim[0] x dim[0] block, each followed by a space
void WriteMatrix(std::string fname, const Matrix m) {
  std::ofstream re((fname + "_real").c_str());
  std::ofstream im((fname + "_imag").c_str());
  const int n = m.dim[0];
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) {
      const complex v = (*m.data)[(std::size_t)j * n + i];
      re << std::real(v) << " ";
      im << std::imag(v) << " ";
    }
    re << std::endl;
    im << std::endl;
  }
}

// Per element (geometry order), npoints samples at t = j / npoints: the point
// Map(t), then for every column of m the real parts, then the imaginary
// parts, of sum_u m(u, col) phi_u.  The basis argument is the integer
// quotient j / npoints (0 for every sample), as in the reference's
// (*base)(j/npoints).
void WriteDensity(std::string name, const Matrix& m, pGeometry pgeom, int npoints) {
  std::vector<pElement> el = pgeom->elements();
  std::shared_ptr<Geometry::flat_basis_map> fm = pgeom->FlatMap();
  std::map<std::size_t, std::size_t> pos;  // element index() -> position
  for (std::size_t e = 0; e < el.size(); ++e) pos[el[e]->index()] = e;
  const int ncol = m.dim[1];
  std::vector<std::vector<Point> > pts(el.size());
  std::vector<std::vector<cvector> > val(el.size());
  for (std::size_t u = 0; u < fm->size(); ++u) {
    const pElement& elem = (*fm)[u].first;
    const pBasis& base = (*fm)[u].second;
    const std::size_t e = pos[elem->index()];
    if (pts[e].empty()) {
      for (int j = 0; j < npoints; ++j) pts[e].push_back(elem->Map((1.0 * j) / npoints));
      val[e].assign(npoints, cvector(ncol));
    }
    for (int j = 0; j < npoints; ++j)
      for (int c = 0; c < ncol; ++c)
        val[e][j][c] += (*base)(j / npoints) * (*m.data)[(std::size_t)c * m.dim[0] + u];
  }
  std::ofstream out(name.c_str());
  for (std::size_t e = 0; e < el.size(); ++e)
    for (int j = 0; j < npoints; ++j) {
      out << pts[e][j].x << " " << pts[e][j].y << " ";
      for (int c = 0; c < ncol; ++c) out << std::real(val[e][j][c]) << " ";
      for (int c = 0; c < ncol; ++c) out << std::imag(val[e][j][c]) << " ";
      out << std::endl;
    }
}

// Map(j / npoints), j < npoints, for every element in geometry order
void WriteDomain(std::string name, pGeometry pgeom, int npoints) {
  std::vector<pElement> el = pgeom->elements();
  std::ofstream out(name.c_str());
  for (std::size_t e = 0; e < el.size(); ++e)
    for (int j = 0; j < npoints; ++j) {
      const Point p = el[e]->Map((1.0 * j) / npoints);
      out << p.x << " " << p.y << std::endl;
    }
}

pdvector OutputHandler::RealData(const cvector& vals) {
  pdvector r(new dvector(vals.size()));
  for (std::size_t i = 0; i < vals.size(); ++i) (*r)[i] = std::real(vals[i]);
  return r;
}
pdvector OutputHandler::ImagData(const cvector& vals) {
  pdvector r(new dvector(vals.size()));
  for (std::size_t i = 0; i < vals.size(); ++i) (*r)[i] = std::imag(vals[i]);
  return r;
}
pdvector OutputHandler::TurnToRealImag(const cvector& vals) { return real_ ? RealData(vals) : ImagData(vals); }

GplotOutput::GplotOutput(int xpts, int ypts, double ax, double bx, double ay, double by, std::string name)
    : name_(name), xpts_(xpts), ypts_(ypts) {
  set_real(true);
  isroot_ = true;
  mesh_ = *MeshGrid(ax, bx, ay, by, xpts, ypts);
}

// <name>inc, <name>scatt, <name>full: the real (set_real(true), the default)
// or imaginary parts on the mesh
void GplotOutput::WriteIncident(const cvector& vals) {
  GplotOut(name_ + "inc", mesh_, *TurnToRealImag(vals), xpts_, ypts_);
}
void GplotOutput::WriteScattered(const cvector& vals) {
  GplotOut(name_ + "scatt", mesh_, *TurnToRealImag(vals), xpts_, ypts_);
}
void GplotOutput::WriteFull(const cvector& vals) {
  GplotOut(name_ + "full", mesh_, *TurnToRealImag(vals), xpts_, ypts_);
}
void GplotOutput::WriteAll(const cvector& a, const cvector& b, const cvector& c) {
  WriteIncident(a);
  WriteScattered(b);
  WriteFull(c);
}

}  // namespace bem2d
