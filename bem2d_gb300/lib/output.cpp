// bem2d C++ API (GB300 build): text output (plot grids, matrices, densities).
#include <fstream>

#include "bem2d_outputhandler.h"
#include "bem2d_outputroutines.h"

namespace bem2d {

void Abrange(dvector& xx, double a, double b, int n) {
  xx.resize(n);
  for (int i = 0; i < n; ++i) xx[i] = n > 1 ? a + (b - a) * i / (n - 1) : a;
}

std::shared_ptr<std::vector<Point> > MeshGrid(double ax, double bx, double ay, double by, int xpts,
                                              int ypts) {
  dvector xs, ys;
  Abrange(xs, ax, bx, xpts);
  Abrange(ys, ay, by, ypts);
  std::shared_ptr<std::vector<Point> > p(new std::vector<Point>);
  for (int j = 0; j < ypts; ++j)
    for (int i = 0; i < xpts; ++i) p->push_back(Point(xs[i], ys[j]));
  return p;
}

void GplotOut(std::string name, const std::vector<Point>& points, const dvector& z, int xpts, int ypts) {
  std::ofstream d((name + ".dat").c_str());
  for (int j = 0; j < ypts; ++j) {
    for (int i = 0; i < xpts; ++i) {
      const std::size_t k = (std::size_t)j * xpts + i;
      d << points[k].x << " " << points[k].y << " " << z[k] << "\n";
    }
    d << "\n";
  }
  std::ofstream s((name + ".gnuplot").c_str());
  s << "set pm3d map\nset size ratio -1\nsplot '" << name << ".dat' with pm3d notitle\n";
}

void WriteMatrix(std::string fname, const Matrix m) {
  std::ofstream out(fname.c_str());
  out.precision(16);
  for (int i = 0; i < m.dim[0]; ++i) {
    for (int j = 0; j < m.dim[1]; ++j) {
      const complex v = (*m.data)[i + (size_t)m.dim[0] * j];
      out << std::real(v) << " " << std::imag(v) << " ";
    }
    out << "\n";
  }
}

void WriteDensity(std::string name, const Matrix& m, pGeometry pgeom, int npoints) {
  std::shared_ptr<Geometry::flat_basis_map> fm = pgeom->FlatMap();
  std::ofstream out(name.c_str());
  out.precision(16);
  std::vector<pElement>& el = pgeom->elements();
  for (std::size_t e = 0; e < el.size(); ++e)
    for (int q = 0; q < npoints; ++q) {
      const double t = npoints > 1 ? (double)q / (npoints - 1) : 0.5;
      complex v = 0;
      for (std::size_t u = 0; u < fm->size(); ++u)
        if ((*fm)[u].first == el[e]) v += (*m.data)[u] * (*(*fm)[u].second)(t);
      const Point p = el[e]->Map(t);
      out << p.x << " " << p.y << " " << std::real(v) << " " << std::imag(v) << "\n";
    }
}

void WriteDomain(std::string name, pGeometry pgeom, int npoints) {
  std::ofstream out(name.c_str());
  for (const pElement& e : pgeom->elements()) {
    for (int q = 0; q < npoints; ++q) {
      const Point p = e->Map(npoints > 1 ? (double)q / (npoints - 1) : 0.5);
      out << p.x << " " << p.y << "\n";
    }
    out << "\n";
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
  mesh_ = *MeshGrid(ax, bx, ay, by, xpts, ypts);
}

void GplotOutput::Write(const std::string& field, const cvector& vals) {
  GplotOut(name_ + "_" + field + "_real", mesh_, *RealData(vals), xpts_, ypts_);
  GplotOut(name_ + "_" + field + "_imag", mesh_, *ImagData(vals), xpts_, ypts_);
}
void GplotOutput::WriteIncident(const cvector& vals) { Write("incident", vals); }
void GplotOutput::WriteScattered(const cvector& vals) { Write("scattered", vals); }
void GplotOutput::WriteFull(const cvector& vals) { Write("full", vals); }
void GplotOutput::WriteAll(const cvector& a, const cvector& b, const cvector& c) {
  WriteIncident(a);
  WriteScattered(b);
  WriteFull(c);
}

}  // namespace bem2d
