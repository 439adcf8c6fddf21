// A program written against the bem2d C++ API (only "bem2d.h" and the public
// classes) that writes every text output format of the library into the
// current directory: WriteMatrix, WriteDensity (two columns, several bases
// per element), WriteDomain, MeshGrid + GplotOut, and GplotOutput's
// incident / scattered / full files with real and imaginary parts.  The
// same source is built against the reference library (oracle/Makefile,
// target ref_output: tests/golden/make_golden.py stores its files as
// fixtures) and against this build's library (tests/test_cpp_api.py), and
// the files must agree byte for byte.  No GPU work: only host-side types.
#include <cmath>
#include <vector>

#include "bem2d.h"

int main() {
  using bem2d::Point;
  // an L-shaped hexagon of straight elements, 3 per side, linked as a loop
  const double vx[] = {0.0, 1.0, 1.0, 0.5, 0.5, 0.0};
  const double vy[] = {0.0, 0.0, 0.5, 0.5, 1.0, 1.0};
  std::vector<bem2d::pElement> elems;
  const int per = 3, nv = 6, ne = per * nv;
  for (int s = 0; s < nv; ++s) {
    const Point a(vx[s], vy[s]), b(vx[(s + 1) % nv], vy[(s + 1) % nv]);
    for (int q = 0; q < per; ++q) {
      const Point p1 = a + (1.0 * q / per) * (b - a), p2 = a + (1.0 * (q + 1) / per) * (b - a);
      const int i = s * per + q;
      bem2d::pElement e(new bem2d::ConstElement(p1, p2, i));
      e->set_next((i + 1) % ne);
      e->set_prev((i + ne - 1) % ne);
      elems.push_back(e);
    }
  }
  bem2d::pGeometry g(new bem2d::Geometry(elems));
  bem2d::PolBasis::AddBasis(0, g);
  bem2d::LinBasis::AddBasis(g);
  const int n = (int)g->FlatMap()->size();

  // a deterministic complex matrix: n x 2 for the densities, n x n below
  bem2d::Matrix dens(n, 2);
  for (int c = 0; c < 2; ++c)
    for (int u = 0; u < n; ++u)
      (*dens.data)[c * n + u] = bem2d::complex(std::sin(0.37 * u + c) + 0.125 * c,
                                               std::cos(1.3 * u - 0.5 * c) / (1 + u));
  bem2d::WriteDensity("out_density", dens, g, 7);
  bem2d::WriteDomain("out_domain", g, 5);

  bem2d::Matrix m(6);
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i)
      (*m.data)[j * 6 + i] = bem2d::complex(1.0 / (1 + i + 2 * j), std::exp(-0.3 * i) - 0.25 * j);
  bem2d::WriteMatrix("out_matrix", m);

  // plotting grid and gnuplot files
  std::vector<Point> grid = *bem2d::MeshGrid(-1.0, 2.0, -0.5, 1.5, 4, 3);
  bem2d::dvector z(grid.size());
  for (std::size_t i = 0; i < grid.size(); ++i) z[i] = grid[i].x * grid[i].x - 0.5 * grid[i].y;
  bem2d::GplotOut("out_gplot", grid, z, 4, 3);
  bem2d::GplotOutput go(3, 5, -1.0, 1.0, 0.0, 2.0, "out_fre_");
  bem2d::GplotOutput gi(3, 5, -1.0, 1.0, 0.0, 2.0, "out_fim_");
  const std::vector<Point>& mesh = go.mesh();
  bem2d::cvector inc(mesh.size()), sca(mesh.size()), full(mesh.size());
  for (std::size_t i = 0; i < mesh.size(); ++i) {
    inc[i] = bem2d::complex(mesh[i].x, mesh[i].y);
    sca[i] = bem2d::complex(0.5 * mesh[i].y, -mesh[i].x);
    full[i] = inc[i] + sca[i];
  }
  go.WriteAll(inc, sca, full);
  gi.set_real(false);
  gi.WriteIncident(inc);
  gi.WriteScattered(sca);
  gi.WriteFull(full);
  return 0;
}
