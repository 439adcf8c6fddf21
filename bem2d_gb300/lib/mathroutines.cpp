// bem2d C++ API (GB300 build): Matrix and the dense linear algebra.  LU solve,
// norms / condition numbers, change of basis and the numerical range run on
// the GPU (include/bem2d_gpu.h), and so does the matrix product; the
// elementwise operators stay on the host where the reference's Matrix lives.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <thread>
#include <vector>

#include "bem2d_mathroutines.h"
#include "bem2d_pnpoly.h"
#include "gpu_glue.h"

namespace bem2d {

Matrix::Matrix(int n) : data(new cvector((size_t)n * n)), msize(n), nsize(n) {
  dim[0] = n;
  dim[1] = n;
}
Matrix::Matrix(int m, int n) : data(new cvector((size_t)m * n)), msize(m), nsize(n) {
  dim[0] = m;
  dim[1] = n;
}
Matrix::Matrix(const Matrix& m) : data(new cvector(*m.data)), msize(m.msize), nsize(m.nsize) {
  dim[0] = m.dim[0];
  dim[1] = m.dim[1];
}

// Elementwise operators: host passes over the reference's host-resident
// Matrix (it calls zaxpy / zscal there), split over the hardware threads.
template <typename F>
static void parallel_for(std::size_t n, F f) {
  const std::size_t grain = (std::size_t)1 << 18;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const std::size_t nt = std::min<std::size_t>(hw, (n + grain - 1) / grain);
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const std::size_t chunk = (n + nt - 1) / nt;
  for (std::size_t t = 0; t < nt; ++t) {
    const std::size_t a = t * chunk, b = std::min(n, a + chunk);
    if (a < b) th.emplace_back(f, a, b);
  }
  for (auto& t : th) t.join();
}

Matrix operator+(const Matrix& lhs, const Matrix& rhs) {
  if (lhs.dim[0] != rhs.dim[0] || lhs.dim[1] != rhs.dim[1]) throw ArrayMismatch();
  Matrix r(rhs);
  complex* d = &(*r.data)[0];
  const complex* a = &(*lhs.data)[0];
  parallel_for(r.data->size(), [=](std::size_t b, std::size_t e) {
    for (std::size_t i = b; i < e; ++i) d[i] += a[i];
  });
  return r;
}
Matrix operator-(const Matrix& lhs, const Matrix& rhs) {
  if (lhs.dim[0] != rhs.dim[0] || lhs.dim[1] != rhs.dim[1]) throw ArrayMismatch();
  Matrix r(lhs);
  complex* d = &(*r.data)[0];
  const complex* a = &(*rhs.data)[0];
  parallel_for(r.data->size(), [=](std::size_t b, std::size_t e) {
    for (std::size_t i = b; i < e; ++i) d[i] -= a[i];
  });
  return r;
}
Matrix operator*(const Matrix& lhs, const complex& alpha) {
  Matrix r(lhs);
  complex* d = &(*r.data)[0];
  parallel_for(r.data->size(), [=](std::size_t b, std::size_t e) {
    for (std::size_t i = b; i < e; ++i) d[i] *= alpha;
  });
  return r;
}
Matrix operator*(const complex& alpha, const Matrix& rhs) { return rhs * alpha; }
Matrix operator*(const Matrix& lhs, const double& alpha) {
  Matrix r(lhs);
  complex* d = &(*r.data)[0];
  parallel_for(r.data->size(), [=](std::size_t b, std::size_t e) {
    for (std::size_t i = b; i < e; ++i) d[i] *= alpha;
  });
  return r;
}
Matrix operator*(const double& alpha, const Matrix& rhs) { return rhs * alpha; }

// Matrix product on the GPU (bem2d_matmul): the reference calls cblas_zgemm
Matrix operator*(const Matrix& lhs, const Matrix& rhs) {
  if (lhs.dim[1] != rhs.dim[0]) throw ArrayMismatch();
  const int m = lhs.dim[0], n = rhs.dim[1], k = lhs.dim[1];
  Matrix r(m, n);
  detail::check(bem2d_matmul(detail::ctx(), m, n, k, &(*lhs.data)[0], m, &(*rhs.data)[0], k,
                             &(*r.data)[0], m),
                "Matrix product");
  return r;
}

static int g_precision = -1;
void SetSolverPrecision(int p) { g_precision = p; }
int GetSolverPrecision() {
  if (g_precision < 0) {
    const char* e = std::getenv("BEM2D_PRECISION");
    g_precision = (e && std::strcmp(e, "mixed") == 0)        ? BEM2D_PREC_MIXED
                  : (e && std::strcmp(e, "mixed_tf32") == 0) ? BEM2D_PREC_MIXED_TF32
                                                             : BEM2D_PREC_FP64;
  }
  return g_precision;
}

pMatrix SolveSystem(Matrix& m, Matrix& rhs) {
  if (m.dim[0] != m.dim[1] || rhs.dim[0] != m.dim[0]) throw ArrayMismatch();
  const int n = m.dim[0];
  pMatrix res(new Matrix(rhs));
  for (int j = 0; j < rhs.dim[1]; ++j) {
    bem2d_solve_info info;
    detail::check(bem2d_solve_system(detail::ctx(), n, &(*m.data)[0], n, &(*rhs.data)[(size_t)n * j],
                                     &(*res->data)[(size_t)n * j], GetSolverPrecision(), 0.0, &info),
                  "SolveSystem");
  }
  return res;
}

void L2NormCond(const Matrix& stiff, double& norm, double& cond) {
  if (stiff.dim[0] != stiff.dim[1]) throw ArrayMismatch();
  detail::check(bem2d_l2_norm_cond(detail::ctx(), stiff.dim[0], &(*stiff.data)[0], stiff.dim[0], 0.0,
                                   &norm, &cond),
                "L2NormCond");
}

void SingularValues(const Matrix& stiff, pdvector& singvals) {
  if (stiff.dim[0] != stiff.dim[1]) throw ArrayMismatch();
  const int n = stiff.dim[0];
  singvals = pdvector(new dvector(n));
  detail::check(bem2d_singular_values(detail::ctx(), n, &(*stiff.data)[0], n, &(*singvals)[0]),
                "SingularValues");
}
void HermitianEigenvalues(const Matrix& k, pdvector& evalues) {
  if (k.dim[0] != k.dim[1]) throw ArrayMismatch();
  const int n = k.dim[0];
  evalues = pdvector(new dvector(n));
  detail::check(bem2d_hermitian_eigenvalues(detail::ctx(), n, &(*k.data)[0], n, &(*evalues)[0]),
                "HermitianEigenvalues");
}
void Eigenvalues(const Matrix& k, pcvector& evalues) {
  if (k.dim[0] != k.dim[1]) throw ArrayMismatch();
  const int n = k.dim[0];
  evalues = pcvector(new cvector(n));
  detail::check(bem2d_eigenvalues(detail::ctx(), n, &(*k.data)[0], n, &(*evalues)[0]),
                "Eigenvalues");
}
void Eigenvalues(const Matrix& k, pcvector& evalues, pMatrix& evectors) {
  const int n = k.dim[0];
  evalues = pcvector(new cvector(n));
  evectors = pMatrix(new Matrix(n));
  detail::check(bem2d_eigenvectors(detail::ctx(), n, &(*k.data)[0], n, &(*evalues)[0],
                                   &(*evectors->data)[0], n),
                "Eigenvalues");
}

Matrix ChangeBasis(const Matrix& k, const Matrix& m) {
  const int n = k.dim[0];
  if (k.dim[1] != n || m.dim[0] != n || m.dim[1] != n) throw ArrayMismatch();
  // blocks of the (block-diagonal) mass matrix: maximal runs closed under
  // the nonzero pattern
  const complex* M = &(*m.data)[0];
  std::vector<int32_t> bstart(1, 0);
  int end = 0;
  for (int i = 0; i < n; ++i) {
    for (int j = i; j < n; ++j)
      if (M[i + (size_t)n * j] != complex(0) || M[j + (size_t)n * i] != complex(0)) end = std::max(end, j);
    if (end == i) bstart.push_back(i + 1);
    else if (end < i) end = i;
  }
  Matrix out(n);
  detail::check(bem2d_change_basis(detail::ctx(), n, &(*k.data)[0], n, M, n, bstart.data(),
                                   (int)bstart.size() - 1, &(*out.data)[0], n),
                "ChangeBasis");
  return out;
}

void NumRange(const Matrix& m, int n, std::string filename) {
  const int N = m.dim[0];
  const double step = PI / n;
  // lambda_max at th_i and th_i + pi (the latter gives lambda_min(th_i))
  std::vector<double> th(2 * n), lmax(2 * n);
  for (int i = 0; i < n; ++i) {
    th[i] = i * step;
    th[n + i] = i * step + PI;
  }
  detail::check(bem2d_num_range(detail::ctx(), N, &(*m.data)[0], N, 2 * n, th.data(), 0.0,
                                GetSolverPrecision() == BEM2D_PREC_FP64 ? BEM2D_PREC_FP64
                                                                        : BEM2D_PREC_MIXED,
                                lmax.data()),
                "NumRange");
  dvector eigs(2 * n), steps(2 * n);
  for (int i = 0; i < n; ++i) {
    steps[i] = i * step;
    steps[n + i] = i * step;
    eigs[i] = -lmax[n + i];  // lambda_min
    eigs[n + i] = lmax[i];
  }
  steps.push_back(0);
  eigs.push_back(eigs[0]);
  const complex im(0, 1);
  cvector pts(2 * n + 1);
  for (int i = 0; i < 2 * n; ++i) {
    const double c1 = std::cos(steps[i]), c2 = std::cos(steps[i + 1]);
    const double s1 = std::sin(steps[i]), s2 = std::sin(steps[i + 1]);
    const double t1 = (eigs[i + 1] - eigs[i] * (c1 * c2 + s1 * s2)) / (s1 * c2 - s2 * c1);
    pts[i] = std::exp(-im * steps[i]) * (eigs[i] + im * t1);
  }
  pts[2 * n] = pts[0];
  std::ofstream out(filename.c_str());
  for (int i = 0; i < 2 * n + 1; ++i) out << std::real(pts[i]) << " " << std::imag(pts[i]) << std::endl;
}

Matrix ConjTranspose(const Matrix& m) {
  const int M = m.dim[0], N = m.dim[1];
  Matrix r(N, M);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < N; ++j) (*r.data)[j + (size_t)N * i] = std::conj((*m.data)[i + (size_t)M * j]);
  return r;
}

Matrix ExtractColumn(const Matrix& m, int j) {
  Matrix r(m.dim[0], 1);
  for (int i = 0; i < m.dim[0]; ++i) (*r.data)[i] = (*m.data)[(size_t)j * m.dim[0] + i];
  return r;
}

complex DotProduct(const Matrix& a, const Matrix& b) {
  if (a.nsize != 1 || b.nsize != 1 || a.msize != b.msize) throw ArrayMismatch();
  complex s = 0;
  for (int i = 0; i < a.msize; ++i) s += std::conj((*a.data)[i]) * (*b.data)[i];
  return s;
}

int pnpoly(int nvert, double* vx, double* vy, double tx, double ty) {
  int c = 0;
  for (int i = 0, j = nvert - 1; i < nvert; j = i++)
    if (((vy[i] > ty) != (vy[j] > ty)) && (tx < (vx[j] - vx[i]) * (ty - vy[i]) / (vy[j] - vy[i]) + vx[i]))
      c = !c;
  return c;
}

void InPolygon(const pGeometry polygon, const std::vector<Point>& testpoints, std::vector<int>& inpoly) {
  const PointVector& p = polygon->points();
  std::vector<double> vx(p.size()), vy(p.size());
  for (std::size_t i = 0; i < p.size(); ++i) {
    vx[i] = p[i].x;
    vy[i] = p[i].y;
  }
  for (std::size_t i = 0; i < testpoints.size(); ++i)
    if (pnpoly((int)p.size(), vx.data(), vy.data(), testpoints[i].x, testpoints[i].y)) inpoly[i] = 1;
}

void InPolygon(const std::vector<pGeometry> polygons, const std::vector<Point>& testpoints,
               std::vector<int>& inpoly) {
  for (const pGeometry& g : polygons) InPolygon(g, testpoints, inpoly);
}

}  // namespace bem2d
