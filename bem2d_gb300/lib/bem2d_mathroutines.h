// bem2d C++ API (GB300 build): dense matrices and the linear-algebra routines
// of the reference (LU solve, norms, change of basis, numerical range).  The
// heavy routines run on the GPU through include/bem2d_gpu.h.
#ifndef BEM2D_MATHROUTINES_H
#define BEM2D_MATHROUTINES_H

#include <string>
#include <vector>

#include "bem2d_defs.h"
#include "bem2d_exceptions.h"
#include "bem2d_geometry.h"
#include "bem2d_point.h"

namespace bem2d {

// Hankel functions of the first kind, real argument (host evaluation with
// the GPU's evaluator).  Complex arguments are not supported in this build.
complex BesselH0(double x);
complex BesselH1(double x);
complex BesselH0(complex x);
complex BesselH1(complex x);

// m x n complex matrix, column-major, entry (i,j) at data[i + m*j]
struct Matrix {
  explicit Matrix(int n);
  explicit Matrix(int m, int n);
  Matrix(const Matrix& m);
  Matrix& operator=(const Matrix& m) = default;
  pcvector data;
  int dim[2];
  int msize;
  int nsize;
};

typedef std::shared_ptr<Matrix> pMatrix;

Matrix operator+(const Matrix& lhs, const Matrix& rhs);
Matrix operator-(const Matrix& lhs, const Matrix& rhs);
Matrix operator*(const Matrix& lhs, const complex& alpha);
Matrix operator*(const complex& alpha, const Matrix& rhs);
Matrix operator*(const Matrix& lhs, const double& alpha);
Matrix operator*(const double& alpha, const Matrix& rhs);
Matrix operator*(const Matrix& lhs, const Matrix& rhs);

// ||A||_2 and cond_2(A) from the extreme singular values (GPU Lanczos).
void L2NormCond(const Matrix& stiff, double& norm, double& cond);
// All singular values, descending (GPU Householder tridiagonalisation of
// [0 A; A^H 0] and bisection).
void SingularValues(const Matrix& stiff, pdvector& singvals);
// x = m^{-1} rhs (GPU LU; precision from BEM2D_PRECISION=fp64|mixed|mixed_tf32).
pMatrix SolveSystem(Matrix& m, Matrix& rhs);
// All eigenvalues of the Hermitian matrix the upper triangle of k defines,
// ascending (GPU Householder tridiagonalisation and bisection).
void HermitianEigenvalues(const Matrix& k, pdvector& evalues);
// All eigenvalues of a general matrix (GPU Hessenberg reduction and
// shifted QR); the variant with eigenvectors is not available in this build
// (UnsupportedError).
void Eigenvalues(const Matrix& k, pcvector& evalues);
void Eigenvalues(const Matrix& k, pcvector& evalues, pMatrix& evectors);
// U^{-H} k U^{-1} with m = U^H U (m block diagonal per element, as mass
// matrices are).
Matrix ChangeBasis(const Matrix& k, const Matrix& m);
// Boundary of the numerical range of m from n angles in [0, pi): 2n+1
// points written to `filename`, as the reference does.
void NumRange(const Matrix& m, int n, std::string filename);
Matrix ConjTranspose(const Matrix& m);
Matrix ExtractColumn(const Matrix& m, int j);
complex DotProduct(const Matrix& a, const Matrix& b);

void InPolygon(const std::vector<pGeometry> polygons, const std::vector<Point>& testpoints,
               std::vector<int>& inpoly);
void InPolygon(const pGeometry polygon, const std::vector<Point>& testpoints,
               std::vector<int>& inpoly);

// Solver precision of SolveSystem / SoundSoftScattering::Solve:
// 0 = complex128 LU (default), 1 = complex64 LU + FP64 refinement,
// 2 = as 1 with 1xTF32 tensor-core updates in the LU.
void SetSolverPrecision(int precision);
int GetSolverPrecision();

}  // namespace bem2d

#endif
