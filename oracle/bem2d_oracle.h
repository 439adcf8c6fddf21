/*
 * CPU oracle for the bem2d Galerkin assembly path: a plain C restatement of
 * the reference's algorithm (TEST INFRASTRUCTURE ONLY).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or the timed CPU baseline, never as the product path.
 *
 * Geometry tables use the same layout as the GPU C-ABI (include/bem2d_gpu.h):
 * one row of 8 doubles per element plus index/next/prev, and a flat
 * (element, basis) list in Geometry::FlatMap() order.
 */
#ifndef BEM2D_ORACLE_H
#define BEM2D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t n_elem;
  const int32_t* kind;     /* element kind, see BEM2D_ELEM_* in bem2d_gpu.h */
  const double* param;     /* n_elem x 8 */
  const int64_t* index;
  const int64_t* next;
  const int64_t* prev;
  int32_t n_unk;
  const int32_t* unk_elem;  /* position of the unknown's element */
  const int32_t* unk_kind;  /* basis kind, see BEM2D_BASIS_* */
  const double* unk_param;  /* degree (poly) or sign (lin) */
} orc_geometry;

/* Gauss-Legendre rule on [0,1] by Golub-Welsch (implicit QL). */
int orc_gauss(int n, double* x, double* w);

/* out (complex128, n_unk x n_unk, column-major) = beta*Id + alpha*K. */
int orc_discrete_kernel(const orc_geometry* g, int L, int N, double sigma,
                        int kernel, double k, double eta, double alpha,
                        double beta, double* out, int nthreads);

/* orc_discrete_kernel with a complex wavenumber k + i ki. */
int orc_discrete_kernel_c(const orc_geometry* g, int L, int N, double sigma,
                          int kernel, double k, double ki, double eta, double alpha,
                          double beta, double* out, int nthreads);

/* rows of beta*Id + alpha*K: out[q*n_unk + j] = entry (rows[q], j). */
int orc_discrete_kernel_rows(const orc_geometry* g, int L, int N, double sigma,
                             int kernel, double k, double eta, double alpha,
                             double beta, int nrows, const int32_t* rows,
                             double* out, int nthreads);

/* out = mass matrix (EvalIdent). */
int orc_eval_ident(const orc_geometry* g, int N, double* out);

/* out (complex128, n_unk) = scale * <f, phi_i> for the incident-field
 * functional `fun` (0 = PlaneWave, 1 = NormalPlaneWave, 2 = CombinedPlaneWave). */
int orc_rhs(const orc_geometry* g, int N, int fun, double k, double dx,
            double dy, double eta, double scale, double* out);

/* orc_rhs with a complex wavenumber k + i ki. */
int orc_rhs_c(const orc_geometry* g, int N, int fun, double k, double ki, double dx,
              double dy, double eta, double scale, double* out);

/* potential of the density coeffs (complex128[n_unk]) at npts points
 * (x0 y0 x1 y1 ...): EvalKernel. */
int orc_potential(const orc_geometry* g, int N, int kernel, double k, double eta,
                  const double* coeffs, int npts, const double* pts, double* out);

/* orc_potential with a complex wavenumber k + i ki. */
int orc_potential_c(const orc_geometry* g, int N, int kernel, double k, double ki, double eta,
                    const double* coeffs, int npts, const double* pts, double* out);

#ifdef __cplusplus
}
#endif
#endif
