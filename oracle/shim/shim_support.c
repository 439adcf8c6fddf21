/*
 * Link-time stand-ins for the third-party libraries the reference library
 * calls (GSL, LAPACK, CBLAS, AMOS).  Test infrastructure only: this file is
 * compiled into oracle/_ref together with the reference sources, which are
 * compiled in place and never copied.
 *
 *  - GSL real Bessel J0/J1/Y0/Y1 -> POSIX libm j0/j1/y0/y1.
 *  - LAPACK/CBLAS -> the OpenBLAS that scipy bundles, whose exported names
 *    carry a "scipy_" prefix (same LP64 signatures).
 *  - GSL qag / odeiv (curve length, arc-length parametrisation) -> simple
 *    fixed rules; these only feed AnalyticCurve, which the parity cases
 *    do not use.
 *  - AMOS zbesh_ (complex wavenumbers only) -> H0 / H1 of the first kind
 *    (fnu = 0, 1; kode = 1; one value) in 113-bit binary128 arithmetic
 *    (../hankel_q.h).  Checked against scipy.special.hankel1 (AMOS itself)
 *    when the fixtures are generated.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../hankel_q.h"


#include "gsl/gsl_integration.h"
#include "gsl/gsl_odeiv.h"
#include "gsl/gsl_sf_bessel.h"

/* ---- GSL Bessel (lib/bem2d_mathroutines.cpp:20-42) -------------------- */
double gsl_sf_bessel_J0(double x) { return j0(x); }
double gsl_sf_bessel_J1(double x) { return j1(x); }
double gsl_sf_bessel_Y0(double x) { return y0(x); }
double gsl_sf_bessel_Y1(double x) { return y1(x); }

/* ---- GSL integration (lib/bem2d_curve.cpp:15-28) ----------------------- */
static const double kGL8x[4] = {0.1834346424956498, 0.5255324099163290,
                                0.7966664774136267, 0.9602898564975363};
static const double kGL8w[4] = {0.3626837833783620, 0.3137066458778873,
                                0.2223810344533745, 0.1012285362903763};

gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) {
  (void)n;
  return (gsl_integration_workspace*)calloc(1, sizeof(gsl_integration_workspace));
}
void gsl_integration_workspace_free(gsl_integration_workspace* w) { free(w); }

int gsl_integration_qag(const gsl_function* f, double a, double b,
                        double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace* w, double* result,
                        double* abserr) {
  (void)epsabs; (void)epsrel; (void)limit; (void)key; (void)w;
  const int panels = 512;
  double h = (b - a) / panels, sum = 0.0;
  for (int p = 0; p < panels; ++p) {
    double c = a + (p + 0.5) * h, r = 0.5 * h;
    for (int q = 0; q < 4; ++q) {
      sum += kGL8w[q] * r * (f->function(c - r * kGL8x[q], f->params) +
                             f->function(c + r * kGL8x[q], f->params));
    }
  }
  *result = sum;
  *abserr = 0.0;
  return 0;
}

/* ---- GSL odeiv (lib/bem2d_shape.cpp:334-368) --------------------------- */
static const gsl_odeiv_step_type kRk2Type = {0};
const gsl_odeiv_step_type* gsl_odeiv_step_rk2 = &kRk2Type;

gsl_odeiv_step* gsl_odeiv_step_alloc(const gsl_odeiv_step_type* T, size_t dim) {
  (void)T;
  gsl_odeiv_step* s = (gsl_odeiv_step*)calloc(1, sizeof(gsl_odeiv_step));
  s->dim = dim;
  return s;
}
void gsl_odeiv_step_free(gsl_odeiv_step* s) { free(s); }
gsl_odeiv_control* gsl_odeiv_control_y_new(double eps_abs, double eps_rel) {
  (void)eps_rel;
  gsl_odeiv_control* c = (gsl_odeiv_control*)calloc(1, sizeof(gsl_odeiv_control));
  c->eps = eps_abs;
  return c;
}
void gsl_odeiv_control_free(gsl_odeiv_control* c) { free(c); }
gsl_odeiv_evolve* gsl_odeiv_evolve_alloc(size_t dim) {
  gsl_odeiv_evolve* e = (gsl_odeiv_evolve*)calloc(1, sizeof(gsl_odeiv_evolve));
  e->dim = dim;
  return e;
}
void gsl_odeiv_evolve_free(gsl_odeiv_evolve* e) { free(e); }

/* Advances the scalar ODE from *t to t1 in 256 classical RK4 sub-steps. */
int gsl_odeiv_evolve_apply(gsl_odeiv_evolve* e, gsl_odeiv_control* con,
                           gsl_odeiv_step* step, const gsl_odeiv_system* sys,
                           double* t, double t1, double* h, double y[]) {
  (void)e; (void)con; (void)step; (void)h;
  const int sub = 256;
  double dt = (t1 - *t) / sub, tt = *t, yy = y[0];
  for (int i = 0; i < sub; ++i) {
    double k1, k2, k3, k4, tmp;
    sys->function(tt, &yy, &k1, sys->params);
    tmp = yy + 0.5 * dt * k1;
    sys->function(tt + 0.5 * dt, &tmp, &k2, sys->params);
    tmp = yy + 0.5 * dt * k2;
    sys->function(tt + 0.5 * dt, &tmp, &k3, sys->params);
    tmp = yy + dt * k3;
    sys->function(tt + dt, &tmp, &k4, sys->params);
    yy += dt / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4);
    tt += dt;
  }
  *t = t1;
  y[0] = yy;
  return 0;
}

/* ---- LAPACK (lib/bem2d_defs.h:37-58) ----------------------------------- */
typedef struct { double re, im; } zc;
void scipy_dstev_(char*, int*, double*, double*, double*, int*, double*, int*);
void scipy_zaxpy_(int*, zc*, zc*, int*, zc*, int*);
void scipy_zgetrf_(int*, int*, zc*, int*, int*, int*);
void scipy_zgetrs_(char*, int*, int*, zc*, int*, int*, zc*, int*, int*);
void scipy_zgesvd_(char*, char*, int*, int*, zc*, int*, double*, zc*, int*,
                   zc*, int*, zc*, int*, double*, int*);
void scipy_zpotrf_(const char*, const int*, zc*, const int*, int*);
void scipy_zheev_(const char*, const char*, const int*, zc*, const int*,
                  double*, zc*, const int*, double*, int*);
void scipy_zgeev_(const char*, const char*, const int*, zc*, const int*, zc*,
                  zc*, const int*, zc*, const int*, zc*, const int*, double*,
                  int*);

void dstev_(char* a, int* b, double* c, double* d, double* e, int* f,
            double* g, int* h) { scipy_dstev_(a, b, c, d, e, f, g, h); }
void zaxpy_(int* a, zc* b, zc* c, int* d, zc* e, int* f) {
  scipy_zaxpy_(a, b, c, d, e, f);
}
void zgetrf_(int* a, int* b, zc* c, int* d, int* e, int* f) {
  scipy_zgetrf_(a, b, c, d, e, f);
}
void zgetrs_(char* a, int* b, int* c, zc* d, int* e, int* f, zc* g, int* h,
             int* i) { scipy_zgetrs_(a, b, c, d, e, f, g, h, i); }
void zgesvd_(char* a, char* b, int* c, int* d, zc* e, int* f, double* g,
             zc* h, int* i, zc* j, int* k, zc* l, int* m, double* n, int* o) {
  scipy_zgesvd_(a, b, c, d, e, f, g, h, i, j, k, l, m, n, o);
}
void zpotrf_(const char* a, const int* b, zc* c, const int* d, int* e) {
  scipy_zpotrf_(a, b, c, d, e);
}
void zheev_(const char* a, const char* b, const int* c, zc* d, const int* e,
            double* f, zc* g, const int* h, double* i, int* j) {
  scipy_zheev_(a, b, c, d, e, f, g, h, i, j);
}
void zgeev_(const char* a, const char* b, const int* c, zc* d, const int* e,
            zc* f, zc* g, const int* h, zc* i, const int* j, zc* k,
            const int* l, double* m, int* n) {
  scipy_zgeev_(a, b, c, d, e, f, g, h, i, j, k, l, m, n);
}

/* ---- CBLAS (lib/bem2d_cblas.h) ----------------------------------------- */
void scipy_cblas_zaxpy(int, const void*, const void*, int, void*, int);
void scipy_cblas_zscal(int, const void*, void*, int);
void scipy_cblas_zdscal(int, double, void*, int);
void scipy_cblas_zgemm(int, int, int, int, int, int, const void*, const void*,
                       int, const void*, int, const void*, void*, int);
void scipy_cblas_ztrsm(int, int, int, int, int, int, int, const void*,
                       const void*, int, void*, int);
void scipy_cblas_zdotc_sub(int, const void*, int, const void*, int, void*);

void cblas_zaxpy(const int N, const void* alpha, const void* X, const int incX,
                 void* Y, const int incY) {
  scipy_cblas_zaxpy(N, alpha, X, incX, Y, incY);
}
void cblas_zscal(const int N, const void* alpha, void* X, const int incX) {
  scipy_cblas_zscal(N, alpha, X, incX);
}
void cblas_zdscal(const int N, const double alpha, void* X, const int incX) {
  scipy_cblas_zdscal(N, alpha, X, incX);
}
void cblas_zgemm(const int Order, const int TransA, const int TransB,
                 const int M, const int N, const int K, const void* alpha,
                 const void* A, const int lda, const void* B, const int ldb,
                 const void* beta, void* C, const int ldc) {
  scipy_cblas_zgemm(Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb,
                    beta, C, ldc);
}
void cblas_ztrsm(const int Order, const int Side, const int Uplo,
                 const int TransA, const int Diag, const int M, const int N,
                 const void* alpha, const void* A, const int lda, void* B,
                 const int ldb) {
  scipy_cblas_ztrsm(Order, Side, Uplo, TransA, Diag, M, N, alpha, A, lda, B,
                    ldb);
}
void cblas_zdotc_sub(const int N, const void* X, const int incX, const void* Y,
                     const int incY, void* dotc) {
  scipy_cblas_zdotc_sub(N, X, incX, Y, incY, dotc);
}

/* ---- AMOS (lib/bem2d_mathroutines.cpp:44-75) --------------------------- */
void zbesh_(const double* zr, const double* zi, const double* fnu,
            const int* kode, const int* M, const int* N, double* cyr,
            double* cyi, int* nz, int* ierr) {
  *nz = 0;
  if ((*fnu != 0.0 && *fnu != 1.0) || *kode != 1 || *M != 1 || *N != 1 ||
      (*zr == 0.0 && *zi == 0.0)) {
    fprintf(stderr, "oracle: zbesh shim covers H0/H1 of the first kind only\n");
    *cyr = NAN;
    *cyi = NAN;
    *ierr = 4;
    return;
  }
  const qcplx h = hankel1_q((int)*fnu, (qreal)*zr, (qreal)*zi);
  *cyr = (double)h.re;
  *cyi = (double)h.im;
  *ierr = 0;
}
