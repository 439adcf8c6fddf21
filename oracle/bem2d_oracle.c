/*
 * CPU oracle for the bem2d Galerkin assembly path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain C restatement of the reference algorithm, written for checking the
 * GPU path and for timing a CPU baseline.  It follows, function by function:
 *   Gauss rule (Golub-Welsch)      lib/bem2d_quadrature.cpp:10-56
 *   MapPoints2d / Gauss2D          lib/bem2d_quadrature.cpp:69-76,
 *                                  lib/bem2d_quadpoints.cpp:31-73
 *   AdaptedGauss1/2/3              lib/bem2d_quadpoints.cpp:75-183
 *   element Map/Deriv/Normal       lib/bem2d_element.h:17-116
 *   curve types                    lib/bem2d_curvetypes.h:13-99
 *   bases PolBasis / LinBasis      lib/bem2d_basistypes.h:28-62
 *   kernels S, D, D', combined     lib/bem2d_kernel.cpp:15-112
 *   Hankel H0/H1 (real argument)   lib/bem2d_mathroutines.cpp:20-42, with
 *                                  POSIX j0/j1/y0/y1 standing in for GSL
 *   Hankel H0/H1 (complex argument, lib/bem2d_mathroutines.cpp:44-75, AMOS
 *   zbesh): binary128 series / asymptotic expansion (hankel_q.h)
 *   Integrate / IntegrateIdent     lib/bem2d_quadrature.h:37-109
 *   DiscreteKernel                 lib/bem2d_quadrature.h:231-294
 *   EvalIdent                      lib/bem2d_quadrature.cpp:79-127
 *   Integrate(testfun,fun) + DotProdBasFuns  lib/bem2d_quadrature.h:111-156
 *   PlaneWave / NormalPlaneWave / CombinedPlaneWave  lib/bem2d_fun.h:14-93
 */
#define _DEFAULT_SOURCE 1 /* POSIX j0/j1/y0/y1 */
#include "bem2d_oracle.h"
#include "hankel_q.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

enum { K_SINGLE = 0, K_DOUBLE = 1, K_CONJDOUBLE = 2, K_COMBINED = 3 };
enum { E_SEGMENT = 0, E_CIRCLE = 1, E_TREFOIL = 2, E_KITE = 3, E_ELLIPSE = 4,
       E_ELLIPSEARC = 5, E_INVELLIPSE = 6 };
enum { B_POLY = 0, B_LIN = 1 };

typedef struct { double re, im; } cplx;

static cplx cscale(cplx a, double s) {
  cplx r = {a.re * s, a.im * s};
  return r;
}

/* ---- Gauss rule: eigen-decomposition of the Jacobi matrix by implicit QL
 * with Wilkinson shifts (Golub-Welsch), lib/bem2d_quadrature.cpp:10-56. */
static int tridiag_ql(int n, double* d, double* e, double* z) {
  /* d: diagonal, e: sub-diagonal with e[n-1] = 0, z: n x n row-major,
   * initialised to the identity; column j of z is eigenvector j. */
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m;
      for (m = l; m < n - 1; ++m) {
        double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) <= 1e-300 + 2.2e-16 * dd) break;
      }
      if (m == l) break;
      if (++iter > 60) return -1;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
      double s = 1.0, c = 1.0, p = 0.0;
      int i;
      int early = 0;
      for (i = m - 1; i >= l; --i) {
        double f = s * e[i], b = c * e[i];
        r = hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[m] = 0.0;
          early = 1;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        for (int k = 0; k < n; ++k) {
          f = z[k * n + i + 1];
          z[k * n + i + 1] = s * z[k * n + i] + c * f;
          z[k * n + i] = c * z[k * n + i] - s * f;
        }
      }
      if (early) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  return 0;
}

int orc_gauss(int n, double* x, double* w) {
  if (n < 1) return -1;
  if (n == 1) {
    x[0] = 0.5;
    w[0] = 1.0;
    return 0;
  }
  double* d = (double*)calloc((size_t)n, sizeof(double));
  double* e = (double*)calloc((size_t)n, sizeof(double));
  double* z = (double*)calloc((size_t)n * n, sizeof(double));
  for (int i = 0; i < n; ++i) z[i * n + i] = 1.0;
  for (int i = 0; i < n - 1; ++i)
    e[i] = 0.5 / sqrt(1.0 - 1.0 / (4.0 * (i + 1) * (i + 1)));
  int rc = tridiag_ql(n, d, e, z);
  /* ascending order, as LAPACK dstev returns it */
  int* ord = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  for (int i = 1; i < n; ++i) {
    int v = ord[i], j = i - 1;
    while (j >= 0 && d[ord[j]] > d[v]) {
      ord[j + 1] = ord[j];
      --j;
    }
    ord[j + 1] = v;
  }
  for (int i = 0; i < n; ++i) {
    int j = ord[i];
    x[i] = (1.0 + d[j]) / 2.0;
    w[i] = z[j] * z[j]; /* first component of eigenvector j */
  }
  free(ord);
  free(d);
  free(e);
  free(z);
  return rc;
}

/* ---- quadrature rules on [0,1]^2 --------------------------------------- */
typedef struct {
  int n;
  double *x, *y, *w;
} rule2d;

static void rule_alloc(rule2d* r, int n) {
  r->n = 0;
  r->x = (double*)malloc(sizeof(double) * (size_t)n);
  r->y = (double*)malloc(sizeof(double) * (size_t)n);
  r->w = (double*)malloc(sizeof(double) * (size_t)n);
}
static void rule_free(rule2d* r) {
  free(r->x);
  free(r->y);
  free(r->w);
}

/* Gauss2D tensor rule, index i*N+j -> (xt[i], xt[j]), lib/bem2d_quadpoints.cpp:31-50 */
static void gauss2d(int N, const double* xt, const double* wt, rule2d* r) {
  rule_alloc(r, N * N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      r->x[i * N + j] = xt[i];
      r->y[i * N + j] = xt[j];
      r->w[i * N + j] = wt[i] * wt[j];
    }
  r->n = N * N;
}

/* Gauss2D::Rescale + MapPoints2d, appended to `r`. */
static void append_box(rule2d* r, const rule2d* g, double a, double b,
                       double c, double d) {
  for (int i = 0; i < g->n; ++i) {
    r->x[r->n] = a + (b - a) * g->x[i];
    r->y[r->n] = c + (d - c) * g->y[i];
    r->w[r->n] = (b - a) * (d - c) * g->w[i];
    r->n++;
  }
}

static void adapted1(const rule2d* g, int L, double sigma, rule2d* r) {
  double* xl = (double*)malloc(sizeof(double) * (size_t)(L + 1));
  for (int i = 0; i < L; ++i) xl[i] = pow(sigma, L - i);
  xl[L] = 1.0;
  rule_alloc(r, g->n * L * L);
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j)
      append_box(r, g, xl[i], xl[i + 1], xl[j], xl[j + 1]);
  free(xl);
}

static void adapted2(const rule2d* g, int L, double sigma, rule2d* r) {
  rule_alloc(r, 3 * g->n * L);
  double a = sigma, b = 1;
  while (L > 0) {
    append_box(r, g, 0, a, 1 - b, 1 - a);
    append_box(r, g, a, b, 1 - b, 1 - a);
    append_box(r, g, a, b, 1 - a, 1);
    a *= sigma;
    b *= sigma;
    L--;
  }
}

static void adapted3(const rule2d* g, int L, double sigma, rule2d* r) {
  rule_alloc(r, 3 * g->n * L);
  double a = 1, b = sigma;
  while (L > 0) {
    append_box(r, g, 1 - a, 1 - b, 0, b);
    append_box(r, g, 1 - a, 1 - b, b, a);
    append_box(r, g, 1 - b, 1, b, a);
    a *= sigma;
    b *= sigma;
    L--;
  }
}

/* ---- geometry ---------------------------------------------------------- */
static void curve_eval(int kind, const double* c, double t, double* mx,
                       double* my, double* dx, double* dy) {
  const double tp = 2 * ORC_PI * t;
  switch (kind) {
    case E_CIRCLE:
      *mx = cos(tp);
      *my = sin(tp);
      *dx = 2 * ORC_PI * (-1.0 * sin(tp));
      *dy = 2 * ORC_PI * cos(tp);
      break;
    case E_TREFOIL: {
      double r = 1 + 0.3 * cos(3 * 2 * ORC_PI * t);
      double rp = -0.3 * 3 * 2 * ORC_PI * sin(3 * 2 * ORC_PI * t);
      *mx = r * cos(tp);
      *my = r * sin(tp);
      *dx = rp * cos(tp) - r * 2 * ORC_PI * sin(tp);
      *dy = rp * sin(tp) + r * 2 * ORC_PI * cos(tp);
      break;
    }
    case E_KITE:
      *mx = cos(tp) + 0.65 * cos(4 * ORC_PI * t) - 0.65;
      *my = 1.5 * sin(tp);
      *dx = -2 * ORC_PI * sin(tp) - 0.65 * 4 * ORC_PI * sin(4 * ORC_PI * t);
      *dy = 1.5 * 2 * ORC_PI * cos(tp);
      break;
    case E_ELLIPSE: {
      double rho = c[0];
      *mx = rho * cos(tp);
      *my = 1 / rho * sin(tp);
      *dx = -rho * 2 * ORC_PI * sin(tp);
      *dy = 2 * ORC_PI / rho * cos(tp);
      break;
    }
    case E_ELLIPSEARC: {
      double a = c[0], b = c[1], t1 = c[2], t2 = c[3];
      double th = t1 + t * (t2 - t1);
      *mx = a * cos(th);
      *my = b * sin(th);
      *dx = -a * (t2 - t1) * sin(th);
      *dy = b * (t2 - t1) * cos(th);
      break;
    }
    case E_INVELLIPSE: {
      double al = c[0];
      /* e^s with s = 2*pi*t*i; q = 1 + al*e^{2s} */
      double er = cos(tp), ei = sin(tp);
      double e2r = er * er - ei * ei, e2i = 2 * er * ei;
      double qr = 1.0 + al * e2r, qi = al * e2i;
      double qn = qr * qr + qi * qi;
      /* res = e^s / q */
      *mx = (er * qr + ei * qi) / qn;
      *my = (ei * qr - er * qi) / qn;
      /* deriv = 2 pi i e^s (1 - al e^{2s}) / q^2 */
      double q2r = qr * qr - qi * qi, q2i = 2 * qr * qi;
      double q2n = q2r * q2r + q2i * q2i;
      double ur = 1.0 - al * e2r, ui = -al * e2i;
      double nr = er * ur - ei * ui, ni = er * ui + ei * ur; /* e^s (1-al e^2s) */
      double ir = -2 * ORC_PI * ni, ii = 2 * ORC_PI * nr;    /* times 2 pi i */
      *dx = (ir * q2r + ii * q2i) / q2n;
      *dy = (ii * q2r - ir * q2i) / q2n;
      break;
    }
    default:
      *mx = *my = *dx = *dy = NAN;
  }
}

typedef struct {
  double mx, my;  /* Map(t) */
  double dx, dy;  /* Deriv(t) */
} elem_pt;

static elem_pt elem_eval(const orc_geometry* g, int e, double t) {
  elem_pt r;
  const double* p = g->param + 8 * (size_t)e;
  if (g->kind[e] == E_SEGMENT) {
    double ddx = p[2] - p[0], ddy = p[3] - p[1];
    r.mx = p[0] + ddx * t;
    r.my = p[1] + ddy * t;
    r.dx = ddx;
    r.dy = ddy;
  } else {
    double t1 = p[0], t2 = p[1];
    double tt = t1 + t * (t2 - t1);
    double cx, cy;
    curve_eval(g->kind[e], p + 2, tt, &r.mx, &r.my, &cx, &cy);
    r.dx = (t2 - t1) * cx;
    r.dy = (t2 - t1) * cy;
  }
  return r;
}

static double plength(double x, double y) { return sqrt(x * x + y * y); }

static void normal_of(const elem_pt* p, double* nx, double* ny) {
  double ax = p->dy, ay = -p->dx;
  double l = plength(ax, ay);
  *nx = ax / l;
  *ny = ay / l;
}

static double basis_eval(const orc_geometry* g, int u, double t) {
  if (g->unk_kind[u] == B_LIN) return g->unk_param[u] == -1 ? 1 - t : t;
  int deg = (int)g->unk_param[u];
  double r = 1;
  for (int i = 0; i < deg; ++i) r = r * t;
  return r;
}

/* ---- kernels ----------------------------------------------------------- */
/* Complex wavenumber k + i ki (lib/bem2d_kernel.cpp:15-112, k.im != 0
 * branches): S = i/4 H0(kd), D / D' = -i k/4 H1(kd)/d (n.w), combined
 * D' - i eta S with eta real. */
static cplx kernel_eval_c(int kernel, double k, double ki, double eta, double xx, double xy,
                          double yx, double yy, double n1x, double n1y, double n2x,
                          double n2y) {
  double wx = xx - yx, wy = xy - yy;
  double d = plength(wx, wy);
  double h0r, h0i, h1r, h1i;
  orc_hankel01_q(k * d, ki * d, &h0r, &h0i, &h1r, &h1i);
  cplx r;
  if (kernel == K_SINGLE) {
    r.re = -h0i / 4.0;
    r.im = h0r / 4.0;
    return r;
  }
  double dot = kernel == K_DOUBLE ? -(n2x * wx + n2y * wy) : (n1x * wx + n1y * wy);
  /* p = k H1 dot / d; -i p / 4 */
  double pr = (k * h1r - ki * h1i) * dot / d, pi = (k * h1i + ki * h1r) * dot / d;
  r.re = pi / 4.0;
  r.im = -pr / 4.0;
  if (kernel == K_COMBINED) {
    r.re += eta * (h0r / 4.0);
    r.im += eta * (h0i / 4.0);
  }
  return r;
}

static cplx kernel_eval(int kernel, double k, double ki, double eta, double xx, double xy,
                        double yx, double yy, double n1x, double n1y,
                        double n2x, double n2y) {
  cplx r;
  if (ki != 0.0)
    return kernel_eval_c(kernel, k, ki, eta, xx, xy, yx, yy, n1x, n1y, n2x, n2y);
  if (kernel == K_SINGLE) {
    double d = plength(xx - yx, xy - yy);
    double kd = k * d;
    /* i/4 * (J0 + i Y0) */
    r.re = -y0(kd) / 4.0;
    r.im = j0(kd) / 4.0;
  } else if (kernel == K_DOUBLE) {
    double wx = yx - xx, wy = yy - xy;
    double d = plength(wx, wy);
    double kd = k * d, dot = n2x * wx + n2y * wy;
    double hr = j1(kd) / d * dot, hi = y1(kd) / d * dot;
    /* -i k/4 * (hr + i hi) */
    r.re = k / 4.0 * hi;
    r.im = -k / 4.0 * hr;
  } else {
    double wx = xx - yx, wy = xy - yy;
    double d = plength(wx, wy);
    double kd = k * d, dot = n1x * wx + n1y * wy;
    double hr = j1(kd) / d * dot, hi = y1(kd) / d * dot;
    r.re = k / 4.0 * hi;
    r.im = -k / 4.0 * hr;
    if (kernel == K_COMBINED) {
      /* cdlayer - i*eta*(i/4 H0) = cdlayer + eta/4 H0 */
      r.re += eta * (j0(kd) / 4.0);
      r.im += eta * (y0(kd) / 4.0);
    }
  }
  return r;
}

/* Integrate<kernel,T>, lib/bem2d_quadrature.h:37-65 */
static cplx integrate(const orc_geometry* g, int ui, int uj, int kernel,
                      double k, double ki, double eta, const rule2d* r) {
  int e1 = g->unk_elem[ui], e2 = g->unk_elem[uj];
  cplx acc = {0, 0};
  for (int q = 0; q < r->n; ++q) {
    elem_pt p1 = elem_eval(g, e1, r->x[q]);
    elem_pt p2 = elem_eval(g, e2, r->y[q]);
    double n1x, n1y, n2x, n2y;
    normal_of(&p1, &n1x, &n1y);
    normal_of(&p2, &n2x, &n2y);
    double f1 = basis_eval(g, ui, r->x[q]);
    double f2 = basis_eval(g, uj, r->y[q]);
    cplx v = kernel_eval(kernel, k, ki, eta, p1.mx, p1.my, p2.mx, p2.my, n1x, n1y,
                         n2x, n2y);
    double s1 = plength(p1.dx, p1.dy), s2 = plength(p2.dx, p2.dy);
    v = cscale(v, f1 * f2);
    v = cscale(v, s1);
    v = cscale(v, s2);
    v = cscale(v, r->w[q]);
    acc.re += v.re;
    acc.im += v.im;
  }
  return acc;
}

/* IntegrateIdent, lib/bem2d_quadrature.h:67-109 (Duffy split of the
 * self-element square into two triangles). */
static cplx integrate_ident(const orc_geometry* g, int ui, int uj, int kernel,
                            double k, double ki, double eta, const rule2d* r) {
  int e1 = g->unk_elem[ui], e2 = g->unk_elem[uj];
  cplx acc = {0, 0};
  for (int q = 0; q < r->n; ++q) {
    double x = r->x[q], y = r->y[q];
    double s[2] = {x, 1 - x};
    double t[2] = {(1 - y) * x, 1 - x + y * x};
    for (int h = 0; h < 2; ++h) {
      elem_pt p1 = elem_eval(g, e1, s[h]);
      elem_pt p2 = elem_eval(g, e2, t[h]);
      double n1x, n1y, n2x, n2y;
      normal_of(&p1, &n1x, &n1y);
      normal_of(&p2, &n2x, &n2y);
      double f1 = basis_eval(g, ui, s[h]);
      double f2 = basis_eval(g, uj, t[h]);
      cplx v = kernel_eval(kernel, k, ki, eta, p1.mx, p1.my, p2.mx, p2.my, n1x,
                           n1y, n2x, n2y);
      double s1 = plength(p1.dx, p1.dy), s2 = plength(p2.dx, p2.dy);
      v = cscale(v, x);
      v = cscale(v, f1 * f2);
      v = cscale(v, s1);
      v = cscale(v, s2);
      v = cscale(v, r->w[q]);
      acc.re += v.re;
      acc.im += v.im;
    }
  }
  return acc;
}

static cplx ident_entry(const orc_geometry* g, int ui, int uj, int N,
                        const double* x, const double* w) {
  int ej = g->unk_elem[uj];
  cplx acc = {0, 0};
  for (int t = 0; t < N; ++t) {
    elem_pt p = elem_eval(g, ej, x[t]);
    double s = plength(p.dx, p.dy);
    acc.re += s * basis_eval(g, ui, x[t]) * basis_eval(g, uj, x[t]) * w[t];
  }
  return acc;
}

typedef struct {
  double xt[64], wt[64];
  rule2d g0, g1, g2, g3;
} rules_t;

static int rules_make(rules_t* r, int L, int N, double sigma) {
  if (N < 1 || N > 64 || L < 0) return -1;
  if (orc_gauss(N, r->xt, r->wt)) return -2;
  gauss2d(N, r->xt, r->wt, &r->g0);
  adapted1(&r->g0, L, sigma, &r->g1);
  adapted2(&r->g0, L, sigma, &r->g2);
  adapted3(&r->g0, L, sigma, &r->g3);
  return 0;
}

static void rules_free(rules_t* r) {
  rule_free(&r->g0);
  rule_free(&r->g1);
  rule_free(&r->g2);
  rule_free(&r->g3);
}

/* One entry of beta*Id + alpha*K, with DiscreteKernel's rule selection
 * (lib/bem2d_quadrature.h:264-289). */
static cplx entry(const orc_geometry* g, const rules_t* r, int N, int i, int j,
                  int kernel, double k, double ki, double eta, double alpha, double beta) {
  int ei = g->unk_elem[i], ej = g->unk_elem[j];
  int64_t indi = g->index[ei], indj = g->index[ej];
  cplx v;
  int same = indi == indj;
  if (same) v = integrate_ident(g, i, j, kernel, k, ki, eta, &r->g1);
  else if (g->next[ei] == indj) v = integrate(g, i, j, kernel, k, ki, eta, &r->g3);
  else if (g->prev[ei] == indj) v = integrate(g, i, j, kernel, k, ki, eta, &r->g2);
  else v = integrate(g, i, j, kernel, k, ki, eta, &r->g0);
  cplx o = {alpha * v.re, alpha * v.im};
  if (beta != 0.0 && same) {
    cplx m = ident_entry(g, i, j, N, r->xt, r->wt);
    o.re += beta * m.re;
    o.im += beta * m.im;
  }
  return o;
}

int orc_discrete_kernel(const orc_geometry* g, int L, int N, double sigma,
                        int kernel, double k, double eta, double alpha,
                        double beta, double* out, int nthreads) {
  return orc_discrete_kernel_c(g, L, N, sigma, kernel, k, 0.0, eta, alpha, beta, out, nthreads);
}

int orc_discrete_kernel_c(const orc_geometry* g, int L, int N, double sigma,
                          int kernel, double k, double ki, double eta, double alpha,
                          double beta, double* out, int nthreads) {
  rules_t r;
  int rc = rules_make(&r, L, N, sigma);
  if (rc) return rc;
  const int n = g->n_unk;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) {
      cplx v = entry(g, &r, N, i, j, kernel, k, ki, eta, alpha, beta);
      out[2 * ((size_t)i + (size_t)n * j)] = v.re;
      out[2 * ((size_t)i + (size_t)n * j) + 1] = v.im;
    }
  }
  rules_free(&r);
  return 0;
}

int orc_discrete_kernel_rows(const orc_geometry* g, int L, int N, double sigma,
                             int kernel, double k, double eta, double alpha,
                             double beta, int nrows, const int32_t* rows,
                             double* out, int nthreads) {
  rules_t r;
  int rc = rules_make(&r, L, N, sigma);
  if (rc) return rc;
  const int n = g->n_unk;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int q = 0; q < nrows; ++q) {
    for (int j = 0; j < n; ++j) {
      cplx v = entry(g, &r, N, rows[q], j, kernel, k, 0.0, eta, alpha, beta);
      out[2 * ((size_t)q * n + j)] = v.re;
      out[2 * ((size_t)q * n + j) + 1] = v.im;
    }
  }
  rules_free(&r);
  return 0;
}

int orc_eval_ident(const orc_geometry* g, int N, double* out) {
  double xt[64], wt[64];
  if (N < 1 || N > 64) return -1;
  if (orc_gauss(N, xt, wt)) return -2;
  const int n = g->n_unk;
  memset(out, 0, sizeof(double) * 2 * (size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (g->index[g->unk_elem[i]] == g->index[g->unk_elem[j]]) {
        cplx m = ident_entry(g, i, j, N, xt, wt);
        out[2 * ((size_t)i + (size_t)n * j)] = m.re;
        out[2 * ((size_t)i + (size_t)n * j) + 1] = m.im;
      }
  return 0;
}

int orc_rhs(const orc_geometry* g, int N, int fun, double k, double dx,
            double dy, double eta, double scale, double* out) {
  return orc_rhs_c(g, N, fun, k, 0.0, dx, dy, eta, scale, out);
}

/* Complex wavenumber k + i ki: f = exp(i (k + i ki) d.x) (lib/bem2d_fun.h:14-93). */
int orc_rhs_c(const orc_geometry* g, int N, int fun, double k, double ki, double dx,
              double dy, double eta, double scale, double* out) {
  double xt[64], wt[64];
  if (N < 1 || N > 64) return -1;
  if (orc_gauss(N, xt, wt)) return -2;
  for (int u = 0; u < g->n_unk; ++u) {
    int e = g->unk_elem[u];
    cplx acc = {0, 0};
    for (int q = 0; q < N; ++q) {
      elem_pt p = elem_eval(g, e, xt[q]);
      double nx, ny;
      normal_of(&p, &nx, &ny);
      double dd = dx * p.mx + dy * p.my;
      double ph = k * dd;
      double amp = ki != 0.0 ? exp(-ki * dd) : 1.0;
      cplx f = {amp * cos(ph), amp * sin(ph)};
      cplx v;
      if (fun == 0) {
        v = f;
      } else {
        double nd = nx * dx + ny * dy;
        /* i (k + i ki) f */
        cplx ikf = {-k * f.im - ki * f.re, k * f.re - ki * f.im};
        v = cscale(ikf, nd);
        if (fun == 2) {
          /* - i eta f */
          v.re += eta * f.im;
          v.im -= eta * f.re;
        }
      }
      double s = plength(p.dx, p.dy);
      v = cscale(v, s);
      v = cscale(v, basis_eval(g, u, xt[q]));
      v = cscale(v, wt[q]);
      acc.re += v.re;
      acc.im += v.im;
    }
    out[2 * (size_t)u] = scale * acc.re;
    out[2 * (size_t)u + 1] = scale * acc.im;
  }
  return 0;
}

/* EvalKernel (lib/bem2d_quadrature.h:184-228): out[j] = sum_u c_u sum_q
 * K(p_j, y_uq) |J| phi_u(y_uq) w_q, both normals set to the source normal. */
int orc_potential(const orc_geometry* g, int N, int kernel, double k, double eta,
                  const double* coeffs, int npts, const double* pts, double* out) {
  return orc_potential_c(g, N, kernel, k, 0.0, eta, coeffs, npts, pts, out);
}

int orc_potential_c(const orc_geometry* g, int N, int kernel, double k, double ki, double eta,
                    const double* coeffs, int npts, const double* pts, double* out) {
  double xt[64], wt[64];
  if (N < 1 || N > 64) return -1;
  if (orc_gauss(N, xt, wt)) return -2;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int j = 0; j < npts; ++j) {
    double ar = 0, ai = 0;
    for (int u = 0; u < g->n_unk; ++u) {
      const int e = g->unk_elem[u];
      for (int q = 0; q < N; ++q) {
        elem_pt p = elem_eval(g, e, xt[q]);
        double nx, ny;
        normal_of(&p, &nx, &ny);
        cplx v = kernel_eval(kernel, k, ki, eta, pts[2 * j], pts[2 * j + 1], p.mx, p.my, nx,
                             ny, nx, ny);
        const double w = plength(p.dx, p.dy) * basis_eval(g, u, xt[q]) * wt[q];
        const double cr = coeffs[2 * u], ci = coeffs[2 * u + 1];
        ar += (cr * v.re - ci * v.im) * w;
        ai += (cr * v.im + ci * v.re) * w;
      }
    }
    out[2 * j] = ar;
    out[2 * j + 1] = ai;
  }
  return 0;
}
