// Shared device-side definitions of the bem2d GB300 path: element geometry,
// bases, kernel functions and the internal launch interfaces between the
// translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/bem2d_gpu.h"
#include "hankel_c.cuh"

namespace bem2d_gpu {

constexpr double kPi = 3.14159265358979323846;

// ---- device view of a geometry ------------------------------------------
// Element table and flat unknown list (see bem2d_geometry in bem2d_gpu.h).
struct DevGeom {
  int n_elem;
  int n_unk;
  const int* kind;
  const double* param;  // 8 per element
  const long long* index;
  const long long* next;
  const long long* prev;
  const int* unk_elem;
  const int* unk_kind;
  const double* unk_param;
};

// Element Map(t) and Deriv(t) (lib/bem2d_element.h:72-116): an affine
// ConstElement or an AnalyticCurveElement on one of the library curves
// (lib/bem2d_curvetypes.h:13-99), evaluated in FP64.
struct ElemPt {
  double mx, my, dx, dy;
};

__device__ __forceinline__ void curve_eval(int kind, const double* c, double t,
                                           ElemPt* r) {
  const double tp = 2 * kPi * t;
  double s, co;
  switch (kind) {
    case BEM2D_ELEM_CIRCLE:
      sincos(tp, &s, &co);
      r->mx = co;
      r->my = s;
      r->dx = 2 * kPi * (-1.0 * s);
      r->dy = 2 * kPi * co;
      break;
    case BEM2D_ELEM_TREFOIL: {
      sincos(tp, &s, &co);
      double s3, c3;
      sincos(3 * 2 * kPi * t, &s3, &c3);
      const double rr = 1 + 0.3 * c3;
      const double rp = -0.3 * 3 * 2 * kPi * s3;
      r->mx = rr * co;
      r->my = rr * s;
      r->dx = rp * co - rr * 2 * kPi * s;
      r->dy = rp * s + rr * 2 * kPi * co;
      break;
    }
    case BEM2D_ELEM_KITE: {
      sincos(tp, &s, &co);
      double s2, c2;
      sincos(4 * kPi * t, &s2, &c2);
      r->mx = co + 0.65 * c2 - 0.65;
      r->my = 1.5 * s;
      r->dx = -2 * kPi * s - 0.65 * 4 * kPi * s2;
      r->dy = 1.5 * 2 * kPi * co;
      break;
    }
    case BEM2D_ELEM_ELLIPSE: {
      const double rho = c[0];
      sincos(tp, &s, &co);
      r->mx = rho * co;
      r->my = 1 / rho * s;
      r->dx = -rho * 2 * kPi * s;
      r->dy = 2 * kPi / rho * co;
      break;
    }
    case BEM2D_ELEM_ELLIPSEARC: {
      const double a = c[0], b = c[1], t1 = c[2], t2 = c[3];
      sincos(t1 + t * (t2 - t1), &s, &co);
      r->mx = a * co;
      r->my = b * s;
      r->dx = -a * (t2 - t1) * s;
      r->dy = b * (t2 - t1) * co;
      break;
    }
    case BEM2D_ELEM_INVELLIPSE: {
      // z(t) = e^s / (1 + alpha e^{2s}), s = 2 pi i t
      const double al = c[0];
      double s2, c2;
      sincos(tp, &s, &co);
      sincos(2 * tp, &s2, &c2);
      const double qr = 1.0 + al * c2, qi = al * s2;
      const double qn = qr * qr + qi * qi;
      r->mx = (co * qr + s * qi) / qn;
      r->my = (s * qr - co * qi) / qn;
      // z'(t) = 2 pi i e^s (1 - alpha e^{2s}) / q^2
      const double q2r = qr * qr - qi * qi, q2i = 2 * qr * qi;
      const double q2n = q2r * q2r + q2i * q2i;
      const double ur = 1.0 - al * c2, ui = -al * s2;
      const double nr = co * ur - s * ui, ni = co * ui + s * ur;
      const double ir = -2 * kPi * ni, ii = 2 * kPi * nr;
      r->dx = (ir * q2r + ii * q2i) / q2n;
      r->dy = (ii * q2r - ir * q2i) / q2n;
      break;
    }
    default:
      r->mx = r->my = r->dx = r->dy = __longlong_as_double(0x7ff8000000000000LL);
  }
}

__device__ __forceinline__ ElemPt elem_eval(int kind, const double* p, double t) {
  ElemPt r;
  if (kind == BEM2D_ELEM_SEGMENT) {
    const double ddx = p[2] - p[0], ddy = p[3] - p[1];
    r.mx = p[0] + ddx * t;
    r.my = p[1] + ddy * t;
    r.dx = ddx;
    r.dy = ddy;
  } else {
    const double t1 = p[0], t2 = p[1];
    curve_eval(kind, p + 2, t1 + t * (t2 - t1), &r);
    r.dx *= (t2 - t1);
    r.dy *= (t2 - t1);
  }
  return r;
}

// Normal(t) = normalize(Deriv.y, -Deriv.x) (lib/bem2d_element.h:29-34).
__device__ __forceinline__ void elem_normal(const ElemPt& p, double* nx, double* ny) {
  const double l = sqrt(p.dy * p.dy + p.dx * p.dx);
  *nx = p.dy / l;
  *ny = -p.dx / l;
}

__device__ __forceinline__ double elem_jac(const ElemPt& p) {
  return sqrt(p.dx * p.dx + p.dy * p.dy);
}

// PolBasis t^d / LinBasis (lib/bem2d_basistypes.h:28-62); all library bases
// used here are real, so conj(phi) = phi.
__device__ __forceinline__ double basis_eval(int kind, double param, double t) {
  if (kind == BEM2D_BASIS_LIN) return param == -1.0 ? 1 - t : t;
  const int deg = (int)param;
  double r = 1;
  for (int i = 0; i < deg; ++i) r *= t;
  return r;
}

// ---- kernels (lib/bem2d_kernel.cpp:15-112), real wavenumber ---------------
// Returns K(x, y) for test point x with normal n1 and trial point y with
// normal n2.  kq = k/4, eq = eta/4.
template <int KERNEL>
__device__ __forceinline__ void kernel_d(double kk, double kq, double eq,
                                         double xx, double xy, double yx,
                                         double yy, double n1x, double n1y,
                                         double n2x, double n2y, double* re,
                                         double* im) {
  const double wx = xx - yx, wy = xy - yy;
  const double d = sqrt(wx * wx + wy * wy);
  double j0, y0, j1, y1;
  hankel01_d(kk * d, &j0, &y0, &j1, &y1);
  if (KERNEL == BEM2D_KERNEL_SINGLE) {
    *re = -0.25 * y0;
    *im = 0.25 * j0;
  } else {
    // DoubleLayer uses w = y - x and the trial normal; the others w = x - y
    // and the test normal.
    const double dot = (KERNEL == BEM2D_KERNEL_DOUBLE) ? -(n2x * wx + n2y * wy)
                                                       : (n1x * wx + n1y * wy);
    const double c = dot / d;
    *re = kq * c * y1;
    *im = -kq * c * j1;
    if (KERNEL == BEM2D_KERNEL_COMBINED) {
      *re = fma(eq, j0, *re);
      *im = fma(eq, y0, *im);
    }
  }
}

// Both orientations of a pair at once: K(x, y) with the normal n1 at x and
// n2 at y (re1, im1), and K(y, x) with the roles swapped (re2, im2).  One
// distance and one Hankel evaluation serve both.
template <int KERNEL>
__device__ __forceinline__ void kernel_d_pair(double kk, double kq, double eq, double xx,
                                              double xy, double yx, double yy, double n1x,
                                              double n1y, double n2x, double n2y, double* re1,
                                              double* im1, double* re2, double* im2) {
  const double wx = xx - yx, wy = xy - yy;
  const double d = sqrt(wx * wx + wy * wy);
  double j0, y0, j1, y1;
  hankel01_d(kk * d, &j0, &y0, &j1, &y1);
  if (KERNEL == BEM2D_KERNEL_SINGLE) {
    *re1 = *re2 = -0.25 * y0;
    *im1 = *im2 = 0.25 * j0;
  } else {
    const double n1w = n1x * wx + n1y * wy, n2w = n2x * wx + n2y * wy;
    // DoubleLayer: n_y . (y - x); the others: n_x . (x - y)
    const double dot1 = (KERNEL == BEM2D_KERNEL_DOUBLE) ? -n2w : n1w;
    const double dot2 = (KERNEL == BEM2D_KERNEL_DOUBLE) ? n1w : -n2w;
    const double c1 = dot1 / d, c2 = dot2 / d;
    *re1 = kq * c1 * y1;
    *im1 = -kq * c1 * j1;
    *re2 = kq * c2 * y1;
    *im2 = -kq * c2 * j1;
    if (KERNEL == BEM2D_KERNEL_COMBINED) {
      *re1 = fma(eq, j0, *re1);
      *im1 = fma(eq, y0, *im1);
      *re2 = fma(eq, j0, *re2);
      *im2 = fma(eq, y0, *im2);
    }
  }
}

// ---- kernels with a complex wavenumber k = kr + i ki ----------------------
// The reference's complex-k branches (lib/bem2d_kernel.cpp:15-112, AMOS
// zbesh through BesselH0/H1(complex)); eta stays real, as there.
//   S = (i/4) H0(k d),  D' = -(i k/4) H1(k d) (n1.(x-y))/d,
//   D = -(i k/4) H1(k d) (n2.(y-x))/d,  combined = D' - i eta S.
// eq = eta/4.
template <int KERNEL>
__device__ __forceinline__ void kernel_c(double kr, double ki, double eq, double xx, double xy,
                                         double yx, double yy, double n1x, double n1y,
                                         double n2x, double n2y, double* re, double* im) {
  const double wx = xx - yx, wy = xy - yy;
  const double d = sqrt(wx * wx + wy * wy);
  cd h0, h1;
  hankel01_c(cd{kr * d, ki * d}, &h0, &h1);
  if (KERNEL == BEM2D_KERNEL_SINGLE) {
    *re = -0.25 * h0.im;
    *im = 0.25 * h0.re;
  } else {
    const double dot = (KERNEL == BEM2D_KERNEL_DOUBLE) ? -(n2x * wx + n2y * wy)
                                                       : (n1x * wx + n1y * wy);
    const double c = 0.25 * dot / d;
    const cd p = cd_mul(cd{kr, ki}, h1);  // k H1
    *re = c * p.im;
    *im = -c * p.re;
    if (KERNEL == BEM2D_KERNEL_COMBINED) {
      *re = fma(eq, h0.re, *re);
      *im = fma(eq, h0.im, *im);
    }
  }
}

// Both orientations of a pair (see kernel_d_pair), complex wavenumber.
template <int KERNEL>
__device__ __forceinline__ void kernel_c_pair(double kr, double ki, double eq, double xx,
                                              double xy, double yx, double yy, double n1x,
                                              double n1y, double n2x, double n2y, double* re1,
                                              double* im1, double* re2, double* im2) {
  const double wx = xx - yx, wy = xy - yy;
  const double d = sqrt(wx * wx + wy * wy);
  cd h0, h1;
  hankel01_c(cd{kr * d, ki * d}, &h0, &h1);
  if (KERNEL == BEM2D_KERNEL_SINGLE) {
    *re1 = *re2 = -0.25 * h0.im;
    *im1 = *im2 = 0.25 * h0.re;
  } else {
    const double n1w = n1x * wx + n1y * wy, n2w = n2x * wx + n2y * wy;
    const double dot1 = (KERNEL == BEM2D_KERNEL_DOUBLE) ? -n2w : n1w;
    const double dot2 = (KERNEL == BEM2D_KERNEL_DOUBLE) ? n1w : -n2w;
    const double c1 = 0.25 * dot1 / d, c2 = 0.25 * dot2 / d;
    const cd p = cd_mul(cd{kr, ki}, h1);
    *re1 = c1 * p.im;
    *im1 = -c1 * p.re;
    *re2 = c2 * p.im;
    *im2 = -c2 * p.re;
    if (KERNEL == BEM2D_KERNEL_COMBINED) {
      *re1 = fma(eq, h0.re, *re1);
      *im1 = fma(eq, h0.im, *im1);
      *re2 = fma(eq, h0.re, *re2);
      *im2 = fma(eq, h0.im, *im2);
    }
  }
}

// ---- near-pair rules -------------------------------------------------------
// RULE_G3_PAIR: the pair (i, j), j the next element of i, integrated with
// AdaptedGauss3 together with its reverse (j, i), whose rule AdaptedGauss2
// is the mirror image of AdaptedGauss3 ((x, y) -> (y, x), same weights).
enum NearRule : int { RULE_SELF = 0, RULE_G2 = 1, RULE_G3 = 2, RULE_G3_PAIR = 3 };

struct NearPair {
  int i;     // test unknown (row)
  int j;     // trial unknown (column)
  int rule;  // NearRule
  int same;  // element indices equal (mass-matrix term applies)
};

// Quadrature rules on the device: Gauss nodes on [0,1] and the three
// adapted rules (lib/bem2d_quadpoints.cpp:75-183), points as (x, y, w).
struct DevRules {
  int ng;                // Gauss points
  const double* gx;      // [ng]
  const double* gw;      // [ng]
  int n1, n2, n3;        // sizes of AdaptedGauss1/2/3
  const double* r1;      // [3*n1] x, y, w
  const double* r2;
  const double* r3;
  // Distinct coordinates of each rule, for the near-field geometry tables:
  // u1 [nu1] the x values of AdaptedGauss1; u2/v2 [nu2]/[nv2] and u3/v3 the
  // x and y values of AdaptedGauss2/3.  k1/k2/k3 [n*]: per point, the index
  // of its x value (low 16 bits) and of its y value (high 16 bits).
  int nu1, nu2, nv2, nu3, nv3;
  const double* u1;
  const double* u2;
  const double* v2;
  const double* u3;
  const double* v3;
  const int* k1;
  const int* k2;
  const int* k3;
};

// ---- launch interfaces (assembly.cu) ------------------------------------
struct NodeTable {
  // Far-field node data per unknown u and Gauss node q (index u*ng + q).
  double* x;
  double* y;
  double* nx;
  double* ny;
  double* w;  // |J(x_q)| * w_q * phi_u(x_q)
};

// Far-field node data for the float-float kernel: node offsets from the
// unknown's element centre, normals and weights as (hi, lo) float pairs,
// the centre in FP64 and the largest offset (radius) per unknown.
struct NodeTableFF {
  float2* ox;
  float2* oy;
  float2* nx;
  float2* ny;
  float2* w;
  double2* c;
  float* rad;
};

// Fills the FP64 table and, when tf != nullptr, the float-float one.
void launch_node_table(const DevGeom& g, const DevRules& r, NodeTable t,
                       const NodeTableFF* tf, cudaStream_t s);

// Entries the float-float far kernel leaves to a second pass (an argument
// k|x-y| <= 4 somewhere on the element pair): (row, column) list with a
// counter.
struct DeferList {
  int2* ij;
  unsigned* count;
  unsigned capacity;
};

// Mixed far field: float-float evaluation, writes complex128 (out) and
// complex64 (out32) copies; deferred entries go to `dl`.  Returns
// BEM2D_ERR_NOMEM if the device reduction table could not be made.
int launch_far_ff(const DevGeom& g, const NodeTable& t, const NodeTableFF& tf, int ng,
                  int kernel, double k, double eta, double alpha, double2* out,
                  long long ld, float2* out32, long long ld32, DeferList dl,
                  cudaStream_t s);
// Float-float evaluation of the deferred entries, small-argument Bessel
// branch included (both outputs).  Returns BEM2D_ERR_NOMEM if the device
// reduction table could not be made.
int launch_deferred(const NodeTableFF& tf, int ng, int kernel, double k, double eta,
                    double alpha, const DeferList& dl, double2* out, long long ld,
                    float2* out32, long long ld32, cudaStream_t s);
void launch_far_fp64(const DevGeom& g, const NodeTable& t, int ng, int kernel,
                     double k, double eta, double alpha, double2* out,
                     long long ld, cudaStream_t s);
// FP64 far field with a complex wavenumber k + i ki (complex-argument Hankel
// functions).
void launch_far_fp64_ck(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                        double ki, double eta, double alpha, double2* out, long long ld,
                        cudaStream_t s);
// Near field (self and adjacent pairs).  out32 == nullptr: FP64 kernel
// evaluation into out.  Otherwise the mixed-precision variant (float-float
// Bessel functions) writes both out and out32.  Returns BEM2D_ERR_NOMEM if
// the device reduction table could not be made.
int launch_near(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                int kernel, double k, double eta, double alpha, double beta, double2* out,
                long long ld, cudaStream_t s, float2* out32 = nullptr, long long ld32 = 0);
// FP64 near field with a complex wavenumber k + i ki.
int launch_near_ck(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                   int kernel, double k, double ki, double eta, double alpha, double beta,
                   double2* out, long long ld, cudaStream_t s);
// Shared-memory bytes per warp of the near-field geometry tables for rules r.
size_t near_table_bytes(const DevRules& r);
void launch_ident(const DevGeom& g, const DevRules& r, const NearPair* pairs,
                  int npairs, double2* out, long long ld, cudaStream_t s);
// ki: imaginary part of the wavenumber (0 for a real k).
void launch_rhs(const DevGeom& g, const NodeTable& t, int ng, int fun, double k,
                double dx, double dy, double eta, double scale, double2* out,
                cudaStream_t s, double ki = 0.0);

// ki: imaginary part of the wavenumber (0 for a real k).
void launch_potential(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                      double eta, const double2* coef, int npts, const double* pts,
                      double2* out, cudaStream_t s, double ki = 0.0);

// ---- context accessors (capi.cu) ------------------------------------------
int ctx_device(const bem2d_ctx* c);
cudaStream_t ctx_stream(const bem2d_ctx* c);
long long* ctx_launches(bem2d_ctx* c);
// Worker contexts (own stream and workspace each) of the batched sweep.
std::vector<bem2d_ctx*>& ctx_workers(bem2d_ctx* c);
// Makes c a sweep worker: a high-priority stream for the factor/solve phase
// of its scattering solves and throughput-sized LU panels.
int ctx_make_sweep_worker(bem2d_ctx* c);
// Phase timers of a sweep: whether `c` times its phases, and adding a
// worker's phase totals (and counts) to `dst`.
bool ctx_timers_on(const bem2d_ctx* c);
void ctx_add_timers(bem2d_ctx* dst, const bem2d_ctx* src);
// Records msg as the context's last error and returns code.
int ctx_fail(bem2d_ctx* c, int code, const char* msg);

// ---- launch interfaces (lu.cu) --------------------------------------------
struct LuWork {
  int* ipiv;             // [n] pivot rows (0-based): row i was swapped with ipiv[i]
  int* info;             // [1] first zero pivot (1-based) or 0
  int* status;           // [1] nonzero: a bounded device wait gave up
  void* scratch;         // panel exchange slots (lu_scratch_bytes)
  size_t scratch_bytes;
  int* perm;             // [n] row permutation of the pivots (filled by lu_factor)
  // workspace of the complex64 tensor-core update (lu_pack_bytes(n)); null:
  // the update runs on the CUDA cores
  void* pack = nullptr;
  size_t pack_bytes = 0;
  void* dinv;            // inverses of the 64 x 64 diagonal blocks of L and U
  // complex64 register-window panel: minimum rows per CTA (0: the default,
  // which spreads a panel over up to 16 CTAs for the shortest column chain;
  // larger values use fewer, fuller CTAs, so that more panels of concurrent
  // factorisations fit on the GPU at once)
  int min_rows = 0;
  // persistent CTAs of the tensor-core update (0: one per SM); fewer leave
  // SMs to concurrent factorisations
  int tc_ctas = 0;
  // products per term of the tensor-core update: 3 (3xTF32) or 1 (1xTF32)
  int tc_passes = 3;
  // look-ahead of the blocked complex64 factorisation (all set, or none):
  // the trailing update of the columns beyond the next block runs on `aux`
  // (packing buffer pack2, aux_ctas persistent CTAs) while the next block's
  // panels run on the main stream; ev_u12 / ev_far order the two
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_u12 = nullptr, ev_far = nullptr;
  void* pack2 = nullptr;
  size_t pack2_bytes = 0;
  int aux_ctas = 0;
};

// Bytes of LuWork::scratch the panel kernels need for n unknowns.
size_t lu_scratch_bytes(int n);
// Bytes of perm + dinv for n unknowns of `elem` bytes each.
size_t lu_aux_bytes(int n, size_t elem);
// Bytes of LuWork::pack for a complex64 factorisation of order n.
size_t lu_pack_bytes(int n);
// Whether a complex64 factorisation of order n uses the look-ahead (and so
// LuWork::aux, ev_u12, ev_far, pack2 of lu_pack_bytes(n) bytes), and the
// persistent CTAs its far updates get (the rest of the SMs stay free for
// the next block's panels).
bool lu_lookahead(int n);
int lu_lookahead_ctas();

// LU with partial pivoting in place; T = double2 (complex128) or float2.
// Also fills w.perm and w.dinv for lu_solve.
template <typename T>
int lu_factor(T* A, long long lda, int n, const LuWork& w, cudaStream_t s,
              long long* launches);
// Bounded-wait check of the grid panel (lu.cu): one complex64 panel whose
// waits never complete; gives up after `polls` polls and sets *w.status.
int lu_panel_timeout_probe(float2* A, long long lda, int n, const LuWork& w, unsigned polls,
                           cudaStream_t s);
// x = A^{-1} b with the factor of lu_factor (b and x may alias).
template <typename T>
int lu_solve(const T* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
             cudaStream_t s, long long* launches);

// x = A^{-1} b with a complex64 factor of lu_factor<float2>, the solves
// arithmetic in complex128 (a fixed operator; b and x may alias).
int lu_solve_mixed(const float2* LU, long long lda, int n, const LuWork& w, const double2* b,
                   double2* x, cudaStream_t s, long long* launches);
// x = A^{-H} b with the factor of lu_factor (b and x must differ).
template <typename T>
int lu_solve_h(const T* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
               cudaStream_t s, long long* launches);

// W = U^{-1} L^{-1} (complex64, n x n, ld ldw) from the factor of
// lu_factor<float2> (needs w.pack for K = 64 and w.dinv): A^{-1} x =
// W (P x), A^{-H} x = P^T (W^H x), P x = x[w.perm[i]].
int lu_inverse_c64(const float2* LU, long long lda, int n, const LuWork& w, float2* W,
                   long long ldw, cudaStream_t s, long long* launches);
// dst[i] = (complex64)(scale src[perm[i]]);  dst[perm[i]] = src[i]
void launch_gather_to_c64(int n, const double2* src, const int* perm, double scale, float2* dst,
                          cudaStream_t s);
void launch_scatter_c64(int n, const float2* src, const int* perm, float2* dst, cudaStream_t s);

// C -= A B for complex64 column-major operands on the tensor cores
// (tcgen05 kind::tf32; lu_tc.cu).  C is M x N, A M x K, B K x N.
// passes = 3: 3xTF32 split (FP32-accurate products); 1: 1xTF32 (operands
// rounded to TF32, a third of the tensor work).
// Sets *status on a device-side wait timeout.
// `pack` (tc_pack_bytes(M, N, K) bytes) holds the split, re-laid-out operands.
size_t tc_pack_bytes(int M, int N, int K);
int launch_tc_cgemm_sub(float2* C, long long ldc, const float2* A, long long lda,
                        const float2* B, long long ldb, int M, int N, int K, void* pack,
                        size_t pack_bytes, int* status, cudaStream_t s, int max_ctas = 0,
                        int passes = 3);

void launch_residual(const double2* A, long long lda, int n, const double2* x,
                     const double2* b, double2* r, double2* part, cudaStream_t s);
size_t residual_part_bytes(int n);
void launch_to_c64(const double2* src, long long lds, float2* dst, long long ldd,
                   int rows, int cols, cudaStream_t s);
void launch_scale_to_c64(int n, const double2* src, double scale, float2* dst,
                         cudaStream_t s);
void launch_axpy_c64(int n, double scale, const float2* d, double2* x, cudaStream_t s);
// *out = sum |a_ij|^2 (part: sumsq_part_bytes() of scratch)
void launch_sumsq(const double2* A, long long ld, int rows, int cols, double* part,
                  double* out, cudaStream_t s);
size_t sumsq_part_bytes();
// *flag |= 1 if the rows x cols column-major block holds a NaN or an
// infinity (the flag is not cleared here)
void launch_nonfinite_scan(const double2* A, long long ld, int rows, int cols, int* flag,
                           cudaStream_t s);

// ---- launch interfaces (spectra.cu) ---------------------------------------
// Work bytes of launch_tridiag_eigs for order N.
size_t spectra_work_bytes(int N);
// M (n x n, ld n) = the Hermitian matrix defined by the upper triangle of A.
void launch_herm_from_upper(const double2* A, long long lda, int n, double2* M, cudaStream_t s);
// M (2n x 2n, ld 2n) = [0 A; A^H 0].
void launch_jordan_wielandt(const double2* A, long long lda, int n, double2* M, cudaStream_t s);
// Householder reduction of the Hermitian M (N x N, ld N, overwritten) to
// tridiagonal form and bisection for `count` of its eigenvalues: ascending
// from the smallest, or (descending != 0) descending from the largest, into
// out (device).  Returns the number of kernels launched.
long long launch_tridiag_eigs(double2* M, int N, int count, int descending, void* work,
                              double* out, int sms, cudaStream_t s);

// ---- launch interfaces (eig.cu) --------------------------------------------
// Work bytes of launch_eigenvalues for order n.
size_t eig_work_bytes(int n);
// Eigenvalues of the general A (n x n, ld n, overwritten by its Hessenberg
// form and the QR iterates) into w (device, n complex128).  Returns the
// number of kernels launched; eig_status_ptr(work, n) then holds 0 or the
// number of eigenvalues not found within the iteration limit.
// Z (n x n, optional): if given, receives the Schur vectors (A on exit holds
// the triangular Schur factor T).
long long launch_eigenvalues(double2* A, int n, void* work, double2* w, int sms, cudaStream_t s,
                             double2* Z = nullptr);
// Right eigenvectors X (n x n) from the Schur factor T and the Schur
// vectors Z (Y: n x n scratch), normalised as zgeev does.
long long launch_eigenvectors(const double2* T, const double2* Z, int n, double2* Y, double2* X,
                              cudaStream_t s);
int* eig_status_ptr(void* work, int n);

}  // namespace bem2d_gpu
