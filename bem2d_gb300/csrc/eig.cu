// Eigenvalues (and right eigenvectors) of a general complex matrix on
// sm_103a: Eigenvalues (lib/bem2d_mathroutines.cpp:437-528, LAPACK zgeev
// with jobvl = 'N', jobvr = 'N' or 'V').
//
// 1. Householder reduction to upper Hessenberg form (the unblocked
//    reduction of Golub & Van Loan, sec. 7.4.3), step j = 0..n-3 with
//    x = A[j+1:n, j], H = I - tau v v^H, H^H x = beta e_1:
//      A[:, j+1:] -= tau (A[:, j+1:] v) v^H            (right, all rows)
//      A[j+1:, j+1:] -= conj(tau) v (v^H A[j+1:, j+1:]) (left)
//    six launches per column: reflector, column-split products with a
//    fixed-order reduction, rank-1 update from the right, one warp per
//    column for v^H A, rank-1 update from the left.
// 2. Implicitly shifted single-shift QR on the Hessenberg matrix (Golub &
//    Van Loan, sec. 7.5), eigenvalues only: deflation where |h(k,k-1)| <=
//    eps (|h(k-1,k-1)| + |h(k,k)|) (1-norms of the complex entries),
//    Wilkinson shift from the trailing 2 x 2 block, an exceptional shift
//    every tenth iteration on a block, 2 x 2 blocks solved in closed form,
//    at most 30 max(10, n) iterations (then BEM2D_ERR_NOCONV).  One CTA of
//    1024 threads runs the whole iteration: thread 0 forms each rotation,
//    all threads apply it to the two rows and the two columns it touches in
//    the active block.  Every loop bound and decision is broadcast through
//    shared memory before the threads use it, so all threads meet every
//    barrier.
// 3. Eigenvectors (jobvr = 'V'): the reduction's reflectors and the QR
//    rotations are accumulated into Z and the QR runs on the whole matrix
//    (the Schur form A = Z T Z^H, T upper triangular), then back
//    substitution on T (ztrevc's scheme, one CTA per vector), X = Z Y on the
//    FP64 pipe, and zgeev's normalisation (unit norm, largest entry real).
// No balancing (zgebal) is applied; the boundary-element matrices this
// library produces are well scaled.
#include <float.h>

#include <algorithm>

#include "common.cuh"
#include "cplx.cuh"
#include "dense.cuh"

namespace bem2d_gpu {

namespace {

constexpr int kHessThreads = 256;
constexpr int kGvRows = 128;
constexpr int kGvSplit = 32;
constexpr int kQrThreads = 1024;

__device__ __forceinline__ double2 cconjd(double2 a) { return make_double2(a.x, -a.y); }

__device__ __forceinline__ double cabs1d(double2 a) { return fabs(a.x) + fabs(a.y); }

// Principal square root.
__device__ __forceinline__ double2 csqrtd(double2 w) {
  const double m = hypot(w.x, w.y);
  if (m == 0.0) return make_double2(0.0, 0.0);
  if (w.x >= 0) {
    const double s = sqrt(0.5 * (m + w.x));
    return make_double2(s, w.y / (2 * s));
  }
  const double t = sqrt(0.5 * (m - w.x));
  return make_double2(fabs(w.y) / (2 * t), w.y >= 0 ? t : -t);
}

// Reflector for x = A[j+1:n, j] (m = n - j - 1 >= 2): v (v[0] = 1), S[0] =
// tau; column j becomes (beta, 0, ..., 0) below the diagonal.
__global__ void __launch_bounds__(kHessThreads)
hess_house_kernel(double2* __restrict__ A, long long ld, int n, int j, double2* __restrict__ v,
                  double2* __restrict__ S) {
  __shared__ double red[kHessThreads / 32];
  __shared__ double2 sh_scale;
  __shared__ double sh_beta;
  const int m = n - j - 1;
  double2* x = A + (size_t)j * ld + (j + 1);
  double s = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += kHessThreads) {
    const double2 xi = x[i];
    s = fma(xi.x, xi.x, fma(xi.y, xi.y, s));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double xn2 = 0.0;
    for (int w = 0; w < kHessThreads / 32; ++w) xn2 += red[w];
    const double2 a = x[0];
    double2 tau, scale;
    double beta;
    if (xn2 == 0.0 && a.y == 0.0) {
      tau = make_double2(0.0, 0.0);
      scale = make_double2(0.0, 0.0);
      beta = a.x;
    } else {
      beta = -copysign(sqrt(fma(a.x, a.x, fma(a.y, a.y, xn2))), a.x);
      tau = make_double2((beta - a.x) / beta, -a.y / beta);
      const double2 am = make_double2(a.x - beta, a.y);
      const double q = fma(am.x, am.x, am.y * am.y);
      scale = make_double2(am.x / q, -am.y / q);
    }
    S[0] = tau;
    sh_scale = scale;
    sh_beta = beta;
  }
  __syncthreads();
  const double2 sc = sh_scale;
  for (int i = threadIdx.x; i < m; i += kHessThreads)
    v[i] = i == 0 ? make_double2(1.0, 0.0) : cmul(x[i], sc);
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += kHessThreads)
    x[i] = i == 0 ? make_double2(sh_beta, 0.0) : make_double2(0.0, 0.0);
}

// P[s * rows + r] = sum_{c in chunk s} B[r + c ld] v[c]   (B: rows x cols)
__global__ void __launch_bounds__(kGvRows)
gemv_part_kernel(const double2* __restrict__ B, long long ld, int rows, int cols,
                 const double2* __restrict__ v, int chunk, double2* __restrict__ P) {
  __shared__ double2 sv[kGvRows];
  const int r = blockIdx.x * kGvRows + threadIdx.x;
  const int c0 = blockIdx.y * chunk, c1 = min(cols, c0 + chunk);
  double2 acc = make_double2(0.0, 0.0);
  for (int cb = c0; cb < c1; cb += kGvRows) {
    const int cn = min(kGvRows, c1 - cb);
    __syncthreads();
    if (threadIdx.x < cn) sv[threadIdx.x] = v[cb + threadIdx.x];
    __syncthreads();
    if (r < rows) {
      const double2* col = B + (size_t)cb * ld + r;
      for (int t = 0; t < cn; ++t) acc = cfma(col[(size_t)t * ld], sv[t], acc);
    }
  }
  if (r < rows) P[(size_t)blockIdx.y * rows + r] = acc;
}

// u[r] = tau * sum_s P[s * rows + r]
__global__ void reduce_u_kernel(int rows, int ns, const double2* __restrict__ P,
                                const double2* __restrict__ S, double2* __restrict__ u) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int s = 0; s < ns; ++s) {
    const double2 t = P[(size_t)s * rows + r];
    acc.x += t.x;
    acc.y += t.y;
  }
  u[r] = cmul(S[0], acc);
}

// B[r + c ld] -= u[r] conj(v[c])   (B: rows x cols; 32 x 8 threads, 32 x 32 tile)
__global__ void __launch_bounds__(256)
rank1_right_kernel(double2* __restrict__ B, long long ld, int rows, int cols,
                   const double2* __restrict__ u, const double2* __restrict__ v) {
  const int r = blockIdx.x * 32 + threadIdx.x;
  if (r >= rows) return;
  const double2 ur = u[r];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = blockIdx.y * 32 + threadIdx.y + 8 * k;
    if (c >= cols) break;
    const double2 vc = cconjd(v[c]);
    double2* p = B + (size_t)c * ld + r;
    *p = cfms(*p, ur, vc);
  }
}

// w[c] = sum_r conj(v[r]) B[r + c ld]   (B: m x m; one warp per column)
__global__ void __launch_bounds__(256)
gemv_left_kernel(const double2* __restrict__ B, long long ld, int m,
                 const double2* __restrict__ v, double2* __restrict__ w) {
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= m) return;
  const double2* col = B + (size_t)c * ld;
  double2 acc = make_double2(0.0, 0.0);
  for (int r = lane; r < m; r += 32) acc = cfma(cconjd(v[r]), col[r], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  if (lane == 0) w[c] = acc;
}

// B[r + c ld] -= conj(tau) v[r] w[c]   (B: m x m)
__global__ void __launch_bounds__(256)
rank1_left_kernel(double2* __restrict__ B, long long ld, int m, const double2* __restrict__ v,
                  const double2* __restrict__ w, const double2* __restrict__ S) {
  const int r = blockIdx.x * 32 + threadIdx.x;
  if (r >= m) return;
  const double2 tv = cmul(cconjd(S[0]), v[r]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = blockIdx.y * 32 + threadIdx.y + 8 * k;
    if (c >= m) break;
    double2* p = B + (size_t)c * ld + r;
    *p = cfms(*p, tv, w[c]);
  }
}

// Eigenvalues of the 2 x 2 block [a b; c d]: (a + d)/2 +- sqrt(((a - d)/2)^2 + bc).
__device__ void eig2(double2 a, double2 b, double2 c, double2 d, double2* l1, double2* l2) {
  const double2 t = make_double2(0.5 * (a.x - d.x), 0.5 * (a.y - d.y));
  const double2 disc = csqrtd(cfma(t, t, cmul(b, c)));
  const double2 h = make_double2(0.5 * (a.x + d.x), 0.5 * (a.y + d.y));
  *l1 = make_double2(h.x + disc.x, h.y + disc.y);
  *l2 = make_double2(h.x - disc.x, h.y - disc.y);
}

// Shifted QR on the upper Hessenberg H (n x n, ld); eigenvalues into w as
// they deflate (bottom up).  status[0] = 0, or the number of eigenvalues
// not found when the iteration limit was reached.
// VEC: the Schur form as well (zlahqr with wantt = wantz = true): every
// rotation is applied to the whole rows (columns to n - 1) and the whole
// columns (rows from 0) of H and to the columns of Z (n x n, ld, the
// accumulated Hessenberg reduction on entry), and a deflated 2 x 2 block is
// made upper triangular by one more rotation, so that on exit H holds the
// upper triangular T with A = Z T Z^H and w[i] = T(i, i).
template <bool VEC>
__global__ void __launch_bounds__(kQrThreads)
hess_qr_kernel(double2* __restrict__ H, long long ld, int n, double2* __restrict__ w,
               int* __restrict__ status, double2* __restrict__ Z) {
  __shared__ int s_lo, s_hi, s_mode, s_defl;
  __shared__ double s_c;
  __shared__ double2 s_s, s_g0, s_g1;
  const int tid = threadIdx.x;
  auto at = [&](int i, int j) -> double2& { return H[(size_t)j * ld + i]; };
  int its = 0, total = 0;
  const int itmax = 30 * max(10, n);
  if (tid == 0) {
    s_hi = n - 1;
    status[0] = 0;
  }
  __syncthreads();
  for (;;) {
    const int hi = s_hi;  // read by all after the previous barrier
    if (hi < 0) break;
    // deflation search: the largest k in [1, hi] with a negligible h(k, k-1)
    if (tid == 0) s_defl = 0;
    __syncthreads();
    for (int k = hi - tid; k >= 1; k -= kQrThreads) {
      const double sub = cabs1d(at(k, k - 1));
      if (sub <= DBL_EPSILON * (cabs1d(at(k - 1, k - 1)) + cabs1d(at(k, k))) ||
          sub < DBL_MIN) {
        atomicMax(&s_defl, k);
        break;  // smaller k of this thread cannot beat it
      }
    }
    __syncthreads();
    if (tid == 0) {
      const int lo = s_defl;
      if (lo > 0) at(lo, lo - 1) = make_double2(0.0, 0.0);
      s_lo = lo;
      if (lo == hi) {
        w[hi] = at(hi, hi);
        s_hi = hi - 1;
        s_mode = 0;
        its = 0;
      } else if (lo == hi - 1) {
        double2 l1, l2;
        eig2(at(hi - 1, hi - 1), at(hi - 1, hi), at(hi, hi - 1), at(hi, hi), &l1, &l2);
        if (VEC) {
          // rotation whose first column is the unit eigenvector of the block
          // for l1: (b, l1 - a) or (l1 - d, c), the better scaled one
          const double2 a = at(hi - 1, hi - 1), b = at(hi - 1, hi), cc = at(hi, hi - 1),
                        d = at(hi, hi);
          double2 x = b, y = make_double2(l1.x - a.x, l1.y - a.y);
          const double2 x2 = make_double2(l1.x - d.x, l1.y - d.y), y2 = cc;
          if (cabs1d(x2) + cabs1d(y2) > cabs1d(x) + cabs1d(y)) {
            x = x2;
            y = y2;
          }
          const double r = hypot(hypot(x.x, x.y), hypot(y.x, y.y));
          // G = [x -conj(y); y conj(x)] / r: G^H [a b; c d] G is upper triangular
          s_g0 = r > 0 ? make_double2(x.x / r, x.y / r) : make_double2(1.0, 0.0);
          s_g1 = r > 0 ? make_double2(y.x / r, y.y / r) : make_double2(0.0, 0.0);
          s_mode = 2;
        } else {
          w[hi - 1] = l1;
          w[hi] = l2;
          s_hi = hi - 2;
          s_mode = 0;
        }
        its = 0;
      } else if (++total > itmax) {
        status[0] = hi + 1;
        s_hi = -1;
        s_mode = 0;
      } else {
        ++its;
        double2 mu;
        const double2 d = at(hi, hi);
        if (its % 10 == 0) {  // exceptional shift
          mu = make_double2(d.x + 0.75 * fabs(at(hi, hi - 1).x), d.y);
        } else {  // Wilkinson: the eigenvalue of the trailing 2 x 2 block nearer d
          const double2 a = at(hi - 1, hi - 1), b = at(hi - 1, hi), c = at(hi, hi - 1);
          const double2 t = make_double2(0.5 * (a.x - d.x), 0.5 * (a.y - d.y));
          const double2 bc = cmul(b, c);
          const double2 disc = csqrtd(cfma(t, t, bc));
          const double2 p = make_double2(t.x + disc.x, t.y + disc.y);
          const double2 q = make_double2(t.x - disc.x, t.y - disc.y);
          const double2 den = cabs1d(p) >= cabs1d(q) ? p : q;
          mu = (den.x == 0.0 && den.y == 0.0) ? d : cfms(d, bc, crcp(den));
        }
        // the first rotation's vector (h(lo,lo) - mu, h(lo+1,lo)) is formed
        // in the sweep below from s_c / s_s
        s_s = mu;
        s_mode = 1;
      }
    }
    __syncthreads();
    if (s_mode == 0) continue;  // uniform: every thread read the same flag
    if (VEC && s_mode == 2) {
      // triangularise the deflated 2 x 2 block at rows / columns hi-1, hi
      // with G = [g0 -conj(g1); g1 conj(g0)]: rows (all columns from hi-1)
      // by G^H, columns (rows 0..hi) and Z's columns by G
      const double2 g0 = s_g0, g1 = s_g1;
      const int p = hi - 1;
      for (int jc = p + tid; jc < n; jc += kQrThreads) {
        const double2 h1 = at(p, jc), h2 = at(hi, jc);
        at(p, jc) = cfma(cconjd(g1), h2, cmul(cconjd(g0), h1));
        at(hi, jc) = cfms(cmul(g0, h2), g1, h1);
      }
      __syncthreads();
      for (int i = tid; i <= hi; i += kQrThreads) {
        const double2 h1 = at(i, p), h2 = at(i, hi);
        at(i, p) = cfma(h2, g1, cmul(h1, g0));
        at(i, hi) = cfms(cmul(h2, cconjd(g0)), h1, cconjd(g1));
      }
      for (int i = tid; i < n; i += kQrThreads) {
        double2* z1 = Z + (size_t)p * ld + i;
        double2* z2 = Z + (size_t)hi * ld + i;
        const double2 a1 = *z1, a2 = *z2;
        *z1 = cfma(a2, g1, cmul(a1, g0));
        *z2 = cfms(cmul(a2, cconjd(g0)), a1, cconjd(g1));
      }
      __syncthreads();
      if (tid == 0) {
        at(hi, p) = make_double2(0.0, 0.0);
        w[p] = at(p, p);
        w[hi] = at(hi, hi);
        s_hi = hi - 2;
      }
      __syncthreads();
      continue;
    }
    const int lo = s_lo;
    const double2 mu = s_s;
    __syncthreads();  // all threads have read mu before s_s is reused
    for (int k = lo; k < hi; ++k) {
      if (tid == 0) {
        double2 x, y;
        if (k == lo) {
          const double2 h = at(lo, lo);
          x = make_double2(h.x - mu.x, h.y - mu.y);
          y = at(lo + 1, lo);
        } else {
          x = at(k, k - 1);
          y = at(k + 1, k - 1);
        }
        const double ax = hypot(x.x, x.y), ay = hypot(y.x, y.y);
        const double r = hypot(ax, ay);
        double c;
        double2 s;
        if (r == 0.0) {
          c = 1.0;
          s = make_double2(0.0, 0.0);
        } else if (ax == 0.0) {
          c = 0.0;
          s = make_double2(y.x / ay, -y.y / ay);  // conj(y) / |y|
        } else {
          c = ax / r;
          // s = (x / |x|) conj(y) / r
          const double2 ux = make_double2(x.x / ax, x.y / ax);
          const double2 cy = make_double2(y.x / r, -y.y / r);
          s = cmul(ux, cy);
        }
        s_c = c;
        s_s = s;
      }
      __syncthreads();
      const double c = s_c;
      const double2 s = s_s;
      const double2 sc = cconjd(s);
      // rows k, k+1, columns max(lo, k-1)..hi (..n-1 with VEC):
      // (h1, h2) <- (c h1 + s h2, -conj(s) h1 + c h2)
      const int jend = VEC ? n - 1 : hi;
      for (int jc = max(lo, k - 1) + tid; jc <= jend; jc += kQrThreads) {
        const double2 h1 = at(k, jc), h2 = at(k + 1, jc);
        const double2 n1 = cfma(s, h2, make_double2(c * h1.x, c * h1.y));
        const double2 n2 = cfms(make_double2(c * h2.x, c * h2.y), sc, h1);
        at(k, jc) = n1;
        at(k + 1, jc) = n2;
      }
      __syncthreads();
      if (tid == 0 && k > lo) at(k + 1, k - 1) = make_double2(0.0, 0.0);
      // columns k, k+1, rows lo..min(k+2, hi) (from 0 with VEC):
      // (h1, h2) <- (c h1 + conj(s) h2, -s h1 + c h2)
      const int i1 = min(k + 2, hi);
      for (int i = (VEC ? 0 : lo) + tid; i <= i1; i += kQrThreads) {
        const double2 h1 = at(i, k), h2 = at(i, k + 1);
        const double2 n1 = cfma(sc, h2, make_double2(c * h1.x, c * h1.y));
        const double2 n2 = cfms(make_double2(c * h2.x, c * h2.y), s, h1);
        at(i, k) = n1;
        at(i, k + 1) = n2;
      }
      if (VEC) {  // the Schur vectors: columns k, k+1 of Z, the same rotation
        for (int i = tid; i < n; i += kQrThreads) {
          double2* z1 = Z + (size_t)k * ld + i;
          double2* z2 = Z + (size_t)(k + 1) * ld + i;
          const double2 h1 = *z1, h2 = *z2;
          *z1 = cfma(sc, h2, make_double2(c * h1.x, c * h1.y));
          *z2 = cfms(make_double2(c * h2.x, c * h2.y), s, h1);
        }
      }
      __syncthreads();
    }
  }
}

// Eigenvectors of the upper triangular T (n x n, ld): column j of Y (ld)
// solves (T - T(j,j) I) y = 0 with y_j = 1, y_i = 0 below (ztrevc's back
// substitution, column oriented: after y_k is known, r[0..k-1] -= T[0..k-1, k]
// y_k; divisors below smin = max(eps |T(j,j)|, DBL_MIN) are raised to smin).
// One CTA per eigenvector; r lives in Y's column.
__global__ void __launch_bounds__(256)
trevc_kernel(const double2* __restrict__ T, long long ld, int n, double2* __restrict__ Y) {
  const int j = blockIdx.x;
  double2* y = Y + (size_t)j * ld;
  const double2 lam = T[(size_t)j * ld + j];
  const double smin = fmax(DBL_EPSILON * cabs1d(lam), DBL_MIN);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (i < j) {
      const double2 t = T[(size_t)j * ld + i];
      y[i] = make_double2(-t.x, -t.y);  // r = -T[0..j-1, j]
    } else {
      y[i] = i == j ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
    }
  }
  __shared__ double2 s_yk;
  __syncthreads();
  for (int k = j - 1; k >= 0; --k) {
    if (threadIdx.x == 0) {
      double2 d = T[(size_t)k * ld + k];
      d = make_double2(d.x - lam.x, d.y - lam.y);
      if (cabs1d(d) < smin) d = make_double2(smin, 0.0);
      const double2 yk = cmul(y[k], crcp(d));
      y[k] = yk;
      s_yk = yk;
    }
    __syncthreads();
    const double2 yk = s_yk;
    const double2* tk = T + (size_t)k * ld;
    for (int i = threadIdx.x; i < k; i += blockDim.x) y[i] = cfms(y[i], tk[i], yk);
    __syncthreads();
  }
}

// zgeev's normalisation of each column of X (n x n, ld): unit 2-norm, then
// the entry of largest |re|^2 + |im|^2 (the first such) made real and
// positive.  One CTA per column.
__global__ void __launch_bounds__(256)
normalize_vectors_kernel(double2* __restrict__ X, long long ld, int n) {
  __shared__ double s_v[256];
  __shared__ int s_i[256];
  double2* x = X + (size_t)blockIdx.x * ld;
  double ss = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) ss = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, ss));
  s_v[threadIdx.x] = ss;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s_v[threadIdx.x] += s_v[threadIdx.x + o];
    __syncthreads();
  }
  const double inv = s_v[0] > 0 ? 1.0 / sqrt(s_v[0]) : 1.0;
  __syncthreads();
  double best = -1.0;
  int bi = n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = make_double2(x[i].x * inv, x[i].y * inv);
    x[i] = v;
    const double m = v.x * v.x + v.y * v.y;
    if (m > best) {
      best = m;
      bi = i;
    }
  }
  s_v[threadIdx.x] = best;
  s_i[threadIdx.x] = bi;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const double v2 = s_v[threadIdx.x + o];
      const int i2 = s_i[threadIdx.x + o];
      if (v2 > s_v[threadIdx.x] || (v2 == s_v[threadIdx.x] && i2 < s_i[threadIdx.x])) {
        s_v[threadIdx.x] = v2;
        s_i[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  const int k = s_i[0];
  if (k >= n || !(s_v[0] > 0)) return;
  const double2 vk = x[k];
  const double a = sqrt(s_v[0]);
  const double2 f = make_double2(vk.x / a, -vk.y / a);  // conj(v_k) / |v_k|
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    x[i] = i == k ? make_double2(a, 0.0) : cmul(x[i], f);
}

// Z = I (n x n, ld)
__global__ void identity_kernel(double2* __restrict__ Z, long long ld, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i < n) Z[(size_t)j * ld + i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
}

}  // namespace

size_t eig_work_bytes(int n) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  // v, u, w (n complex each) | P (kGvSplit * n complex) | S (4 complex) | status
  return 3 * up(sizeof(double2) * n) + up(sizeof(double2) * (size_t)kGvSplit * n) +
         up(sizeof(double2) * 4) + up(sizeof(int) * 4);
}

long long launch_eigenvalues(double2* A, int n, void* work, double2* w, int sms,
                             cudaStream_t s, double2* Z) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* p = static_cast<char*>(work);
  double2* v = reinterpret_cast<double2*>(p);
  p += up(sizeof(double2) * n);
  double2* u = reinterpret_cast<double2*>(p);
  p += up(sizeof(double2) * n);
  double2* wl = reinterpret_cast<double2*>(p);
  p += up(sizeof(double2) * n);
  double2* P = reinterpret_cast<double2*>(p);
  p += up(sizeof(double2) * (size_t)kGvSplit * n);
  double2* S = reinterpret_cast<double2*>(p);
  p += up(sizeof(double2) * 4);
  int* status = reinterpret_cast<int*>(p);
  const long long ld = n;
  long long launches = 0;
  if (Z) {
    identity_kernel<<<dim3((n + 255) / 256, n), 256, 0, s>>>(Z, ld, n);
    ++launches;
  }
  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;
    double2* Bt = A + (size_t)(j + 1) * ld;  // columns j+1.., all rows
    hess_house_kernel<<<1, kHessThreads, 0, s>>>(A, ld, n, j, v, S);
    // right: u = tau A[:, j+1:] v (all n rows), A[:, j+1:] -= u v^H
    const int nb = (n + kGvRows - 1) / kGvRows;
    int ns = std::min(kGvSplit, std::max(1, (4 * sms + nb - 1) / nb));
    const int chunk = (m + ns - 1) / ns;
    ns = (m + chunk - 1) / chunk;
    gemv_part_kernel<<<dim3(nb, ns), kGvRows, 0, s>>>(Bt, ld, n, m, v, chunk, P);
    reduce_u_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, ns, P, S, u);
    rank1_right_kernel<<<dim3((n + 31) / 32, (m + 31) / 32), dim3(32, 8), 0, s>>>(Bt, ld, n, m,
                                                                                   u, v);
    // left: w = v^H A[j+1:, j+1:], A[j+1:, j+1:] -= conj(tau) v w
    double2* Bl = Bt + (j + 1);
    gemv_left_kernel<<<(m + 7) / 8, 256, 0, s>>>(Bl, ld, m, v, wl);
    rank1_left_kernel<<<dim3((m + 31) / 32, (m + 31) / 32), dim3(32, 8), 0, s>>>(Bl, ld, m, v,
                                                                                 wl, S);
    launches += 6;
    if (Z) {  // Z <- Z H_j: the same right update on Z's columns j+1..
      double2* Zt = Z + (size_t)(j + 1) * ld;
      gemv_part_kernel<<<dim3(nb, ns), kGvRows, 0, s>>>(Zt, ld, n, m, v, chunk, P);
      reduce_u_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, ns, P, S, u);
      rank1_right_kernel<<<dim3((n + 31) / 32, (m + 31) / 32), dim3(32, 8), 0, s>>>(Zt, ld, n, m,
                                                                                     u, v);
      launches += 3;
    }
  }
  if (Z)
    hess_qr_kernel<true><<<1, kQrThreads, 0, s>>>(A, ld, n, w, status, Z);
  else
    hess_qr_kernel<false><<<1, kQrThreads, 0, s>>>(A, ld, n, w, status, nullptr);
  return launches + 1;
}

long long launch_eigenvectors(const double2* T, const double2* Z, int n, double2* Y, double2* X,
                              cudaStream_t s) {
  trevc_kernel<<<n, 256, 0, s>>>(T, n, n, Y);
  launch_zgemm_rect(Z, n, n, n, Y, n, n, X, n, s);
  normalize_vectors_kernel<<<n, 256, 0, s>>>(X, n, n);
  return 3;
}

int* eig_status_ptr(void* work, int n) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return reinterpret_cast<int*>(static_cast<char*>(work) + 3 * up(sizeof(double2) * n) +
                                up(sizeof(double2) * (size_t)kGvSplit * n) +
                                up(sizeof(double2) * 4));
}

}  // namespace bem2d_gpu
