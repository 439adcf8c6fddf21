// Dense Hermitian eigenvalues and singular values on sm_103a.
//
// Both are computed from a Householder reduction of a Hermitian matrix to
// real symmetric tridiagonal form followed by Sturm-sequence bisection, one
// thread per wanted eigenvalue:
//  - HermitianEigenvalues (lib/bem2d_mathroutines.cpp:353-433, LAPACK zheev
//    with jobz 'N', uplo 'U'): the matrix the upper triangle defines;
//  - SingularValues (lib/bem2d_mathroutines.cpp:268-320, zgesvd without
//    vectors): the n largest eigenvalues of the Jordan-Wielandt matrix
//    [0 A; A^H 0], whose eigenvalues are +-sigma_i (absolute accuracy
//    eps ||A||, as for the bidiagonal route).
//
// Reduction (the unblocked Householder tridiagonalisation of Golub & Van
// Loan, sec. 8.3.1, on full Hermitian storage), step j, trailing size
// m = n - j - 1, x = M[j+1:n, j]:
//   reflector H = I - tau v v^H with H^H x = beta e_1 (beta real),
//   p = tau M_t v,  w = p - (tau/2)(p^H v) v,  M_t -= v w^H + w v^H,
// four launches per step: house_kernel (one CTA: norm, tau, v),
// hemv_part_kernel (column-split products, coalesced over rows),
// reduce_p_kernel (fixed-order sum of the parts and of p^H v per block) and
// her2_kernel (rank-2 update; every block forms the same p^H v sum).  All
// sums run in a fixed order, so results are deterministic.
#include <float.h>

#include <algorithm>

#include "common.cuh"
#include "cplx.cuh"

namespace bem2d_gpu {

namespace {

constexpr int kHouseThreads = 256;
constexpr int kMvRows = 128;
constexpr int kRedThreads = 256;
constexpr int kMaxSplit = 32;

__global__ void __launch_bounds__(kHouseThreads)
house_kernel(const double2* __restrict__ M, long long ld, int n, int j, double2* __restrict__ v,
             double2* __restrict__ S, double* __restrict__ d, double* __restrict__ e) {
  __shared__ double red[kHouseThreads / 32];
  __shared__ double2 sh_scale;
  const int m = n - j - 1;
  const double2* x = M + (size_t)j * ld + (j + 1);
  double s = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += kHouseThreads) {
    const double2 xi = x[i];
    s = fma(xi.x, xi.x, fma(xi.y, xi.y, s));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double xn2 = 0.0;
    for (int w = 0; w < kHouseThreads / 32; ++w) xn2 += red[w];
    const double2 a = x[0];
    double2 tau, scale;
    double beta;
    if (xn2 == 0.0 && a.y == 0.0) {  // already real and reduced: H = I
      tau = make_double2(0.0, 0.0);
      scale = make_double2(0.0, 0.0);
      beta = a.x;
    } else {
      beta = -copysign(sqrt(fma(a.x, a.x, fma(a.y, a.y, xn2))), a.x);
      tau = make_double2((beta - a.x) / beta, -a.y / beta);
      const double2 am = make_double2(a.x - beta, a.y);  // |am| >= |beta| > 0
      const double q = fma(am.x, am.x, am.y * am.y);
      scale = make_double2(am.x / q, -am.y / q);          // 1 / (a - beta)
    }
    S[0] = tau;
    sh_scale = scale;
    d[j] = M[(size_t)j * ld + j].x;
    e[j] = beta;
  }
  __syncthreads();
  const double2 sc = sh_scale;
  for (int i = threadIdx.x; i < m; i += kHouseThreads)
    v[i] = i == 0 ? make_double2(1.0, 0.0) : cmul(x[i], sc);
}

// P[s * n + r] = sum_{c in chunk s} M_t[r, c] v[c], M_t = M[j+1:n, j+1:n].
__global__ void __launch_bounds__(kMvRows)
hemv_part_kernel(const double2* __restrict__ M, long long ld, int n, int j,
                 const double2* __restrict__ v, int chunk, double2* __restrict__ P) {
  __shared__ double2 sv[kMvRows];
  const int m = n - j - 1;
  const int r = blockIdx.x * kMvRows + threadIdx.x;
  const int c0 = blockIdx.y * chunk, c1 = min(m, c0 + chunk);
  const double2* Mt = M + (size_t)(j + 1) * ld + (j + 1);
  double2 acc = make_double2(0.0, 0.0);
  for (int cb = c0; cb < c1; cb += kMvRows) {
    const int cn = min(kMvRows, c1 - cb);
    __syncthreads();
    if (threadIdx.x < cn) sv[threadIdx.x] = v[cb + threadIdx.x];
    __syncthreads();
    if (r < m) {
      const double2* col = Mt + (size_t)cb * ld + r;
      for (int t = 0; t < cn; ++t) acc = cfma(col[(size_t)t * ld], sv[t], acc);
    }
  }
  if (r < m) P[(size_t)blockIdx.y * n + r] = acc;
}

// p = tau * sum_s P[s], Q[block] = sum over the block's rows of conj(p_i) v_i.
__global__ void __launch_bounds__(kRedThreads)
reduce_p_kernel(int n, int j, int ns, const double2* __restrict__ P,
                const double2* __restrict__ S, const double2* __restrict__ v,
                double2* __restrict__ p, double2* __restrict__ Q) {
  __shared__ double2 red[kRedThreads / 32];
  const int m = n - j - 1;
  const int i = blockIdx.x * kRedThreads + threadIdx.x;
  double dr = 0.0, di = 0.0;
  if (i < m) {
    double2 acc = make_double2(0.0, 0.0);
    for (int s = 0; s < ns; ++s) {
      const double2 t = P[(size_t)s * n + i];
      acc.x += t.x;
      acc.y += t.y;
    }
    const double2 pi = cmul(S[0], acc);
    p[i] = pi;
    const double2 vi = v[i];
    dr = fma(pi.x, vi.x, pi.y * vi.y);
    di = fma(pi.x, vi.y, -pi.y * vi.x);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dr += __shfl_xor_sync(0xffffffffu, dr, o);
    di += __shfl_xor_sync(0xffffffffu, di, o);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(dr, di);
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < kRedThreads / 32; ++w) {
      s.x += red[w].x;
      s.y += red[w].y;
    }
    Q[blockIdx.x] = s;
  }
}

// M_t -= v w^H + w v^H with w = p + a2 v, a2 = -(tau/2) sum_b Q[b].
// Block 32 x 8 threads covers 32 rows x 32 columns (4 columns per thread).
__global__ void __launch_bounds__(256)
her2_kernel(double2* __restrict__ M, long long ld, int n, int j, const double2* __restrict__ v,
            const double2* __restrict__ p, const double2* __restrict__ S,
            const double2* __restrict__ Q, int nq) {
  __shared__ double2 a2s;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = 0; b < nq; ++b) {
      s.x += Q[b].x;
      s.y += Q[b].y;
    }
    const double2 ts = cmul(S[0], s);
    a2s = make_double2(-0.5 * ts.x, -0.5 * ts.y);
  }
  __syncthreads();
  const double2 a2 = a2s;
  const int m = n - j - 1;
  const int r = blockIdx.x * 32 + threadIdx.x;
  if (r >= m) return;
  const double2 vr = v[r], wr = cfma(a2, vr, p[r]);
  double2* Mt = M + (size_t)(j + 1) * ld + (j + 1);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int col = blockIdx.y * 32 + threadIdx.y + 8 * k;
    if (col >= m) break;
    const double2 vc = v[col], wc = cfma(a2, vc, p[col]);
    double2 y = Mt[(size_t)col * ld + r];
    // y -= vr conj(wc) + wr conj(vc)
    y.x -= fma(vr.x, wc.x, vr.y * wc.y) + fma(wr.x, vc.x, wr.y * vc.y);
    y.y -= fma(vr.y, wc.x, -vr.x * wc.y) + fma(wr.y, vc.x, -wr.x * vc.y);
    Mt[(size_t)col * ld + r] = y;
  }
}

__global__ void last_diag_kernel(const double2* __restrict__ M, long long ld, int n,
                                 double* __restrict__ d) {
  d[n - 1] = M[(size_t)(n - 1) * ld + (n - 1)].x;
}

// out[i] = eigenvalue number k of the symmetric tridiagonal (d, e), counted
// from the smallest (k = i) or from the largest (k = n - 1 - i), by
// bisection on the Sturm count (the number of negative pivots of
// T - x I = L D L^T), pivots kept away from zero as in LAPACK dstebz.
__global__ void __launch_bounds__(128)
bisect_kernel(const double* __restrict__ d, const double* __restrict__ e, int n, int count,
              int descending, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int k = descending ? n - 1 - i : i;
  double lo = d[0], hi = d[0], emax2 = 0.0;
  for (int t = 0; t < n; ++t) {
    const double el = t > 0 ? fabs(e[t - 1]) : 0.0, er = t < n - 1 ? fabs(e[t]) : 0.0;
    lo = fmin(lo, d[t] - el - er);
    hi = fmax(hi, d[t] + el + er);
    if (t < n - 1) emax2 = fmax(emax2, e[t] * e[t]);
  }
  const double pivmin = DBL_MIN * fmax(1.0, emax2);
  const double nrm = fmax(fabs(lo), fabs(hi));
  const double pad = 2.0 * DBL_EPSILON * nrm * n + 2.0 * pivmin;
  lo -= pad;
  hi += pad;
  const double abstol = 0.01 * DBL_EPSILON * nrm;
  for (int it = 0; it < 256; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (!(mid > lo && mid < hi)) break;
    if (hi - lo <= fmax(2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)), abstol)) break;
    int cnt = 0;
    double q = d[0] - mid;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += q < 0.0;
    for (int t = 1; t < n; ++t) {
      q = d[t] - mid - e[t - 1] * e[t - 1] / q;
      if (fabs(q) < pivmin) q = -pivmin;
      cnt += q < 0.0;
    }
    if (cnt > k)
      hi = mid;
    else
      lo = mid;
  }
  out[i] = 0.5 * (lo + hi);
}

// M (n x n, ld n) = the Hermitian matrix the upper triangle of A defines
// (real diagonal), as zheev with uplo 'U' reads it.
__global__ void herm_from_upper_kernel(const double2* __restrict__ A, long long lda, int n,
                                       double2* __restrict__ M) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int jc = blockIdx.y * 8 + threadIdx.y;
  if (i >= n || jc >= n) return;
  double2 a;
  if (i < jc) {
    a = A[(size_t)jc * lda + i];
  } else if (i == jc) {
    a = make_double2(A[(size_t)jc * lda + i].x, 0.0);
  } else {
    const double2 t = A[(size_t)i * lda + jc];
    a = make_double2(t.x, -t.y);
  }
  M[(size_t)jc * n + i] = a;
}

// M (2n x 2n, ld 2n) = [0 A; A^H 0].
__global__ void jordan_wielandt_kernel(const double2* __restrict__ A, long long lda, int n,
                                       double2* __restrict__ M) {
  const int N = 2 * n;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int jc = blockIdx.y * 8 + threadIdx.y;
  if (i >= N || jc >= N) return;
  double2 a = make_double2(0.0, 0.0);
  if (i < n && jc >= n) {
    a = A[(size_t)(jc - n) * lda + i];
  } else if (i >= n && jc < n) {
    const double2 t = A[(size_t)(i - n) * lda + jc];
    a = make_double2(t.x, -t.y);
  }
  M[(size_t)jc * N + i] = a;
}

}  // namespace

size_t spectra_work_bytes(int N) {
  // d, e (N doubles each) | v, p (N complex each) | P (kMaxSplit * N complex)
  // | S (4 complex) | Q (N / kRedThreads + 1 complex), each 256-byte aligned
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return 2 * up(sizeof(double) * N) + 2 * up(sizeof(double2) * N) +
         up(sizeof(double2) * (size_t)kMaxSplit * N) + up(sizeof(double2) * 4) +
         up(sizeof(double2) * ((size_t)N / kRedThreads + 1));
}

void launch_herm_from_upper(const double2* A, long long lda, int n, double2* M, cudaStream_t s) {
  dim3 grid((n + 31) / 32, (n + 7) / 8);
  herm_from_upper_kernel<<<grid, dim3(32, 8), 0, s>>>(A, lda, n, M);
}

void launch_jordan_wielandt(const double2* A, long long lda, int n, double2* M, cudaStream_t s) {
  const int N = 2 * n;
  dim3 grid((N + 31) / 32, (N + 7) / 8);
  jordan_wielandt_kernel<<<grid, dim3(32, 8), 0, s>>>(A, lda, n, M);
}

long long launch_tridiag_eigs(double2* M, int N, int count, int descending, void* work,
                              double* out, int sms, cudaStream_t s) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* w = static_cast<char*>(work);
  double* d = reinterpret_cast<double*>(w);
  w += up(sizeof(double) * N);
  double* e = reinterpret_cast<double*>(w);
  w += up(sizeof(double) * N);
  double2* v = reinterpret_cast<double2*>(w);
  w += up(sizeof(double2) * N);
  double2* p = reinterpret_cast<double2*>(w);
  w += up(sizeof(double2) * N);
  double2* P = reinterpret_cast<double2*>(w);
  w += up(sizeof(double2) * (size_t)kMaxSplit * N);
  double2* S = reinterpret_cast<double2*>(w);
  w += up(sizeof(double2) * 4);
  double2* Q = reinterpret_cast<double2*>(w);
  long long launches = 0;
  const long long ld = N;
  for (int j = 0; j + 1 < N; ++j) {
    const int m = N - j - 1;
    house_kernel<<<1, kHouseThreads, 0, s>>>(M, ld, N, j, v, S, d, e);
    // column split: about four blocks per SM in all
    const int nb = (m + kMvRows - 1) / kMvRows;
    int ns = std::min(kMaxSplit, std::max(1, (4 * sms + nb - 1) / nb));
    const int chunk = (m + ns - 1) / ns;
    ns = (m + chunk - 1) / chunk;
    hemv_part_kernel<<<dim3(nb, ns), kMvRows, 0, s>>>(M, ld, N, j, v, chunk, P);
    const int nq = (m + kRedThreads - 1) / kRedThreads;
    reduce_p_kernel<<<nq, kRedThreads, 0, s>>>(N, j, ns, P, S, v, p, Q);
    const int nt = (m + 31) / 32;
    her2_kernel<<<dim3(nt, nt), dim3(32, 8), 0, s>>>(M, ld, N, j, v, p, S, Q, nq);
    launches += 4;
  }
  last_diag_kernel<<<1, 1, 0, s>>>(M, ld, N, d);
  bisect_kernel<<<(count + 127) / 128, 128, 0, s>>>(d, e, N, count, descending, out);
  return launches + 2;
}

}  // namespace bem2d_gpu
