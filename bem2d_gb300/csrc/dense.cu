// Dense operators on the GPU beyond the LU: change of basis with a
// block-diagonal mass matrix, complex matrix-vector and matrix-matrix
// products, the conjugate-transposed LU solve, and the Lanczos drivers behind
// L2NormCond (extreme singular values) and NumRange (extreme eigenvalues of
// the Hermitian parts e^{i th} A + e^{-i th} A^H, all angles batched).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "common.cuh"
#include "cplx.cuh"
#include "dense.cuh"

namespace cg = cooperative_groups;

namespace bem2d_gpu {

// ---- change of basis ------------------------------------------------------
// out_ij = sum_{p in B(i)} sum_{q in B(j)} conj(Ui[p,i]) K_pq Ui[q,j], where Ui
// is the inverse Cholesky factor of the mass block B (stored per row i as
// the block's column: uinv[(size_t)i * 16 + (p - start)] = Ui[p, i]).
__global__ void change_basis_kernel(int n, const double2* __restrict__ K, long long ldk,
                                    const int* __restrict__ bstart_of,
                                    const int* __restrict__ bsize_of,
                                    const double2* __restrict__ uinv, double2* __restrict__ out,
                                    long long ldo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= n) return;
  const int si = bstart_of[i], ni = bsize_of[i];
  const int sj = bstart_of[j], nj = bsize_of[j];
  double2 acc = make_double2(0, 0);
  for (int q = 0; q < nj; ++q) {
    const double2 uq = uinv[(size_t)j * 16 + q];
    double2 t = make_double2(0, 0);
    for (int p = 0; p < ni; ++p) {
      const double2 up = uinv[(size_t)i * 16 + p];
      const double2 kpq = K[(size_t)(sj + q) * ldk + si + p];
      // conj(up) * kpq
      t.x += up.x * kpq.x + up.y * kpq.y;
      t.y += up.x * kpq.y - up.y * kpq.x;
    }
    acc = cfma(t, uq, acc);
  }
  out[(size_t)j * ldo + i] = acc;
}

void launch_change_basis(int n, const double2* K, long long ldk, const int* bstart_of,
                         const int* bsize_of, const double2* uinv, double2* out, long long ldo,
                         cudaStream_t s) {
  dim3 g((n + 127) / 128, n);
  change_basis_kernel<<<g, 128, 0, s>>>(n, K, ldk, bstart_of, bsize_of, uinv, out, ldo);
}

// gather the diagonal blocks of M: blk[i*16 + p] = M[start_i + p, i]
__global__ void gather_blocks_kernel(int n, const double2* __restrict__ M, long long ldm,
                                     const int* __restrict__ bstart_of,
                                     const int* __restrict__ bsize_of, double2* __restrict__ blk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = bstart_of[i], b = bsize_of[i];
  for (int p = 0; p < 16; ++p)
    blk[(size_t)i * 16 + p] = p < b ? M[(size_t)i * ldm + s + p] : make_double2(0, 0);
}

void launch_gather_blocks(int n, const double2* M, long long ldm, const int* bstart_of,
                          const int* bsize_of, double2* blk, cudaStream_t s) {
  gather_blocks_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, M, ldm, bstart_of, bsize_of, blk);
}

// ---- matrix-vector products ---------------------------------------------
// y = A x (n x n), column chunks of 256 with per-row partial sums, then sum.
constexpr int kMvChunk = 256;
__global__ void mv_partial_kernel(const double2* __restrict__ A, long long lda, int n,
                                  const double2* __restrict__ x, double2* part) {
  __shared__ double2 xs[kMvChunk];
  const int c0 = blockIdx.y * kMvChunk;
  const int nc = min(kMvChunk, n - c0);
  for (int v = threadIdx.x; v < nc; v += blockDim.x) xs[v] = x[c0 + v];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double2 acc = make_double2(0, 0);
  const double2* col = A + (size_t)c0 * lda + r;
#pragma unroll 4
  for (int c = 0; c < nc; ++c) acc = cfma(col[(size_t)c * lda], xs[c], acc);
  part[(size_t)blockIdx.y * n + r] = acc;
}

__global__ void mv_final_kernel(int n, int nchunk, const double2* __restrict__ part,
                                double2* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 acc = make_double2(0, 0);
  for (int c = 0; c < nchunk; ++c) {
    acc.x += part[(size_t)c * n + i].x;
    acc.y += part[(size_t)c * n + i].y;
  }
  y[i] = acc;
}

// y = A^H x: one warp per column, lanes over rows (coalesced), shuffle sum.
__global__ void mvh_kernel(const double2* __restrict__ A, long long lda, int n,
                           const double2* __restrict__ x, double2* __restrict__ y) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  const double2* col = A + (size_t)j * lda;
  double sr = 0, si = 0;
  for (int r = lane; r < n; r += 32) {
    const double2 a = col[r], b = x[r];
    sr += a.x * b.x + a.y * b.y;  // conj(a) b
    si += a.x * b.y - a.y * b.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) y[j] = make_double2(sr, si);
}

size_t mv_part_bytes(int n) {
  return sizeof(double2) * (size_t)n * ((n + kMvChunk - 1) / kMvChunk);
}

void launch_mv(const double2* A, long long lda, int n, const double2* x, double2* y,
               double2* part, cudaStream_t s) {
  const int nchunk = (n + kMvChunk - 1) / kMvChunk;
  mv_partial_kernel<<<dim3((n + 127) / 128, nchunk), 128, 0, s>>>(A, lda, n, x, part);
  mv_final_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, nchunk, part, y);
}

void launch_mvh(const double2* A, long long lda, int n, const double2* x, double2* y,
                cudaStream_t s) {
  mvh_kernel<<<(n + 7) / 8, 256, 0, s>>>(A, lda, n, x, y);
}

// ---- matrix-matrix products: C (n x m) = op(A) (n x n) B (n x m) -------------
// op = A or A^H; 64 x 64 output tiles, K in chunks of 16, 4 x 4 per thread.
template <bool HERM>
__global__ void __launch_bounds__(256)
zgemm_kernel(const double2* __restrict__ A, long long lda, int n, const double2* __restrict__ B,
             long long ldb, int m, double2* __restrict__ C, long long ldc) {
  __shared__ double2 As[16][64 + 1];
  __shared__ double2 Bs[16][64 + 1];
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0, 0);
  for (int k0 = 0; k0 < n; k0 += 16) {
    for (int v = threadIdx.x; v < 16 * 64; v += 256) {
      const int kk = v / 64, ii = v - kk * 64;
      const int i = i0 + ii, k = k0 + kk;
      double2 a = make_double2(0, 0);
      if (i < n && k < n) {
        if (HERM) {
          const double2 t = A[(size_t)i * lda + k];  // (A^H)_{ik} = conj(A_{ki})
          a = make_double2(t.x, -t.y);
        } else {
          a = A[(size_t)k * lda + i];
        }
      }
      As[kk][ii] = a;
    }
    for (int v = threadIdx.x; v < 16 * 64; v += 256) {
      const int jj = v / 16, kk = v - jj * 16;
      const int j = j0 + jj, k = k0 + kk;
      Bs[kk][jj] = (j < m && k < n) ? B[(size_t)j * ldb + k] : make_double2(0, 0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; ++kk) {
      double2 av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = cfma(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int j = j0 + ty + 16 * b;
    if (j >= m) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = i0 + tx + 16 * a;
      if (i < n) C[(size_t)j * ldc + i] = acc[a][b];
    }
  }
}

void launch_zgemm(bool herm, const double2* A, long long lda, int n, const double2* B,
                  long long ldb, int m, double2* C, long long ldc, cudaStream_t s) {
  dim3 g((n + 63) / 64, (m + 63) / 64);
  if (herm)
    zgemm_kernel<true><<<g, 256, 0, s>>>(A, lda, n, B, ldb, m, C, ldc);
  else
    zgemm_kernel<false><<<g, 256, 0, s>>>(A, lda, n, B, ldb, m, C, ldc);
}

// ---- batched vector kernels (columns of n x m blocks) ----------------------
// h[c * ldh + i] = sum_r conj(Q[c][r, i]) w[c][r] for i < j (Q[c] = Q + c*qstride)
__global__ void batched_dots_kernel(const double2* __restrict__ Q, long long qstride, int n,
                                    int j, const double2* __restrict__ W, long long wstride,
                                    double2* __restrict__ h, int ldh) {
  const int c = blockIdx.y, i = blockIdx.x;
  if (i >= j) return;
  const double2* q = Q + (size_t)c * qstride + (size_t)i * n;
  const double2* w = W + (size_t)c * wstride;
  double sr = 0, si = 0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const double2 a = q[r], b = w[r];
    sr += a.x * b.x + a.y * b.y;
    si += a.x * b.y - a.y * b.x;
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = sr;
  red[1][threadIdx.x] = si;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) h[(size_t)c * ldh + i] = make_double2(red[0][0], red[1][0]);
}

// w[c] -= Q[c][:, :j] h[c]
__global__ void batched_sub_kernel(const double2* __restrict__ Q, long long qstride, int n, int j,
                                   double2* __restrict__ W, long long wstride,
                                   const double2* __restrict__ h, int ldh) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double2* q = Q + (size_t)c * qstride + r;
  double2 acc = W[(size_t)c * wstride + r];
  for (int i = 0; i < j; ++i) acc = cfms(acc, q[(size_t)i * n], h[(size_t)c * ldh + i]);
  W[(size_t)c * wstride + r] = acc;
}

// norms[c] = ||w[c]||_2^2
__global__ void batched_norm2_kernel(int n, const double2* __restrict__ W, long long wstride,
                                     double* __restrict__ out) {
  const int c = blockIdx.x;
  const double2* w = W + (size_t)c * wstride;
  double s = 0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) s += w[r].x * w[r].x + w[r].y * w[r].y;
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

// dst[c] = src[c] * scale[c]
__global__ void batched_scale_kernel(int n, const double2* __restrict__ src, long long sstride,
                                     const double* __restrict__ scale, double2* __restrict__ dst,
                                     long long dstride) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double f = scale[c];
  const double2 v = src[(size_t)c * sstride + r];
  dst[(size_t)c * dstride + r] = make_double2(v.x * f, v.y * f);
}

// numerical range: w[c] = (e^{i th_c} Y1[c] + e^{-i th_c} Y2[c]) / 2
__global__ void herm_combine_kernel(int n, const double2* __restrict__ Y1,
                                    const double2* __restrict__ Y2, long long stride,
                                    const double* __restrict__ theta, double2* __restrict__ W,
                                    long long wstride) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double s, co;
  sincos(theta[c], &s, &co);
  const double2 a = Y1[(size_t)c * stride + r], b = Y2[(size_t)c * stride + r];
  // (co + i s) a + (co - i s) b
  const double re = co * (a.x + b.x) - s * (a.y - b.y);
  const double im = co * (a.y + b.y) + s * (a.x - b.x);
  W[(size_t)c * wstride + r] = make_double2(0.5 * re, 0.5 * im);
}

void launch_batched_dots(const double2* Q, long long qstride, int n, int j, const double2* W,
                         long long wstride, double2* h, int ldh, int nb, cudaStream_t s) {
  if (j <= 0) return;
  batched_dots_kernel<<<dim3(j, nb), 256, 0, s>>>(Q, qstride, n, j, W, wstride, h, ldh);
}
void launch_batched_sub(const double2* Q, long long qstride, int n, int j, double2* W,
                        long long wstride, const double2* h, int ldh, int nb, cudaStream_t s) {
  if (j <= 0) return;
  batched_sub_kernel<<<dim3((n + 127) / 128, nb), 128, 0, s>>>(Q, qstride, n, j, W, wstride, h,
                                                              ldh);
}
void launch_batched_norm2(int n, const double2* W, long long wstride, double* out, int nb,
                          cudaStream_t s) {
  batched_norm2_kernel<<<nb, 256, 0, s>>>(n, W, wstride, out);
}
void launch_batched_scale(int n, const double2* src, long long sstride, const double* scale,
                          double2* dst, long long dstride, int nb, cudaStream_t s) {
  batched_scale_kernel<<<dim3((n + 127) / 128, nb), 128, 0, s>>>(n, src, sstride, scale, dst,
                                                                dstride);
}
void launch_herm_combine(int n, const double2* Y1, const double2* Y2, long long stride,
                         const double* theta, double2* W, long long wstride, int nb,
                         cudaStream_t s) {
  herm_combine_kernel<<<dim3((n + 127) / 128, nb), 128, 0, s>>>(n, Y1, Y2, stride, theta, W,
                                                               wstride);
}

// y -= a x (real a)
__global__ void axpy_real_kernel(int n, double a, const double2* __restrict__ x,
                                 double2* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  y[r].x -= a * x[r].x;
  y[r].y -= a * x[r].y;
}
void launch_axpy_real(int n, double a, const double2* x, double2* y, cudaStream_t s) {
  axpy_real_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, a, x, y);
}

// ---- host: eigenvalues of a real symmetric tridiagonal matrix ------------------
// Implicit QL with Wilkinson shifts (eigenvalues only); d: diagonal, e:
// sub-diagonal (e[n-1] unused).  Returns false if it did not converge.
bool tridiag_eigenvalues(std::vector<double> d, std::vector<double> e, std::vector<double>* ev) {
  const int n = (int)d.size();
  e.resize(n, 0.0);
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m;
      for (m = l; m < n - 1; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 + 2.2e-16 * dd) break;
      }
      if (m == l) break;
      if (++iter > 80) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      bool early = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[m] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
      }
      if (early) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  *ev = d;
  return true;
}

}  // namespace bem2d_gpu
