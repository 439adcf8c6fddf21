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
// y = A x (n x n), column chunks of 256 with per-row partial sums, then sum;
// complex128 or complex64 (the latter summed on the FP32 pipe).
constexpr int kMvChunk = 256;
template <typename T>
__global__ void mv_partial_kernel(const T* __restrict__ A, long long lda, int n,
                                  const T* __restrict__ x, T* part) {
  __shared__ T xs[kMvChunk];
  const int c0 = blockIdx.y * kMvChunk;
  const int nc = min(kMvChunk, n - c0);
  for (int v = threadIdx.x; v < nc; v += blockDim.x) xs[v] = x[c0 + v];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  T acc = CTraits<T>::make(0, 0);
  const T* col = A + (size_t)c0 * lda + r;
#pragma unroll 4
  for (int c = 0; c < nc; ++c) acc = cfma(col[(size_t)c * lda], xs[c], acc);
  part[(size_t)blockIdx.y * n + r] = acc;
}

template <typename T>
__global__ void mv_final_kernel(int n, int nchunk, const T* __restrict__ part, T* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T acc = CTraits<T>::make(0, 0);
  for (int c = 0; c < nchunk; ++c) {
    acc.x += part[(size_t)c * n + i].x;
    acc.y += part[(size_t)c * n + i].y;
  }
  y[i] = acc;
}

// y = A^H x: one warp per column, lanes over rows (coalesced), shuffle sum.
template <typename T>
__global__ void mvh_kernel(const T* __restrict__ A, long long lda, int n, const T* __restrict__ x,
                           T* __restrict__ y) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  const T* col = A + (size_t)j * lda;
  typename CTraits<T>::R sr = 0, si = 0;
#pragma unroll 4
  for (int r = lane; r < n; r += 32) {
    const T a = col[r], b = x[r];
    sr = fma(a.x, b.x, fma(a.y, b.y, sr));  // conj(a) b
    si = fma(a.x, b.y, fma(-a.y, b.x, si));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) y[j] = CTraits<T>::make(sr, si);
}

size_t mv_part_bytes(int n) {
  return sizeof(double2) * (size_t)n * ((n + kMvChunk - 1) / kMvChunk);
}

template <typename T>
static void mv_t(const T* A, long long lda, int n, const T* x, T* y, T* part, cudaStream_t s) {
  const int nchunk = (n + kMvChunk - 1) / kMvChunk;
  mv_partial_kernel<T><<<dim3((n + 127) / 128, nchunk), 128, 0, s>>>(A, lda, n, x, part);
  mv_final_kernel<T><<<(n + 255) / 256, 256, 0, s>>>(n, nchunk, part, y);
}

void launch_mv(const double2* A, long long lda, int n, const double2* x, double2* y,
               double2* part, cudaStream_t s) {
  mv_t(A, lda, n, x, y, part, s);
}
void launch_mv(const float2* A, long long lda, int n, const float2* x, float2* y, float2* part,
               cudaStream_t s) {
  mv_t(A, lda, n, x, y, part, s);
}

void launch_mvh(const double2* A, long long lda, int n, const double2* x, double2* y,
                cudaStream_t s) {
  mvh_kernel<double2><<<(n + 7) / 8, 256, 0, s>>>(A, lda, n, x, y);
}
void launch_mvh(const float2* A, long long lda, int n, const float2* x, float2* y,
                cudaStream_t s) {
  mvh_kernel<float2><<<(n + 7) / 8, 256, 0, s>>>(A, lda, n, x, y);
}

// ---- matrix-matrix products: C (n x m) = op(A) (n x n) B (n x m) -------------
// op = A or A^H; 64 x BN output tiles (BN = 64, 16 or 4 by the width m),
// K in chunks of 16; 256 threads as TX x TY, each RA x RB outputs.  The K
// range may be split over gridDim.z: split z writes its partial product to
// C + z * cz and zgemm_reduce_kernel adds the partials in a fixed order
// (deterministic), so that narrow products (few Lanczos vectors) still
// fill the GPU.  T = double2 (complex128) or float2 (complex64).
// `rows` is the row count of op(A) and C (n for the square products).
template <typename T, bool HERM, int BN>
__global__ void __launch_bounds__(256)
zgemm_kernel(const T* __restrict__ A, long long lda, int n, const T* __restrict__ B,
             long long ldb, int m, T* __restrict__ C, long long ldc, int kchunk, long long cz,
             int rows) {
  constexpr int TY = BN >= 16 ? 16 : BN, TX = 256 / TY, RA = 64 / TX, RB = BN / TY;
  __shared__ T As[16][64 + 1];
  __shared__ T Bs[16][BN + 1];
  const T zero = CTraits<T>::make(0, 0);
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * BN;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int kb = blockIdx.z * kchunk, ke = min(n, kb + kchunk);
  T* Cz = C + (size_t)blockIdx.z * cz;
  T acc[RA][RB];
#pragma unroll
  for (int a = 0; a < RA; ++a)
#pragma unroll
    for (int b = 0; b < RB; ++b) acc[a][b] = zero;
  for (int k0 = kb; k0 < ke; k0 += 16) {
    for (int v = threadIdx.x; v < 16 * 64; v += 256) {
      const int kk = v / 64, ii = v - kk * 64;
      const int i = i0 + ii, k = k0 + kk;
      T a = zero;
      if (i < rows && k < ke) {
        if (HERM) {
          const T t = A[(size_t)i * lda + k];  // (A^H)_{ik} = conj(A_{ki})
          a = CTraits<T>::make(t.x, -t.y);
        } else {
          a = A[(size_t)k * lda + i];
        }
      }
      As[kk][ii] = a;
    }
    for (int v = threadIdx.x; v < 16 * BN; v += 256) {
      const int jj = v / 16, kk = v - jj * 16;
      const int j = j0 + jj, k = k0 + kk;
      Bs[kk][jj] = (j < m && k < ke) ? B[(size_t)j * ldb + k] : zero;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; ++kk) {
      T av[RA], bv[RB];
#pragma unroll
      for (int a = 0; a < RA; ++a) av[a] = As[kk][tx + TX * a];
#pragma unroll
      for (int b = 0; b < RB; ++b) bv[b] = Bs[kk][ty + TY * b];
#pragma unroll
      for (int a = 0; a < RA; ++a)
#pragma unroll
        for (int b = 0; b < RB; ++b) acc[a][b] = cfma(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < RB; ++b) {
    const int j = j0 + ty + TY * b;
    if (j >= m) continue;
#pragma unroll
    for (int a = 0; a < RA; ++a) {
      const int i = i0 + tx + TX * a;
      if (i < rows) Cz[(size_t)j * ldc + i] = acc[a][b];
    }
  }
}

// C (ldc) = sum over z < nz of P + z cz (leading dimension n), z in order
template <typename T>
__global__ void zgemm_reduce_kernel(const T* __restrict__ P, long long cz, int nz, int n, int m,
                                    T* __restrict__ C, long long ldc) {
  const int j = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || j >= m) return;
  T s = P[(size_t)j * n + i];
  for (int z = 1; z < nz; ++z) {
    const T v = P[(size_t)z * cz + (size_t)j * n + i];
    s.x += v.x;
    s.y += v.y;
  }
  C[(size_t)j * ldc + i] = s;
}

// K splits for an n x m product: enough CTAs for two per SM (152 SMs), each
// split at least 256 deep
static int zgemm_splits(int n, int m, int bn) {
  const long long tiles = (long long)((n + 63) / 64) * ((m + bn - 1) / bn);
  const long long want = (2 * 152 + tiles - 1) / tiles;
  return (int)std::max<long long>(1, std::min<long long>(want, n / 256));
}

static int zgemm_bn(int m) { return m <= 4 ? 4 : (m <= 16 ? 16 : 64); }

// C (rows x m) = A (rows x k) B (k x m), complex128, no K split
void launch_zgemm_rect(const double2* A, long long lda, int rows, int k, const double2* B,
                       long long ldb, int m, double2* C, long long ldc, cudaStream_t s) {
  if (rows <= 0 || m <= 0) return;
  const int bn = zgemm_bn(m);
  const int kchunk = (k + 15) / 16 * 16;
  dim3 g((rows + 63) / 64, (m + bn - 1) / bn, 1);
  if (bn == 4)
    zgemm_kernel<double2, false, 4><<<g, 256, 0, s>>>(A, lda, k, B, ldb, m, C, ldc, kchunk, 0, rows);
  else if (bn == 16)
    zgemm_kernel<double2, false, 16><<<g, 256, 0, s>>>(A, lda, k, B, ldb, m, C, ldc, kchunk, 0, rows);
  else
    zgemm_kernel<double2, false, 64><<<g, 256, 0, s>>>(A, lda, k, B, ldb, m, C, ldc, kchunk, 0, rows);
}

size_t zgemm_work_bytes(int n, int m, size_t elem) {
  const int z = zgemm_splits(n, m, zgemm_bn(m));
  return z > 1 ? elem * (size_t)z * n * m : 0;
}

template <typename T, int BN>
static void zgemm_bn_t(bool herm, const T* A, long long lda, int n, const T* B, long long ldb,
                       int m, T* C, long long ldc, T* P, int z, cudaStream_t s) {
  const int kchunk = ((n + z - 1) / z + 15) / 16 * 16;
  dim3 g((n + 63) / 64, (m + BN - 1) / BN, z);
  T* out = z > 1 ? P : C;
  const long long lo = z > 1 ? n : ldc, cz = z > 1 ? (long long)n * m : 0;
  if (herm)
    zgemm_kernel<T, true, BN><<<g, 256, 0, s>>>(A, lda, n, B, ldb, m, out, lo, kchunk, cz, n);
  else
    zgemm_kernel<T, false, BN><<<g, 256, 0, s>>>(A, lda, n, B, ldb, m, out, lo, kchunk, cz, n);
  if (z > 1)
    zgemm_reduce_kernel<T><<<dim3((n + 255) / 256, m), 256, 0, s>>>(P, cz, z, n, m, C, ldc);
}

template <typename T>
static void zgemm_t(bool herm, const T* A, long long lda, int n, const T* B, long long ldb, int m,
                    T* C, long long ldc, void* work, size_t work_bytes, cudaStream_t s) {
  if (m <= 0 || n <= 0) return;
  const int bn = zgemm_bn(m);
  int z = zgemm_splits(n, m, bn);
  if (z > 1 && work_bytes < sizeof(T) * (size_t)z * n * m) z = 1;  // no room: one pass
  T* P = static_cast<T*>(work);
  if (bn == 4)
    zgemm_bn_t<T, 4>(herm, A, lda, n, B, ldb, m, C, ldc, P, z, s);
  else if (bn == 16)
    zgemm_bn_t<T, 16>(herm, A, lda, n, B, ldb, m, C, ldc, P, z, s);
  else
    zgemm_bn_t<T, 64>(herm, A, lda, n, B, ldb, m, C, ldc, P, z, s);
}
// ---- complex GEMM in float-float on the FP32 pipe ----------------------------
// C = op(A) B for complex128 data whose products are wanted to ~1e-13
// relative (the second, FP64-accurate phase of the numerical range), on the
// FP32 pipe, which issues 64x the FP64 pipe's FMAs on GB300.  A is given
// split once into A_hi = fl32(A), A_lo = fl32(A - A_hi) (float2 each); B is
// split while it is staged.  Per complex multiply-add the four hi*hi real
// products are exact as two-products (p + e) and accumulated with two-sum
// into a float-float sum; the hi*lo and lo*hi terms (2^-24 of the main ones)
// and the two-product errors go into a plain FP32 companion sum; lo*lo
// (2^-48) is dropped.  Result: hi + lo + companion, in FP64.  Partial sums
// of a K split are reduced in FP64.
struct FfAcc {
  float hi, lo, x;  // value = hi + lo + x
};

__device__ __forceinline__ void ffacc_add(FfAcc& a, float p) {
  const float s = a.hi + p;
  const float bb = s - a.hi;
  a.lo += (a.hi - (s - bb)) + (p - bb);
  a.hi = s;
}

template <bool HERM, int BN>
__global__ void __launch_bounds__(256)
zgemm_ff_kernel(const float2* __restrict__ Ahi, const float2* __restrict__ Alo, long long lda,
                int n, const float2* __restrict__ Bhi, const float2* __restrict__ Blo, long long ldb,
                int m, double2* __restrict__ C, long long ldc, int kchunk, long long cz,
                int rows) {
  constexpr int TY = BN >= 16 ? 16 : BN, TX = 256 / TY, RA = 64 / TX, RB = BN / TY;
  constexpr int LA = 16 * 64 / 256, LB = (16 * BN + 255) / 256;  // staged entries per thread
  __shared__ float2 Ah[16][64 + 1], Al[16][64 + 1];
  __shared__ float2 Bh[16][BN + 1], Bl[16][BN + 1];
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * BN;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int kb = blockIdx.z * kchunk, ke = min(n, kb + kchunk);
  double2* Cz = C + (size_t)blockIdx.z * cz;
  FfAcc re[RA][RB], im[RA][RB];
#pragma unroll
  for (int a = 0; a < RA; ++a)
#pragma unroll
    for (int b = 0; b < RB; ++b) re[a][b] = im[a][b] = FfAcc{0.f, 0.f, 0.f};
  // the next chunk's entries, loaded while the current chunk is computed
  float2 nah[LA], nal[LA], nbh[LB], nbl[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int u = 0; u < LA; ++u) {
      const int v = threadIdx.x + 256 * u, kk = v / 64, ii = v - kk * 64;
      const int i = i0 + ii, k = k0 + kk;
      float2 h = make_float2(0.f, 0.f), l = h;
      if (i < rows && k < ke) {
        const size_t o = HERM ? (size_t)i * lda + k : (size_t)k * lda + i;
        h = Ahi[o];
        l = Alo[o];
        if (HERM) {  // (A^H)_{ik} = conj(A_{ki})
          h.y = -h.y;
          l.y = -l.y;
        }
      }
      nah[u] = h;
      nal[u] = l;
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int v = threadIdx.x + 256 * u, jj = v / 16, kk = v - jj * 16;
      const int j = j0 + jj, k = k0 + kk;
      const bool ok = v < 16 * BN && j < m && k < ke;
      nbh[u] = ok ? Bhi[(size_t)j * ldb + k] : make_float2(0.f, 0.f);
      nbl[u] = ok ? Blo[(size_t)j * ldb + k] : make_float2(0.f, 0.f);
    }
  };
  load(kb);
  for (int k0 = kb; k0 < ke; k0 += 16) {
#pragma unroll
    for (int u = 0; u < LA; ++u) {
      const int v = threadIdx.x + 256 * u, kk = v / 64, ii = v - kk * 64;
      Ah[kk][ii] = nah[u];
      Al[kk][ii] = nal[u];
    }
#pragma unroll
    for (int u = 0; u < LB; ++u) {
      const int v = threadIdx.x + 256 * u, jj = v / 16, kk = v - jj * 16;
      if (v < 16 * BN) {
        Bh[kk][jj] = nbh[u];
        Bl[kk][jj] = nbl[u];
      }
    }
    __syncthreads();
    if (k0 + 16 < ke) load(k0 + 16);
#pragma unroll 2
    for (int kk = 0; kk < 16; ++kk) {
      float2 ah[RA], al[RA], bh[RB], bl[RB];
#pragma unroll
      for (int a = 0; a < RA; ++a) {
        ah[a] = Ah[kk][tx + TX * a];
        al[a] = Al[kk][tx + TX * a];
      }
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        bh[b] = Bh[kk][ty + TY * b];
        bl[b] = Bl[kk][ty + TY * b];
      }
#pragma unroll
      for (int a = 0; a < RA; ++a)
#pragma unroll
        for (int b = 0; b < RB; ++b) {
          // re += ar br - ai bi,  im += ar bi + ai br
          const float p1 = __fmul_rn(ah[a].x, bh[b].x), p2 = __fmul_rn(ah[a].y, bh[b].y);
          const float p3 = __fmul_rn(ah[a].x, bh[b].y), p4 = __fmul_rn(ah[a].y, bh[b].x);
          float xr = fmaf(ah[a].x, bh[b].x, -p1) - fmaf(ah[a].y, bh[b].y, -p2);
          float xi = fmaf(ah[a].x, bh[b].y, -p3) + fmaf(ah[a].y, bh[b].x, -p4);
          xr = fmaf(ah[a].x, bl[b].x, xr);
          xr = fmaf(al[a].x, bh[b].x, xr);
          xr = fmaf(-ah[a].y, bl[b].y, xr);
          xr = fmaf(-al[a].y, bh[b].y, xr);
          xi = fmaf(ah[a].x, bl[b].y, xi);
          xi = fmaf(al[a].x, bh[b].y, xi);
          xi = fmaf(ah[a].y, bl[b].x, xi);
          xi = fmaf(al[a].y, bh[b].x, xi);
          ffacc_add(re[a][b], p1);
          ffacc_add(re[a][b], -p2);
          ffacc_add(im[a][b], p3);
          ffacc_add(im[a][b], p4);
          re[a][b].x += xr;
          im[a][b].x += xi;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < RB; ++b) {
    const int j = j0 + ty + TY * b;
    if (j >= m) continue;
#pragma unroll
    for (int a = 0; a < RA; ++a) {
      const int i = i0 + tx + TX * a;
      if (i < rows) {
        const FfAcc& r = re[a][b];
        const FfAcc& q = im[a][b];
        Cz[(size_t)j * ldc + i] = make_double2((double)r.hi + ((double)r.lo + (double)r.x),
                                               (double)q.hi + ((double)q.lo + (double)q.x));
      }
    }
  }
}

// hi / lo (rows x cols, ld rows) = the float-float split of S (complex128,
// column-major, ld lds)
__global__ void split_ff_kernel(const double2* __restrict__ S, long long lds, int rows, int cols,
                                float2* __restrict__ hi, float2* __restrict__ lo) {
  const long long tot = (long long)rows * cols;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < tot;
       v += (long long)gridDim.x * blockDim.x) {
    const long long j = v / rows, i = v - j * rows;
    const double2 d = S[j * lds + i];
    const float hx = (float)d.x, hy = (float)d.y;
    hi[v] = make_float2(hx, hy);
    lo[v] = make_float2((float)(d.x - (double)hx), (float)(d.y - (double)hy));
  }
}

void launch_split_ff(const double2* A, long long lda, int n, float2* hi, float2* lo,
                     cudaStream_t s) {
  split_ff_kernel<<<1024, 256, 0, s>>>(A, lda, n, n, hi, lo);
}

template <int BN>
static void zgemm_ff_bn(bool herm, const float2* Ahi, const float2* Alo, int n, const float2* Bhi,
                        const float2* Blo, int m, double2* C, long long ldc, double2* P, int z,
                        cudaStream_t s) {
  const int kchunk = ((n + z - 1) / z + 15) / 16 * 16;
  dim3 g((n + 63) / 64, (m + BN - 1) / BN, z);
  double2* out = z > 1 ? P : C;
  const long long lo = z > 1 ? n : ldc, cz = z > 1 ? (long long)n * m : 0;
  if (herm)
    zgemm_ff_kernel<true, BN><<<g, 256, 0, s>>>(Ahi, Alo, n, n, Bhi, Blo, n, m, out, lo, kchunk,
                                                cz, n);
  else
    zgemm_ff_kernel<false, BN><<<g, 256, 0, s>>>(Ahi, Alo, n, n, Bhi, Blo, n, m, out, lo, kchunk,
                                                 cz, n);
  if (z > 1)
    zgemm_reduce_kernel<double2><<<dim3((n + 255) / 256, m), 256, 0, s>>>(P, cz, z, n, m, C, ldc);
}

void launch_zgemm_ff(bool herm, const float2* Ahi, const float2* Alo, int n, const double2* B,
                     long long ldb, int m, double2* C, long long ldc, void* work,
                     size_t work_bytes, float2* bsplit, cudaStream_t s) {
  if (m <= 0 || n <= 0) return;
  // B split once here, not once per row tile of the product
  float2* Bhi = bsplit;
  float2* Blo = bsplit + (size_t)n * m;
  split_ff_kernel<<<std::min(1024, (int)(((long long)n * m + 255) / 256)), 256, 0, s>>>(
      B, ldb, n, m, Bhi, Blo);
  const int bn = zgemm_bn(m);
  int z = zgemm_splits(n, m, bn);
  if (z > 1 && work_bytes < sizeof(double2) * (size_t)z * n * m) z = 1;
  double2* P = static_cast<double2*>(work);
  if (bn == 4)
    zgemm_ff_bn<4>(herm, Ahi, Alo, n, Bhi, Blo, m, C, ldc, P, z, s);
  else if (bn == 16)
    zgemm_ff_bn<16>(herm, Ahi, Alo, n, Bhi, Blo, m, C, ldc, P, z, s);
  else
    zgemm_ff_bn<64>(herm, Ahi, Alo, n, Bhi, Blo, m, C, ldc, P, z, s);
}

void launch_zgemm(bool herm, const double2* A, long long lda, int n, const double2* B,
                  long long ldb, int m, double2* C, long long ldc, void* work,
                  size_t work_bytes, cudaStream_t s) {
  zgemm_t(herm, A, lda, n, B, ldb, m, C, ldc, work, work_bytes, s);
}
void launch_zgemm(bool herm, const float2* A, long long lda, int n, const float2* B,
                  long long ldb, int m, float2* C, long long ldc, void* work,
                  size_t work_bytes, cudaStream_t s) {
  zgemm_t(herm, A, lda, n, B, ldb, m, C, ldc, work, work_bytes, s);
}

// ---- batched vector kernels (columns of n x m blocks) ----------------------
// h[c * ldh + i] = sum_r conj(Q[c][r, i]) w[c][r] for i < j (Q[c] = Q + c*qstride);
// sums in double for both element types
template <typename T>
__global__ void batched_dots_kernel(const T* __restrict__ Q, long long qstride, int n, int j,
                                    const T* __restrict__ W, long long wstride,
                                    T* __restrict__ h, int ldh) {
  const int c = blockIdx.y, i = blockIdx.x;
  if (i >= j) return;
  const T* q = Q + (size_t)c * qstride + (size_t)i * n;
  const T* w = W + (size_t)c * wstride;
  // each thread's few terms in the vectors' own precision (complex64: the
  // FP32 pipe; FP64 accumulation there would run on the FP64 pipe, 1/64 of
  // the rate), the 256 partial sums in FP64
  typename CTraits<T>::R pr = 0, pi = 0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const T a = q[r], b = w[r];
    pr = fma(a.x, b.x, fma(a.y, b.y, pr));
    pi = fma(a.x, b.y, fma(-a.y, b.x, pi));
  }
  const double sr = pr, si = pi;
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
  if (threadIdx.x == 0) h[(size_t)c * ldh + i] = CTraits<T>::make(red[0][0], red[1][0]);
}

// w[c] -= Q[c][:, :j] h[c]
template <typename T>
__global__ void batched_sub_kernel(const T* __restrict__ Q, long long qstride, int n, int j,
                                   T* __restrict__ W, long long wstride, const T* __restrict__ h,
                                   int ldh) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const T* q = Q + (size_t)c * qstride + r;
  T acc = W[(size_t)c * wstride + r];
  for (int i = 0; i < j; ++i) acc = cfms(acc, q[(size_t)i * n], h[(size_t)c * ldh + i]);
  W[(size_t)c * wstride + r] = acc;
}

// norms[c] = ||w[c]||_2^2
template <typename T>
__global__ void batched_norm2_kernel(int n, const T* __restrict__ W, long long wstride,
                                     double* __restrict__ out) {
  const int c = blockIdx.x;
  const T* w = W + (size_t)c * wstride;
  double s = 0;
  for (int r = threadIdx.x; r < n; r += blockDim.x)
    s += (double)w[r].x * w[r].x + (double)w[r].y * w[r].y;
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
template <typename T>
__global__ void batched_scale_kernel(int n, const T* __restrict__ src, long long sstride,
                                     const double* __restrict__ scale, T* __restrict__ dst,
                                     long long dstride) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double f = scale[c];
  const T v = src[(size_t)c * sstride + r];
  dst[(size_t)c * dstride + r] = CTraits<T>::make(v.x * f, v.y * f);
}

// numerical range: w[c] = (e^{i th_c} Y1[c] + e^{-i th_c} Y2[c]) / 2
template <typename T>
__global__ void herm_combine_kernel(int n, const T* __restrict__ Y1, const T* __restrict__ Y2,
                                    long long stride, const double* __restrict__ theta,
                                    T* __restrict__ W, long long wstride) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double s, co;
  sincos(theta[c], &s, &co);
  const T a = Y1[(size_t)c * stride + r], b = Y2[(size_t)c * stride + r];
  // (co + i s) a + (co - i s) b
  const double re = co * ((double)a.x + b.x) - s * ((double)a.y - b.y);
  const double im = co * ((double)a.y + b.y) + s * ((double)a.x - b.x);
  W[(size_t)c * wstride + r] = CTraits<T>::make(0.5 * re, 0.5 * im);
}

// dst (complex128) = src (complex64), columns of n x nb blocks
__global__ void widen_kernel(int n, const float2* __restrict__ src, long long sstride,
                             double2* __restrict__ dst, long long dstride) {
  const int c = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float2 v = src[(size_t)c * sstride + r];
  dst[(size_t)c * dstride + r] = make_double2(v.x, v.y);
}

template <typename T>
__global__ void gather_slots_kernel(const T* __restrict__ src, long long sstride,
                                    T* __restrict__ dst, long long dstride, long long len,
                                    const int* __restrict__ map) {
  const int i = blockIdx.y;
  const T* a = src + (size_t)map[i] * sstride;
  T* b = dst + (size_t)i * dstride;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < len;
       r += (long long)gridDim.x * blockDim.x)
    b[r] = a[r];
}

template <typename T>
__global__ void scatter_slots_kernel(const T* __restrict__ src, long long sstride,
                                     T* __restrict__ dst, long long dstride, long long len,
                                     const int* __restrict__ map) {
  const int i = blockIdx.y;
  const T* a = src + (size_t)i * sstride;
  T* b = dst + (size_t)map[i] * dstride;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < len;
       r += (long long)gridDim.x * blockDim.x)
    b[r] = a[r];
}

#define BEM2D_BATCHED_LAUNCHERS(T)                                                            \
  void launch_batched_dots(const T* Q, long long qstride, int n, int j, const T* W,           \
                           long long wstride, T* h, int ldh, int nb, cudaStream_t s) {        \
    if (j <= 0) return;                                                                       \
    batched_dots_kernel<T><<<dim3(j, nb), 256, 0, s>>>(Q, qstride, n, j, W, wstride, h, ldh); \
  }                                                                                           \
  void launch_batched_sub(const T* Q, long long qstride, int n, int j, T* W, long long wstride, \
                          const T* h, int ldh, int nb, cudaStream_t s) {                      \
    if (j <= 0) return;                                                                       \
    batched_sub_kernel<T><<<dim3((n + 127) / 128, nb), 128, 0, s>>>(Q, qstride, n, j, W,      \
                                                                   wstride, h, ldh);          \
  }                                                                                           \
  void launch_batched_norm2(int n, const T* W, long long wstride, double* out, int nb,        \
                            cudaStream_t s) {                                                 \
    batched_norm2_kernel<T><<<nb, 256, 0, s>>>(n, W, wstride, out);                           \
  }                                                                                           \
  void launch_batched_scale(int n, const T* src, long long sstride, const double* scale,      \
                            T* dst, long long dstride, int nb, cudaStream_t s) {              \
    batched_scale_kernel<T><<<dim3((n + 127) / 128, nb), 128, 0, s>>>(n, src, sstride, scale, \
                                                                     dst, dstride);           \
  }                                                                                           \
  void launch_herm_combine(int n, const T* Y1, const T* Y2, long long stride,                 \
                           const double* theta, T* W, long long wstride, int nb,              \
                           cudaStream_t s) {                                                  \
    herm_combine_kernel<T><<<dim3((n + 127) / 128, nb), 128, 0, s>>>(n, Y1, Y2, stride, theta, \
                                                                    W, wstride);              \
  }                                                                                           \
  void launch_gather_slots(const T* src, long long sstride, T* dst, long long dstride,        \
                           long long len, const int* map, int nmap, cudaStream_t s) {         \
    if (nmap <= 0 || len <= 0) return;                                                        \
    const long long bx = std::min<long long>((len + 255) / 256, 64);                         \
    gather_slots_kernel<T><<<dim3((unsigned)bx, nmap), 256, 0, s>>>(src, sstride, dst,       \
                                                                   dstride, len, map);       \
  }                                                                                           \
  void launch_scatter_slots(const T* src, long long sstride, T* dst, long long dstride,       \
                            long long len, const int* map, int nmap, cudaStream_t s) {        \
    if (nmap <= 0 || len <= 0) return;                                                        \
    const long long bx = std::min<long long>((len + 255) / 256, 64);                         \
    scatter_slots_kernel<T><<<dim3((unsigned)bx, nmap), 256, 0, s>>>(src, sstride, dst,      \
                                                                    dstride, len, map);      \
  }
BEM2D_BATCHED_LAUNCHERS(double2)
BEM2D_BATCHED_LAUNCHERS(float2)
#undef BEM2D_BATCHED_LAUNCHERS

void launch_widen(int n, const float2* src, long long sstride, double2* dst, long long dstride,
                  int nb, cudaStream_t s) {
  widen_kernel<<<dim3((n + 127) / 128, nb), 128, 0, s>>>(n, src, sstride, dst, dstride);
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


// Largest eigenvalue of the symmetric tridiagonal (d, e) by bisection on
// Sturm counts (the number of negative pivots of T - x I = L D L^T is the
// number of eigenvalues below x): O(n) per step, about 60 steps to full
// precision, against O(n^2) for a complete QL sweep.
double tridiag_lmax(const std::vector<double>& d, const std::vector<double>& e) {
  return tridiag_kth_largest(d, e, 1, 2.2e-16);
}

double tridiag_lmax_from(const std::vector<double>& d, const std::vector<double>& e, double lo,
                         double step, double atol) {
  const int n = (int)d.size();
  double scale = 0.0;  // Gershgorin bound of |spectrum|
  for (int i = 0; i < n; ++i)
    scale = std::max(scale, std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0) +
                                (i + 1 < n ? std::fabs(e[i]) : 0.0));
  if (!(scale > 0)) return 0.0;
  auto all_below = [&](double x) {  // every eigenvalue < x
    double q = 1.0;
    for (int i = 0; i < n; ++i) {
      q = d[i] - x - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
      if (q == 0.0) q = -1e-300 * scale;
      if (q >= 0) return false;
    }
    return true;
  };
  if (!(lo >= -scale)) lo = -scale;
  const double tol = std::max(atol, 2.2e-16 * scale);
  // grow the step until lo + step is an upper bound; lo stays a lower bound
  double dx = std::max(step, 4.0 * tol);
  double hi = lo + dx;
  for (int it = 0; it < 200 && !all_below(hi); ++it) {
    lo = hi;
    dx *= 4.0;
    hi = std::min(lo + dx, scale * (1.0 + 1e-15) + 1e-300);
    if (hi <= lo) break;
  }
  for (int it = 0; it < 200 && hi - lo > tol; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (all_below(mid))
      hi = mid;
    else
      lo = mid;
  }
  return lo;  // a lower bound again, for the next call
}

double tridiag_kth_largest(const std::vector<double>& d, const std::vector<double>& e, int k,
                           double rel) {
  const int n = (int)d.size();
  double lo = INFINITY, hi = -INFINITY;
  for (int i = 0; i < n; ++i) {  // Gershgorin bounds
    const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < n ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  const double scale = std::max(std::fabs(lo), std::fabs(hi));
  auto below = [&](double x) {  // eigenvalues < x
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < n; ++i) {
      q = d[i] - x - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
      if (q == 0.0) q = -1e-300 * std::max(scale, 1.0);
      if (q < 0) ++cnt;
    }
    return cnt;
  };
  for (int it = 0; it < 200 && hi - lo > rel * std::max(scale, 1e-300); ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (below(mid) > n - k)
      hi = mid;  // fewer than k eigenvalues at or above mid
    else
      lo = mid;
  }
  return 0.5 * (lo + hi);
}

// Inverse iteration: solve (T - sigma I) x = b twice with sigma just above
// lambda, by Gaussian elimination with partial pivoting on the tridiagonal
// (as LAPACK's dgtsv), and normalise.
std::vector<double> tridiag_eigenvector(const std::vector<double>& d, const std::vector<double>& e,
                                        double lambda) {
  const int n = (int)d.size();
  std::vector<double> x(n, 1.0);
  if (n == 1) return x;
  double anorm = 0;
  for (int i = 0; i < n; ++i)
    anorm = std::max(anorm, std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0) +
                                (i + 1 < n ? std::fabs(e[i]) : 0.0));
  const double sigma = lambda + 1e-13 * std::max(anorm, 1e-300);
  for (int it = 0; it < 3; ++it) {
    // rows: sub l[i] (i >= 1), diag m[i], super u[i], second super u2[i]
    std::vector<double> dl(n, 0.0), dm(n), du(n, 0.0), du2(n, 0.0), b(x);
    for (int i = 0; i < n; ++i) {
      dm[i] = d[i] - sigma;
      if (i + 1 < n) {
        du[i] = e[i];
        dl[i + 1] = e[i];
      }
    }
    for (int i = 0; i + 1 < n; ++i) {
      if (std::fabs(dm[i]) >= std::fabs(dl[i + 1])) {
        double f = dm[i] != 0.0 ? dl[i + 1] / dm[i] : 0.0;
        dm[i + 1] -= f * du[i];
        if (i + 2 < n) du[i + 1] -= f * du2[i];  // du2[i] is 0 here
        b[i + 1] -= f * b[i];
      } else {  // swap rows i and i+1
        const double f = dm[i] / dl[i + 1];
        const double t_m = dl[i + 1], t_u = dm[i + 1], t_u2 = (i + 2 < n) ? du[i + 1] : 0.0;
        dm[i + 1] = du[i] - f * t_u;
        if (i + 2 < n) du[i + 1] = -f * t_u2;
        dm[i] = t_m;
        du[i] = t_u;
        du2[i] = t_u2;
        const double tb = b[i];
        b[i] = b[i + 1];
        b[i + 1] = tb - f * b[i];
      }
    }
    const double tiny = 1e-300;
    for (int i = n - 1; i >= 0; --i) {
      double v = b[i];
      if (i + 1 < n) v -= du[i] * x[i + 1];
      if (i + 2 < n) v -= du2[i] * x[i + 2];
      const double piv = std::fabs(dm[i]) > tiny ? dm[i] : tiny;
      x[i] = v / piv;
    }
    double nrm = 0;
    for (double v : x) nrm += v * v;
    nrm = std::sqrt(nrm);
    if (!(nrm > 0) || !std::isfinite(nrm)) {
      std::fill(x.begin(), x.end(), 1.0 / std::sqrt((double)n));
      return x;
    }
    for (double& v : x) v /= nrm;
  }
  return x;
}

}  // namespace bem2d_gpu
