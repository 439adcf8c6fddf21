// Blocked right-looking LU with partial pivoting and the triangular solves,
// for complex128 (double2) and complex64 (float2).  Replaces LAPACK zgetrf +
// zgetrs as called by SolveSystem (lib/bem2d_mathroutines.cpp:323-351).
//
// Per panel of NB columns:
//   panel_kernel   cooperative launch, one CTA per SM; each CTA keeps its
//                  slice of the panel rows in shared memory.  One bounded grid
//                  barrier per column: every CTA publishes its local pivot
//                  candidate (value, row, whole panel row); after the barrier
//                  all CTAs agree on the pivot, swap locally and update.
//   laswp_kernel   applies the panel's row swaps to the trailing columns
//   trsm_kernel    U12 = L11^{-1} A12
//   gemm_kernel    A22 -= L21 U12  (register-tiled, 64 x 64 CTA tiles)
// The swaps are not applied to the columns left of the panel; the forward
// solve applies each panel's swaps to the right-hand side just before that
// panel's columns of L (identical to LAPACK's P, L, U up to row storage).
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>

#include "common.cuh"
#include "cplx.cuh"

namespace bem2d_gpu {

constexpr int kNB = 64;              // panel width
constexpr int kPanelThreads = 256;
constexpr unsigned kSpinLimit = 1u << 25;  // polls of 64 ns: ~2 s

// Bounded grid-wide barrier for a cooperative launch.  A block that waits
// longer than the limit records status = 1 and returns false; every later
// call returns false at once, so the kernel winds down without hanging.
__device__ bool grid_sync(unsigned* bar, unsigned nblocks, int* status) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    if (*(volatile int*)status != 0) {
      ok = 0;
    } else {
      volatile unsigned* vgen = bar + 1;
      const unsigned gen = *vgen;
      __threadfence();
      const unsigned arrived = atomicAdd(bar, 1u);
      if (arrived == nblocks - 1) {
        atomicExch(bar, 0u);
        __threadfence();
        atomicAdd(bar + 1, 1u);
      } else {
        unsigned it = 0;
        while (*vgen == gen) {
          if (++it > kSpinLimit) {
            atomicExch(status, 1);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
  return ok != 0;
}

// (value, row) arg-max with ties to the smaller row, as LAPACK's izamax
// (first maximal |re| + |im|).
template <typename R>
__device__ __forceinline__ void argmax_merge(R& v, int& i, R v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

template <typename R>
__device__ void block_argmax(R& v, int& i) {
  __shared__ R sv[kPanelThreads / 32];
  __shared__ int si[kPanelThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const R v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
    argmax_merge(v, i, v2, i2);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sv[w] = v;
    si[w] = i;
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
  for (int k = 1; k < (int)(blockDim.x >> 5); ++k) argmax_merge(v, i, sv[k], si[k]);
}

// Panel exchange buffers, per parity: candidate value / row / panel row of
// each block, and the current row kc.
template <typename T>
struct PanelBufs {
  typename CTraits<T>::R* val;  // [2][maxb]
  int* idx;                     // [2][maxb]
  T* cand;                      // [2][maxb][kNB]
  T* krow;                      // [2][kNB]
};

constexpr int kMaxPanelBlocks = 1024;

template <typename T>
static PanelBufs<T> panel_bufs(void* scratch) {
  typedef typename CTraits<T>::R R;
  PanelBufs<T> b;
  char* p = static_cast<char*>(scratch);
  b.cand = reinterpret_cast<T*>(p);
  p += sizeof(T) * 2 * kMaxPanelBlocks * kNB;
  b.krow = reinterpret_cast<T*>(p);
  p += sizeof(T) * 2 * kNB;
  b.val = reinterpret_cast<R*>(p);
  p += sizeof(R) * 2 * kMaxPanelBlocks;
  b.idx = reinterpret_cast<int*>(p);
  return b;
}

size_t lu_scratch_bytes(int) {
  return sizeof(double2) * 2 * kMaxPanelBlocks * kNB + sizeof(double2) * 2 * kNB +
         sizeof(double) * 2 * kMaxPanelBlocks + sizeof(int) * 2 * kMaxPanelBlocks + 256;
}

template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_kernel(T* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
             int* __restrict__ ipiv, int* info, int* status, unsigned* bar,
             PanelBufs<T> buf) {
  typedef typename CTraits<T>::R R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // [rpb][kNB] block's panel rows
  T* prow = P + (size_t)rpb * kNB;        // [kNB] pivot row
  T* lcol = prow + kNB;                   // [rpb] multipliers
  __shared__ int s_p, s_bw;
  __shared__ R s_pv;

  const int nblk = gridDim.x, b = blockIdx.x;
  const int r0 = k0 + b * rpb;
  const int r1 = min(r0 + rpb, n);
  const int nr = max(r1 - r0, 0);
  for (int v = threadIdx.x; v < nr * nb; v += blockDim.x) {
    const int c = v / nr, lr = v - c * nr;
    P[lr * kNB + c] = A[(size_t)(k0 + c) * lda + r0 + lr];
  }
  __syncthreads();

  for (int c = 0; c < nb; ++c) {
    const int kc = k0 + c, par = c & 1;
    // (a) local pivot candidate among rows >= kc
    R best = -1;
    int bidx = INT_MAX;
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const int gr = r0 + lr;
      if (gr < kc) continue;
      argmax_merge(best, bidx, cabs1(P[lr * kNB + c]), gr);
    }
    block_argmax(best, bidx);
    // (b) publish candidate and, from the owner, row kc
    if (threadIdx.x == 0) {
      buf.val[par * kMaxPanelBlocks + b] = best;
      buf.idx[par * kMaxPanelBlocks + b] = bidx;
    }
    if (bidx != INT_MAX)
      for (int j = threadIdx.x; j < nb; j += blockDim.x)
        buf.cand[((size_t)par * kMaxPanelBlocks + b) * kNB + j] = P[(bidx - r0) * kNB + j];
    if (kc >= r0 && kc < r1)
      for (int j = threadIdx.x; j < nb; j += blockDim.x)
        buf.krow[par * kNB + j] = P[(kc - r0) * kNB + j];
    __threadfence();
    if (!grid_sync(bar, nblk, status)) return;
    // (c) agree on the pivot
    {
      R v = -1;
      int i = INT_MAX, w = 0;
      for (int q = threadIdx.x; q < nblk; q += blockDim.x) {
        const R v2 = __ldcg(&buf.val[par * kMaxPanelBlocks + q]);
        const int i2 = __ldcg(&buf.idx[par * kMaxPanelBlocks + q]);
        argmax_merge(v, i, v2, i2);
      }
      block_argmax(v, i);
      if (threadIdx.x == 0) {
        // no finite candidate (all NaN): treat as a zero pivot at row kc
        if (i == INT_MAX || i < kc || i >= n) {
          i = kc;
          v = 0;
        }
        // the owner block of row i published it
        w = (i - k0) / rpb;
        s_p = i;
        s_bw = w;
        s_pv = v;
      }
    }
    __syncthreads();
    const int p = s_p, bw = s_bw;
    const bool zero = !(s_pv > 0);
    for (int j = threadIdx.x; j < nb; j += blockDim.x)
      prow[j] = __ldcg(&buf.cand[((size_t)par * kMaxPanelBlocks + bw) * kNB + j]);
    if (b == 0 && threadIdx.x == 0) {
      ipiv[kc] = p;
      if (zero && *info == 0) *info = kc + 1;
    }
    __syncthreads();
    if (!zero && p != kc) {
      if (p >= r0 && p < r1)
        for (int j = threadIdx.x; j < nb; j += blockDim.x)
          P[(p - r0) * kNB + j] = __ldcg(&buf.krow[par * kNB + j]);
      if (kc >= r0 && kc < r1)
        for (int j = threadIdx.x; j < nb; j += blockDim.x) P[(kc - r0) * kNB + j] = prow[j];
    }
    __syncthreads();
    // (d) multipliers and rank-1 update of the block's rows below kc
    if (!zero) {
      const T inv = crcp(prow[c]);
      for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
        if (r0 + lr > kc) {
          const T l = cmul(P[lr * kNB + c], inv);
          P[lr * kNB + c] = l;
          lcol[lr] = l;
        }
      }
      __syncthreads();
      const int w = nb - c - 1;
      if (w > 0) {
        for (int v = threadIdx.x; v < nr * w; v += blockDim.x) {
          const int lr = v / w, cc = c + 1 + (v - lr * w);
          if (r0 + lr > kc) P[lr * kNB + cc] = cfms(P[lr * kNB + cc], lcol[lr], prow[cc]);
        }
      }
    }
    __syncthreads();
  }
  for (int v = threadIdx.x; v < nr * nb; v += blockDim.x) {
    const int c = v / nr, lr = v - c * nr;
    A[(size_t)(k0 + c) * lda + r0 + lr] = P[lr * kNB + c];
  }
}

template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, long long lda, int c0, int ncols,
                             const int* __restrict__ ipiv, int k0, int nb) {
  const int j = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c0 + ncols) return;
  T* col = A + (size_t)j * lda;
  for (int s = 0; s < nb; ++s) {
    const int p = ipiv[k0 + s];
    if (p != k0 + s) {
      const T t = col[k0 + s];
      col[k0 + s] = col[p];
      col[p] = t;
    }
  }
}

// X = L11^{-1} X for X = A[k0:k0+nb, c0:c0+32), L11 unit lower.
template <typename T>
__global__ void __launch_bounds__(256)
trsm_kernel(T* __restrict__ A, long long lda, int k0, int nb, int c0, int ncols) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // [kNB][kNB] column-major
  T* X = L + kNB * kNB;                   // [kNB][32]: X[r*32 + c]
  const int cb = c0 + blockIdx.x * 32;
  const int nc = min(32, c0 + ncols - cb);
  for (int v = threadIdx.x; v < nb * nb; v += blockDim.x) {
    const int s = v / nb, r = v - s * nb;
    L[s * kNB + r] = A[(size_t)(k0 + s) * lda + k0 + r];
  }
  for (int v = threadIdx.x; v < nb * nc; v += blockDim.x) {
    const int c = v / nb, r = v - c * nb;
    X[r * 32 + c] = A[(size_t)(cb + c) * lda + k0 + r];
  }
  const int c = threadIdx.x & 31, rg = threadIdx.x >> 5;
  for (int s = 0; s < nb; ++s) {
    __syncthreads();
    const T xs = X[s * 32 + c];
    for (int r = s + 1 + rg; r < nb; r += 8) X[r * 32 + c] = cfms(X[r * 32 + c], L[s * kNB + r], xs);
  }
  __syncthreads();
  for (int v = threadIdx.x; v < nb * nc; v += blockDim.x) {
    const int cc = v / nb, r = v - cc * nb;
    A[(size_t)(cb + cc) * lda + k0 + r] = X[r * 32 + cc];
  }
}

// C[M x N] -= A[M x K] B[K x N], K <= kNB, column-major operands.
constexpr int kGB = 64;
template <typename T>
__global__ void __launch_bounds__(256)
gemm_sub_kernel(const T* __restrict__ Am, long long lda, const T* __restrict__ Bm,
                long long ldb, T* __restrict__ C, long long ldc, int M, int N, int K) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);  // [K][kGB]
  T* Bs = As + kNB * kGB;                  // [K][kGB]
  const int m0 = blockIdx.x * kGB, n0 = blockIdx.y * kGB;
  for (int v = threadIdx.x; v < K * kGB; v += blockDim.x) {
    const int k = v / kGB, i = v - k * kGB;
    As[k * kGB + i] = (m0 + i < M) ? Am[(size_t)k * lda + m0 + i] : CTraits<T>::make(0, 0);
  }
  for (int v = threadIdx.x; v < K * kGB; v += blockDim.x) {
    const int j = v / K, k = v - j * K;
    Bs[k * kGB + j] = (n0 + j < N) ? Bm[(size_t)(n0 + j) * ldb + k] : CTraits<T>::make(0, 0);
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = CTraits<T>::make(0, 0);
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    T av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = As[k * kGB + tx + 16 * a];
#pragma unroll
    for (int c = 0; c < 4; ++c) bv[c] = Bs[k * kGB + ty + 16 * c];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = cfma(av[a], bv[c], acc[a][c]);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = n0 + ty + 16 * c;
    if (j >= N) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = m0 + tx + 16 * a;
      if (i < M) {
        T* p = C + (size_t)j * ldc + i;
        T v = *p;
        v.x -= acc[a][c].x;
        v.y -= acc[a][c].y;
        *p = v;
      }
    }
  }
}

template <typename T>
static int panel_blocks(int H) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  // at least 64 rows per block: fewer blocks make the per-column barrier
  // and the pivot agreement cheaper; one block per SM at most
  return std::max(1, std::min(nsm, (H + 63) / 64));
}

template <typename T>
int lu_factor(T* A, long long lda, int n, const LuWork& w, cudaStream_t s,
              long long* launches) {
  const PanelBufs<T> buf = panel_bufs<T>(w.scratch);
  cudaMemsetAsync(w.info, 0, sizeof(int), s);
  cudaMemsetAsync(w.status, 0, sizeof(int), s);
  cudaMemsetAsync(w.barrier, 0, 2 * sizeof(unsigned), s);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(T) * (kNB * kNB + kNB * 32)));
    cudaFuncSetAttribute(gemm_sub_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(T) * 2 * kNB * kGB));
    attr = true;
  }
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = std::min(kNB, n - k0);
    const int H = n - k0;
    int nblk = panel_blocks<T>(H);
    int rpb = (H + nblk - 1) / nblk;
    nblk = (H + rpb - 1) / rpb;
    const size_t smem = sizeof(T) * ((size_t)rpb * kNB + kNB + rpb);
    if (smem > 200 * 1024) return BEM2D_ERR_ARG;
    void* args[] = {(void*)&A, (void*)&lda, (void*)&n, (void*)&k0, (void*)&nb, (void*)&rpb,
                    (void*)&w.ipiv, (void*)&w.info, (void*)&w.status, (void*)&w.barrier,
                    (void*)&buf};
    cudaError_t e = cudaLaunchCooperativeKernel((void*)panel_kernel<T>, dim3(nblk),
                                                dim3(kPanelThreads), args, smem, s);
    if (e != cudaSuccess) return BEM2D_ERR_CUDA;
    ++*launches;
    const int c0 = k0 + nb, nc = n - c0;
    if (nc > 0) {
      laswp_kernel<T><<<(nc + 127) / 128, 128, 0, s>>>(A, lda, c0, nc, w.ipiv, k0, nb);
      trsm_kernel<T><<<(nc + 31) / 32, 256, sizeof(T) * (kNB * kNB + kNB * 32), s>>>(
          A, lda, k0, nb, c0, nc);
      dim3 g((nc + kGB - 1) / kGB, (nc + kGB - 1) / kGB);
      gemm_sub_kernel<T><<<g, 256, sizeof(T) * 2 * kNB * kGB, s>>>(
          A + (size_t)k0 * lda + c0, lda, A + (size_t)c0 * lda + k0, lda,
          A + (size_t)c0 * lda + c0, lda, nc, nc, nb);
      *launches += 3;
    }
  }
  return BEM2D_OK;
}

// ---- triangular solves ----------------------------------------------------
// Forward step of panel k0: swaps of the panel applied to b, then
// y = L11^{-1} b[k0:k0+nb].  The nb x nb diagonal block is staged in shared
// memory first (coalesced), so the sequential sweep reads only smem.
template <typename T>
__global__ void fwd_diag_kernel(const T* __restrict__ LU, long long lda, int k0, int nb,
                                const int* __restrict__ ipiv, T* b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);  // [kNB][kNB]
  T* y = D + kNB * kNB;                   // [kNB]
  for (int v = threadIdx.x; v < nb * nb; v += blockDim.x) {
    const int s = v / nb, r = v - s * nb;
    D[s * kNB + r] = LU[(size_t)(k0 + s) * lda + k0 + r];
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < nb; ++s) {
      const int p = ipiv[k0 + s];
      if (p != k0 + s) {
        const T t = b[k0 + s];
        b[k0 + s] = b[p];
        b[p] = t;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < nb) y[threadIdx.x] = b[k0 + threadIdx.x];
  for (int s = 0; s < nb; ++s) {
    __syncthreads();
    const T ys = y[s];
    const int r = threadIdx.x;
    if (r > s && r < nb) y[r] = cfms(y[r], D[s * kNB + r], ys);
  }
  __syncthreads();
  if (threadIdx.x < nb) b[k0 + threadIdx.x] = y[threadIdx.x];
}

// b[r] -= sum_s LU[r, c0+s] * b[c0+s] for rows r in [r0, r1), s < nb.
template <typename T>
__global__ void gemv_sub_kernel(const T* __restrict__ LU, long long lda, int c0, int nb,
                                int r0, int r1, T* b) {
  __shared__ T y[kNB];
  if (threadIdx.x < nb) y[threadIdx.x] = b[c0 + threadIdx.x];
  __syncthreads();
  const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= r1) return;
  T acc = b[r];
  for (int s = 0; s < nb; ++s) acc = cfms(acc, LU[(size_t)(c0 + s) * lda + r], y[s]);
  b[r] = acc;
}

template <typename T>
__global__ void bwd_diag_kernel(const T* __restrict__ LU, long long lda, int k0, int nb, T* b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);  // [kNB][kNB]
  T* rd = D + kNB * kNB;                  // [kNB]
  T* y = rd + kNB;                        // [kNB]
  for (int v = threadIdx.x; v < nb * nb; v += blockDim.x) {
    const int s = v / nb, r = v - s * nb;
    D[s * kNB + r] = LU[(size_t)(k0 + s) * lda + k0 + r];
  }
  __syncthreads();
  if (threadIdx.x < nb) {
    rd[threadIdx.x] = crcp(D[threadIdx.x * kNB + threadIdx.x]);
    y[threadIdx.x] = b[k0 + threadIdx.x];
  }
  for (int s = nb - 1; s >= 0; --s) {
    __syncthreads();
    const T xs = cmul(y[s], rd[s]);
    const int r = threadIdx.x;
    if (r < s) y[r] = cfms(y[r], D[s * kNB + r], xs);
    __syncthreads();
    if (r == s) y[s] = xs;
  }
  __syncthreads();
  if (threadIdx.x < nb) b[k0 + threadIdx.x] = y[threadIdx.x];
}

template <typename T>
void lu_solve(const T* LU, long long lda, int n, const int* ipiv, T* b, cudaStream_t s,
              long long* launches) {
  const size_t dsm = sizeof(T) * (kNB * kNB + 2 * kNB);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(fwd_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm);
    cudaFuncSetAttribute(bwd_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm);
    attr = true;
  }
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = std::min(kNB, n - k0);
    fwd_diag_kernel<T><<<1, kNB, dsm, s>>>(LU, lda, k0, nb, ipiv, b);
    ++*launches;
    const int r0 = k0 + nb;
    if (r0 < n) {
      gemv_sub_kernel<T><<<(n - r0 + 127) / 128, 128, 0, s>>>(LU, lda, k0, nb, r0, n, b);
      ++*launches;
    }
  }
  const int last = ((n - 1) / kNB) * kNB;
  for (int k0 = last; k0 >= 0; k0 -= kNB) {
    const int nb = std::min(kNB, n - k0);
    bwd_diag_kernel<T><<<1, kNB, dsm, s>>>(LU, lda, k0, nb, b);
    ++*launches;
    if (k0 > 0) {
      gemv_sub_kernel<T><<<(k0 + 127) / 128, 128, 0, s>>>(LU, lda, k0, nb, 0, k0, b);
      ++*launches;
    }
  }
}

template int lu_factor<double2>(double2*, long long, int, const LuWork&, cudaStream_t, long long*);
template int lu_factor<float2>(float2*, long long, int, const LuWork&, cudaStream_t, long long*);
template void lu_solve<double2>(const double2*, long long, int, const int*, double2*, cudaStream_t, long long*);
template void lu_solve<float2>(const float2*, long long, int, const int*, float2*, cudaStream_t, long long*);

// ---- refinement helpers -----------------------------------------------------
// r = b - A x in FP64; column chunks of 256 give partial sums per row.
constexpr int kResChunk = 256;
__global__ void residual_partial_kernel(const double2* __restrict__ A, long long lda, int n,
                                        const double2* __restrict__ x, double2* part) {
  __shared__ double2 xs[kResChunk];
  const int c0 = blockIdx.y * kResChunk;
  const int nc = min(kResChunk, n - c0);
  for (int v = threadIdx.x; v < nc; v += blockDim.x) xs[v] = x[c0 + v];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double2 acc = make_double2(0, 0);
  const double2* col = A + (size_t)c0 * lda + r;
  for (int c = 0; c < nc; ++c) acc = cfma(col[(size_t)c * lda], xs[c], acc);
  part[(size_t)blockIdx.y * n + r] = acc;
}

__global__ void residual_final_kernel(int n, int nchunk, const double2* __restrict__ part,
                                      const double2* __restrict__ b, double2* r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 acc = b[i];
  for (int c = 0; c < nchunk; ++c) {
    const double2 p = part[(size_t)c * n + i];
    acc.x -= p.x;
    acc.y -= p.y;
  }
  r[i] = acc;
}

void launch_residual(const double2* A, long long lda, int n, const double2* x,
                     const double2* b, double2* r, double2* part, cudaStream_t s) {
  const int nchunk = (n + kResChunk - 1) / kResChunk;
  dim3 g((n + 127) / 128, nchunk);
  residual_partial_kernel<<<g, 128, 0, s>>>(A, lda, n, x, part);
  residual_final_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, nchunk, part, b, r);
}

size_t residual_part_bytes(int n) {
  return sizeof(double2) * (size_t)n * ((n + kResChunk - 1) / kResChunk);
}

__global__ void to_c64_kernel(const double2* __restrict__ src, long long lds,
                              float2* __restrict__ dst, long long ldd, int rows, int cols) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (long long)rows * cols) return;
  const int j = (int)(v / rows), i = (int)(v - (long long)j * rows);
  const double2 a = src[(size_t)j * lds + i];
  dst[(size_t)j * ldd + i] = make_float2((float)a.x, (float)a.y);
}

void launch_to_c64(const double2* src, long long lds, float2* dst, long long ldd,
                   int rows, int cols, cudaStream_t s) {
  const long long tot = (long long)rows * cols;
  to_c64_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
}

// dst = (complex64)(src * scale)
__global__ void scale_to_c64_kernel(int n, const double2* __restrict__ src, double scale,
                                    float2* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = make_float2((float)(src[i].x * scale), (float)(src[i].y * scale));
}
// x += scale * d
__global__ void axpy_c64_kernel(int n, double scale, const float2* __restrict__ d,
                                double2* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i].x = fma(scale, (double)d[i].x, x[i].x);
    x[i].y = fma(scale, (double)d[i].y, x[i].y);
  }
}

void launch_scale_to_c64(int n, const double2* src, double scale, float2* dst, cudaStream_t s) {
  scale_to_c64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, src, scale, dst);
}
void launch_axpy_c64(int n, double scale, const float2* d, double2* x, cudaStream_t s) {
  axpy_c64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, scale, d, x);
}

// Sum of |a_ij|^2 over a rows x cols column-major block: per-block partial
// sums, then one block adds them (deterministic order).
__global__ void sumsq_partial_kernel(const double2* __restrict__ A, long long ld, int rows,
                                     int cols, double* part) {
  __shared__ double red[256];
  double acc = 0.0;
  const long long tot = (long long)rows * cols;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < tot;
       v += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(v / rows), i = (int)(v - (long long)j * rows);
    const double2 a = A[(size_t)j * ld + i];
    acc = fma(a.x, a.x, fma(a.y, a.y, acc));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_kernel(int n, const double* __restrict__ part, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

constexpr int kSumsqBlocks = 304;
void launch_sumsq(const double2* A, long long ld, int rows, int cols, double* part,
                  double* out, cudaStream_t s) {
  sumsq_partial_kernel<<<kSumsqBlocks, 256, 0, s>>>(A, ld, rows, cols, part);
  sum_kernel<<<1, 256, 0, s>>>(kSumsqBlocks, part, out);
}
size_t sumsq_part_bytes() { return sizeof(double) * kSumsqBlocks; }

}  // namespace bem2d_gpu
