// Blocked right-looking LU with partial pivoting and the triangular solves,
// for complex128 (double2) and complex64 (float2).  Replaces LAPACK zgetrf +
// zgetrs as called by SolveSystem (lib/bem2d_mathroutines.cpp:323-351).
//
// Per panel of NB = 64 columns:
//   panel_cluster_kernel  one thread-block cluster (up to 16 CTAs) holds the
//                  panel rows in distributed shared memory; per column each CTA
//                  writes its pivot candidate (value, row, panel row) to its own
//                  shared memory, one cluster barrier, then every CTA reads the
//                  candidates over DSMEM, agrees on the pivot, swaps and
//                  updates.  Used while the panel fits in the cluster's smem.
//   panel_kernel   the same exchange through global-memory slots with
//                  sequence flags (bounded waits) across a cooperative grid,
//                  for taller panels.
//   laswp_kernel   the panel's row swaps on all other columns (LAPACK order)
//   trsm_kernel    U12 = L11^{-1} A12
//   gemm_kernel    A22 -= L21 U12  (register-tiled, 64 x 64 CTA tiles)
// After the factorisation: perm (the row permutation of the pivots) and the
// inverses of the 64 x 64 diagonal blocks of L and U, so that a solve is a
// chain of small matrix-vector products (trisolve_cluster_kernel).
#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#include <algorithm>
#include <atomic>
#include <climits>
#include <mutex>

#include "common.cuh"
#include "cplx.cuh"

namespace bem2d_gpu {

constexpr int kNB = 64;              // panel width
constexpr int kPanelThreads = 256;
constexpr unsigned kSpinLimit = 1u << 25;  // polls of >= 32 ns: > 1 s

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

// Panel exchange slots in global memory, two per block (column parity):
// {seq, row index, |pivot| value, the block's candidate panel row}, plus a
// slot for the current row kc from its owner.  A slot is valid for column kc
// when its seq equals kc + 1; the slots are zeroed before each factorisation.
constexpr int kMaxPanelBlocks = 1024;
constexpr int kSlotHead = 16;  // int seq, int idx, 8-byte value

template <typename T>
struct PanelSlots {
  char* base;
  __device__ __forceinline__ char* slot(int par, int b) const {
    return base + ((size_t)par * (kMaxPanelBlocks + 1) + b) * (kSlotHead + sizeof(T) * kNB);
  }
  __device__ __forceinline__ char* krow(int par) const { return slot(par, kMaxPanelBlocks); }
};

size_t lu_scratch_bytes(int) {
  return (size_t)2 * (kMaxPanelBlocks + 1) * (kSlotHead + sizeof(double2) * kNB) + 256;
}

static size_t slots_bytes(size_t elem) {
  return (size_t)2 * (kMaxPanelBlocks + 1) * (kSlotHead + elem * kNB);
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait (bounded) until *seq == want (acquire); returns false on timeout.
// Spins without sleeping first: the expected wait is one L2 round trip.
__device__ __forceinline__ bool wait_seq(const int* seq, int want, int* status) {
  unsigned it = 0;
  while (ld_acquire(seq) != want) {
    if (++it > kSpinLimit || (it > 1024 && *(volatile int*)status != 0)) {
      atomicExch(status, 1);
      return false;
    }
    if (it > 256) __nanosleep(32);
  }
  return true;
}

// Publish `epoch` at *flag after every thread of the block has written its
// data: bar.sync orders the block's writes before thread 0's release store.
__device__ __forceinline__ void block_publish(int* flag, int epoch) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(flag, epoch);
  }
}

template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_kernel(T* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
             int* __restrict__ ipiv, int* info, int* status, PanelSlots<T> sl) {
  typedef typename CTraits<T>::R R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // [rpb][kNB] block's panel rows
  T* prow = P + (size_t)rpb * kNB;        // [kNB] pivot row
  T* lcol = prow + kNB;                   // [rpb] multipliers
  __shared__ int s_p, s_bw, s_ok;
  __shared__ R s_pv;

  const int nblk = gridDim.x, b = blockIdx.x;
  const int r0 = k0 + b * rpb;
  const int r1 = min(r0 + rpb, n);
  const int nr = max(r1 - r0, 0);
  for (int v = threadIdx.x; v < nr * nb; v += blockDim.x) {
    const int c = v / nr, lr = v - c * nr;
    P[lr * kNB + c] = A[(size_t)(k0 + c) * lda + r0 + lr];
  }
  if (threadIdx.x == 0) s_ok = 1;
  __syncthreads();

  for (int c = 0; c < nb; ++c) {
    const int kc = k0 + c, par = kc & 1, epoch = kc + 1;
    // (a) local pivot candidate among rows >= kc
    R best = -1;
    int bidx = INT_MAX;
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const int gr = r0 + lr;
      if (gr < kc) continue;
      argmax_merge(best, bidx, cabs1(P[lr * kNB + c]), gr);
    }
    block_argmax(best, bidx);
    // (b) publish the candidate (and row kc from its owner), then the seq
    char* my = sl.slot(par, b);
    T* myrow = reinterpret_cast<T*>(my + kSlotHead);
    if (bidx != INT_MAX)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) myrow[j] = P[(bidx - r0) * kNB + j];
    const bool own_k = kc >= r0 && kc < r1;
    char* kr = sl.krow(par);
    if (own_k)
      for (int j = threadIdx.x; j < nb; j += blockDim.x)
        reinterpret_cast<T*>(kr + kSlotHead)[j] = P[(kc - r0) * kNB + j];
    if (threadIdx.x == 0) {
      reinterpret_cast<int*>(my)[1] = bidx;
      *reinterpret_cast<R*>(my + 8) = best;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_release(reinterpret_cast<int*>(my), epoch);
      if (own_k) st_release(reinterpret_cast<int*>(kr), epoch);
    }
    // (c) wait for every block's candidate, agree on the pivot
    R v = -1;
    int i = INT_MAX;
    if ((int)threadIdx.x < nblk) {
      const char* q = sl.slot(par, threadIdx.x);
      if (!wait_seq(reinterpret_cast<const int*>(q), epoch, status)) {
        s_ok = 0;
      } else {
        i = __ldcg(reinterpret_cast<const int*>(q) + 1);
        v = __ldcg(reinterpret_cast<const R*>(q + 8));
      }
    }
    block_argmax(v, i);  // contains __syncthreads: s_ok visible after it
    if (!s_ok) return;
    if (threadIdx.x == 0) {
      // no finite candidate (all NaN): treat as a zero pivot at row kc
      if (i == INT_MAX || i < kc || i >= n) {
        i = kc;
        v = 0;
      }
      s_p = i;
      s_bw = (i - k0) / rpb;  // the owner block of row i published it
      s_pv = v;
    }
    __syncthreads();
    const int p = s_p, bw = s_bw;
    const bool zero = !(s_pv > 0);
    const T* wrow = reinterpret_cast<const T*>(sl.slot(par, bw) + kSlotHead);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) prow[j] = __ldcg(&wrow[j]);
    if (b == 0 && threadIdx.x == 0) {
      ipiv[kc] = p;
      if (zero && *info == 0) *info = kc + 1;
    }
    if (!zero && p != kc && p >= r0 && p < r1) {
      if (threadIdx.x == 0 && !wait_seq(reinterpret_cast<const int*>(kr), epoch, status))
        s_ok = 0;
      __syncthreads();
      if (!s_ok) return;
      for (int j = threadIdx.x; j < nb; j += blockDim.x)
        P[(p - r0) * kNB + j] = __ldcg(reinterpret_cast<const T*>(kr + kSlotHead) + j);
    }
    __syncthreads();
    if (!zero && p != kc && own_k)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) P[(kc - r0) * kNB + j] = prow[j];
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
        for (int u = threadIdx.x; u < nr * w; u += blockDim.x) {
          const int lr = u / w, cc = c + 1 + (u - lr * w);
          if (r0 + lr > kc) P[lr * kNB + cc] = cfms(P[lr * kNB + cc], lcol[lr], prow[cc]);
        }
      }
    }
    __syncthreads();
  }
  for (int v2 = threadIdx.x; v2 < nr * nb; v2 += blockDim.x) {
    const int c = v2 / nr, lr = v2 - c * nr;
    A[(size_t)(k0 + c) * lda + r0 + lr] = P[lr * kNB + c];
  }
}

// Row swaps of panel [k0, k0+nb) on every column outside it.
template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, long long lda, int n,
                             const int* __restrict__ ipiv, int k0, int nb) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n - nb) return;
  const int j = v < k0 ? v : v + nb;
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
  static const int nsm = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return std::max(v, 1);
  }();
  // at least 64 rows per block: fewer blocks make the per-column barrier
  // and the pivot agreement cheaper; one block per SM at most
  return std::max(1, std::min(nsm, (H + 63) / 64));
}

// ---- cluster panel ---------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_cluster_kernel(T* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
                     int* __restrict__ ipiv, int* info) {
  typedef typename CTraits<T>::R R;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // [rpb][kNB]
  T* prow = P + (size_t)rpb * kNB;        // [kNB]
  T* lcol = prow + kNB;                   // [rpb]
  T* crow = lcol + rpb;                   // [2][kNB] candidate row per parity
  T* krow = crow + 2 * kNB;               // [2][kNB] row kc per parity (owner)
  __shared__ R cval[2];
  __shared__ int cidx[2];
  __shared__ int s_p, s_bw;
  __shared__ R s_pv;
  const int r0 = k0 + rank * rpb;
  const int r1 = min(r0 + rpb, n);
  const int nr = max(r1 - r0, 0);
  for (int v = threadIdx.x; v < nr * nb; v += blockDim.x) {
    const int c = v / nr, lr = v - c * nr;
    P[lr * kNB + c] = A[(size_t)(k0 + c) * lda + r0 + lr];
  }
  cl.sync();  // every CTA of the cluster is running before any DSMEM access
  for (int c = 0; c < nb; ++c) {
    const int kc = k0 + c, par = c & 1;
    R best = -1;
    int bidx = INT_MAX;
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const int gr = r0 + lr;
      if (gr < kc) continue;
      argmax_merge(best, bidx, cabs1(P[lr * kNB + c]), gr);
    }
    block_argmax(best, bidx);
    if (threadIdx.x == 0) {
      cval[par] = best;
      cidx[par] = bidx;
    }
    if (bidx != INT_MAX)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) crow[par * kNB + j] = P[(bidx - r0) * kNB + j];
    const bool own_k = kc >= r0 && kc < r1;
    if (own_k)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) krow[par * kNB + j] = P[(kc - r0) * kNB + j];
    cl.sync();
    if (threadIdx.x < 32) {
      R v = -1;
      int i = INT_MAX;
      for (int q = threadIdx.x; q < C; q += 32) {
        argmax_merge(v, i, *cl.map_shared_rank(&cval[par], q), *cl.map_shared_rank(&cidx[par], q));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        argmax_merge(v, i, v2, i2);
      }
      if (threadIdx.x == 0) {
        if (i == INT_MAX || i < kc || i >= n) {
          i = kc;
          v = 0;
        }
        s_p = i;
        s_bw = (i - k0) / rpb;
        s_pv = v;
      }
    }
    __syncthreads();
    const int p = s_p, bw = s_bw;
    const bool zero = !(s_pv > 0);
    const T* wrow = cl.map_shared_rank(crow, bw) + par * kNB;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) prow[j] = wrow[j];
    if (rank == 0 && threadIdx.x == 0) {
      ipiv[kc] = p;
      if (zero && *info == 0) *info = kc + 1;
    }
    if (!zero && p != kc && p >= r0 && p < r1) {
      const T* kr = cl.map_shared_rank(krow, (kc - k0) / rpb) + par * kNB;
      for (int j = threadIdx.x; j < nb; j += blockDim.x) P[(p - r0) * kNB + j] = kr[j];
    }
    __syncthreads();
    if (!zero && p != kc && own_k)
      for (int j = threadIdx.x; j < nb; j += blockDim.x) P[(kc - r0) * kNB + j] = prow[j];
    __syncthreads();
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
        for (int u = threadIdx.x; u < nr * w; u += blockDim.x) {
          const int lr = u / w, cc = c + 1 + (u - lr * w);
          if (r0 + lr > kc) P[lr * kNB + cc] = cfms(P[lr * kNB + cc], lcol[lr], prow[cc]);
        }
      }
    }
    __syncthreads();
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
  for (int v = threadIdx.x; v < nr * nb; v += blockDim.x) {
    const int c = v / nr, lr = v - c * nr;
    A[(size_t)(k0 + c) * lda + r0 + lr] = P[lr * kNB + c];
  }
}

template <typename K, typename... Args>
static cudaError_t launch_cluster(K kern, int C, int threads, size_t smem, cudaStream_t s,
                                  Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

constexpr int kMaxCluster = 16;
constexpr size_t kClusterSmem = 200 * 1024;

template <typename T>
static size_t panel_cluster_smem(int rpb) {
  return sizeof(T) * ((size_t)rpb * kNB + kNB + rpb + 4 * kNB);
}

// Row permutation of the pivots: perm[i] = the original row that ends at i.
__global__ void perm_kernel(int n, const int* __restrict__ ipiv, int* __restrict__ perm) {
  extern __shared__ int sp[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      const int p = ipiv[i];
      const int t = sp[i];
      sp[i] = sp[p];
      sp[p] = t;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

// Inverses of the diagonal blocks: dinv[(2 k) * 64 * 64 ...] = L_kk^{-1}
// (unit lower), dinv[(2 k + 1) * 64 * 64 ...] = U_kk^{-1}; column-major 64 x 64.
template <typename T>
__global__ void __launch_bounds__(128) dinv_kernel(const T* __restrict__ LU, long long lda, int n,
                                                   T* __restrict__ dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);  // [kNB][kNB] column-major
  const int k0 = blockIdx.x * kNB, nb = min(kNB, n - k0);
  for (int v = threadIdx.x; v < nb * nb; v += blockDim.x) {
    const int c = v / nb, r = v - c * nb;
    D[c * kNB + r] = LU[(size_t)(k0 + c) * lda + k0 + r];
  }
  __syncthreads();
  T* Li = dinv + (size_t)(2 * blockIdx.x) * kNB * kNB;
  T* Ui = Li + kNB * kNB;
  const T zero = CTraits<T>::make(0, 0), one = CTraits<T>::make(1, 0);
  const int j = threadIdx.x & 63;
  // thread j builds column j of one inverse in place in global memory (its
  // own column only, so the reads back hit L1)
  if (threadIdx.x < 64) {
    // L^{-1}: x_j = 1, x_i = -sum_{m=j}^{i-1} L_im x_m
    T* x = Li + j * kNB;
    for (int i = 0; i < kNB; ++i) x[i] = (i == j && j < nb) ? one : zero;
    if (j < nb) {
      for (int i = j + 1; i < nb; ++i) {
        T acc = zero;
        for (int m = j; m < i; ++m) acc = cfma(D[m * kNB + i], x[m], acc);
        x[i] = CTraits<T>::make(-acc.x, -acc.y);
      }
    }
  } else {
    // U^{-1}: x_j = 1/U_jj, x_i = -(sum_{m=i+1}^{j} U_im x_m) / U_ii
    T* x = Ui + j * kNB;
    for (int i = 0; i < kNB; ++i) x[i] = zero;
    if (j < nb) {
      x[j] = crcp(D[j * kNB + j]);
      for (int i = j - 1; i >= 0; --i) {
        T acc = zero;
        for (int m = i + 1; m <= j; ++m) acc = cfma(D[m * kNB + i], x[m], acc);
        const T q = cmul(acc, crcp(D[i * kNB + i]));
        x[i] = CTraits<T>::make(-q.x, -q.y);
      }
    }
  }
}

size_t lu_aux_bytes(int n, size_t elem) {
  const size_t nk = (n + kNB - 1) / kNB;
  return sizeof(int) * (size_t)n + 2 * nk * kNB * kNB * elem + 256;
}

template <typename T>
int lu_factor(T* A, long long lda, int n, const LuWork& w, cudaStream_t s,
              long long* launches) {
  PanelSlots<T> sl;
  sl.base = static_cast<char*>(w.scratch);
  cudaMemsetAsync(w.info, 0, sizeof(int), s);
  cudaMemsetAsync(w.status, 0, sizeof(int), s);
  cudaMemsetAsync(sl.base, 0, slots_bytes(sizeof(T)), s);
  // one-time function attributes; thread-safe (workers of a sweep factor
  // concurrently from several host threads)
  static std::atomic<bool> cluster16{true};
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(panel_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kClusterSmem);
    if (cudaFuncSetAttribute(panel_cluster_kernel<T>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      cluster16 = false;
    }
    cudaFuncSetAttribute(trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(T) * (kNB * kNB + kNB * 32)));
    cudaFuncSetAttribute(gemm_sub_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(T) * 2 * kNB * kGB));
    cudaFuncSetAttribute(dinv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(T) * kNB * kNB));
    cudaFuncSetAttribute(perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = std::min(kNB, n - k0);
    const int H = n - k0;
    // cluster panel: 64 rows or more per CTA, at most 16 (8 portable) CTAs
    bool done = false;
    for (int cmax : {cluster16 ? kMaxCluster : 8, 8}) {
      const int C = std::max(1, std::min(cmax, (H + 63) / 64));
      const int rpb = (H + C - 1) / C;
      const size_t smem = panel_cluster_smem<T>(rpb);
      if (smem > kClusterSmem) continue;
      cudaError_t e = launch_cluster(panel_cluster_kernel<T>, C, kPanelThreads, smem, s, A, lda,
                                     n, k0, nb, rpb, w.ipiv, w.info);
      if (e == cudaSuccess) {
        done = true;
        break;
      }
      cudaGetLastError();
      if (cmax > 8) cluster16 = false;
    }
    if (!done) {
      int nblk = panel_blocks<T>(H);
      int rpb = (H + nblk - 1) / nblk;
      nblk = (H + rpb - 1) / rpb;
      const size_t smem = sizeof(T) * ((size_t)rpb * kNB + kNB + rpb);
      if (smem > 200 * 1024) return BEM2D_ERR_ARG;
      void* args[] = {(void*)&A, (void*)&lda, (void*)&n, (void*)&k0, (void*)&nb, (void*)&rpb,
                      (void*)&w.ipiv, (void*)&w.info, (void*)&w.status, (void*)&sl};
      cudaError_t e = cudaLaunchCooperativeKernel((void*)panel_kernel<T>, dim3(nblk),
                                                  dim3(kPanelThreads), args, smem, s);
      if (e != cudaSuccess) return BEM2D_ERR_CUDA;
    }
    ++*launches;
    if (n > nb) {
      laswp_kernel<T><<<(n - nb + 127) / 128, 128, 0, s>>>(A, lda, n, w.ipiv, k0, nb);
      ++*launches;
    }
    const int c0 = k0 + nb, nc = n - c0;
    if (nc > 0) {
      trsm_kernel<T><<<(nc + 31) / 32, 256, sizeof(T) * (kNB * kNB + kNB * 32), s>>>(
          A, lda, k0, nb, c0, nc);
      dim3 g((nc + kGB - 1) / kGB, (nc + kGB - 1) / kGB);
      gemm_sub_kernel<T><<<g, 256, sizeof(T) * 2 * kNB * kGB, s>>>(
          A + (size_t)k0 * lda + c0, lda, A + (size_t)c0 * lda + k0, lda,
          A + (size_t)c0 * lda + c0, lda, nc, nc, nb);
      *launches += 2;
    }
  }
  // solve aids: permutation and diagonal-block inverses
  const int nk = (n + kNB - 1) / kNB;
  perm_kernel<<<1, 1024, sizeof(int) * n, s>>>(n, w.ipiv, w.perm);
  dinv_kernel<T><<<nk, 128, sizeof(T) * kNB * kNB, s>>>(A, lda, n, reinterpret_cast<T*>(w.dinv));
  *launches += 2;
  return BEM2D_OK;
}

// ---- triangular solves ----------------------------------------------------
// x = U^{-1} L^{-1} P b in one cluster launch.  CTA r owns rows
// [r rpb, (r+1) rpb) of b in shared memory (rpb a multiple of 64).  Step k of
// the forward sweep: the owner of block k forms y_k = L_kk^{-1} b_k from the
// stored inverse; one cluster barrier; every CTA reads y_k over DSMEM and
// updates its rows below the block.  The backward sweep is the mirror with
// U_kk^{-1}.  One cluster barrier per block step.
template <typename T>
__global__ void __launch_bounds__(256)
trisolve_cluster_kernel(const T* __restrict__ LU, long long lda, int n,
                        const int* __restrict__ perm, const T* __restrict__ dinv,
                        const T* __restrict__ bin, T* __restrict__ xout, int rpb) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bc = reinterpret_cast<T*>(smem_raw);  // [rpb] this CTA's rows of b
  T* ys = bc + rpb;                         // [kNB] the current block solution
  T* ps = ys + kNB;                         // [4][max(rpb, kNB)] partial sums
  const int r0 = rank * rpb, r1 = min(n, r0 + rpb), nr = max(r1 - r0, 0);
  for (int i = threadIdx.x; i < nr; i += blockDim.x) bc[i] = bin[perm[r0 + i]];
  const int nk = (n + kNB - 1) / kNB;
  cl.sync();
  for (int step = 0; step < 2 * nk; ++step) {
    const bool fwd = step < nk;
    const int kb = fwd ? step : 2 * nk - 1 - step;
    const int k0 = kb * kNB, nb = min(kNB, n - k0);
    const int owner = k0 / rpb;
    if (rank == owner) {
      // y = D_k^{-1} b_k: four column groups of 16 per row, partial sums in ps
      const T* Di = dinv + (size_t)(2 * kb + (fwd ? 0 : 1)) * kNB * kNB;
      const T* bk = bc + (k0 - r0);
      const int r = threadIdx.x & 63, g = threadIdx.x >> 6;
      T acc = CTraits<T>::make(0, 0);
      if (r < nb) {
        T l[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) l[u] = Di[(g * 16 + u) * kNB + r];
#pragma unroll
        for (int u = 0; u < 16; ++u)
          if (g * 16 + u < nb) acc = cfma(l[u], bk[g * 16 + u], acc);
      }
      ps[g * kNB + r] = acc;
      __syncthreads();
      if ((int)threadIdx.x < nb) {
        const int t = threadIdx.x;
        T v = ps[t];
        v.x += ps[kNB + t].x + ps[2 * kNB + t].x + ps[3 * kNB + t].x;
        v.y += ps[kNB + t].y + ps[2 * kNB + t].y + ps[3 * kNB + t].y;
        bc[k0 - r0 + t] = v;
      }
    }
    cl.sync();
    const T* yk = cl.map_shared_rank(bc, owner) + (k0 - owner * rpb);
    if ((int)threadIdx.x < nb) ys[threadIdx.x] = yk[threadIdx.x];
    __syncthreads();
    // rows below (forward) / above (backward) the block: work items
    // (row, group of 16 columns), 16 independent loads in flight per item
    const int lo = fwd ? max(r0, k0 + nb) : r0;
    const int hi = fwd ? r1 : min(r1, k0);
    const int nrows = max(hi - lo, 0);
    for (int it = threadIdx.x; it < 4 * nrows; it += blockDim.x) {
      const int g = it / nrows, r = lo + (it - g * nrows);
      const T* col = LU + (size_t)(k0 + g * 16) * lda + r;
      T l[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        l[u] = (g * 16 + u < nb) ? col[(size_t)u * lda] : CTraits<T>::make(0, 0);
      T acc = CTraits<T>::make(0, 0);
#pragma unroll
      for (int u = 0; u < 16; ++u) acc = cfma(l[u], ys[(g * 16 + u) & (kNB - 1)], acc);
      ps[g * rpb + (r - r0)] = acc;
    }
    __syncthreads();
    for (int r = lo + threadIdx.x; r < hi; r += blockDim.x) {
      const int i = r - r0;
      T v = bc[i];
      v.x -= ps[i].x + ps[rpb + i].x + ps[2 * rpb + i].x + ps[3 * rpb + i].x;
      v.y -= ps[i].y + ps[rpb + i].y + ps[2 * rpb + i].y + ps[3 * rpb + i].y;
      bc[i] = v;
    }
    __syncthreads();
  }
  cl.sync();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) xout[r0 + i] = bc[i];
}

template <typename T>
int lu_solve(const T* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
             cudaStream_t s, long long* launches) {
  static std::atomic<int> cmax{kMaxCluster};
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(trisolve_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kClusterSmem);
    if (cudaFuncSetAttribute(trisolve_cluster_kernel<T>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      cmax = 8;
    }
  });
  for (;;) {
    const int nk = (n + kNB - 1) / kNB;
    const int C = std::max(1, std::min(cmax.load(), nk));
    const int rpb = ((nk + C - 1) / C) * kNB;
    const size_t smem = sizeof(T) * ((size_t)rpb + kNB + 4 * (size_t)std::max(rpb, kNB));
    if (smem > kClusterSmem) return BEM2D_ERR_ARG;
    cudaError_t e = launch_cluster(trisolve_cluster_kernel<T>, C, 256, smem, s, LU, lda, n,
                                   (const int*)w.perm, (const T*)w.dinv, b, x, rpb);
    if (e == cudaSuccess) break;
    cudaGetLastError();
    if (cmax == 8) return BEM2D_ERR_CUDA;
    cmax = 8;
  }
  ++*launches;
  return BEM2D_OK;
}

// x = A^{-H} b = P^T L^{-H} U^{-H} b in one cluster launch.  Forward sweep
// with U^H (lower), backward with L^H (upper, unit diagonal).  Per step
// every CTA forms the partial sums sum_r conj(M[r, k0+c]) x_r over its own,
// already final rows; one cluster barrier; the owner of block k adds the
// partials over DSMEM and applies the conjugate transpose of the stored
// diagonal-block inverse.  Partial buffers alternate by step parity.
template <typename T>
__global__ void __launch_bounds__(256)
trisolve_h_cluster_kernel(const T* __restrict__ LU, long long lda, int n,
                          const int* __restrict__ perm, const T* __restrict__ dinv,
                          const T* __restrict__ bin, T* __restrict__ xout, int rpb) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bc = reinterpret_cast<T*>(smem_raw);  // [rpb]
  T* part = bc + rpb;                       // [2][kNB]
  T* v = part + 2 * kNB;                    // [kNB]
  const int r0 = rank * rpb, r1 = min(n, r0 + rpb), nr = max(r1 - r0, 0);
  for (int i = threadIdx.x; i < nr; i += blockDim.x) bc[i] = bin[r0 + i];
  const int nk = (n + kNB - 1) / kNB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  cl.sync();
  for (int step = 0; step < 2 * nk; ++step) {
    const bool fwd = step < nk;
    const int kb = fwd ? step : 2 * nk - 1 - step;
    const int k0 = kb * kNB, nb = min(kNB, n - k0), par = step & 1;
    const int lo = fwd ? r0 : max(r0, k0 + nb);
    const int hi = fwd ? min(r1, k0) : r1;
    for (int c = warp * 8; c < warp * 8 + 8; ++c) {
      double sr = 0, si = 0;
      if (c < nb) {
        const T* col = LU + (size_t)(k0 + c) * lda;
        for (int r = lo + lane; r < hi; r += 32) {
          const T a = col[r], b = bc[r - r0];
          sr += (double)a.x * b.x + (double)a.y * b.y;
          si += (double)a.x * b.y - (double)a.y * b.x;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
      }
      if (lane == 0) part[par * kNB + c] = CTraits<T>::make(sr, si);
    }
    cl.sync();
    const int owner = k0 / rpb;
    if (rank == owner) {
      const int t = threadIdx.x;
      if (t < nb) {
        T acc = bc[k0 - r0 + t];
        for (int q = 0; q < C; ++q) {
          const T pq = cl.map_shared_rank(part, q)[par * kNB + t];
          acc.x -= pq.x;
          acc.y -= pq.y;
        }
        v[t] = acc;
      }
      __syncthreads();
      // x_k = D^{-H} v with D^{-1} = (U or L)_kk^{-1} stored column-major
      const T* Di = dinv + (size_t)(2 * kb + (fwd ? 1 : 0)) * kNB * kNB;
      if (t < nb) {
        T acc = CTraits<T>::make(0, 0);
        for (int m = 0; m < nb; ++m) {
          const T d = Di[t * kNB + m];  // D^{-1}[m, t]
          // conj(d) * v[m]
          acc.x += d.x * v[m].x + d.y * v[m].y;
          acc.y += d.x * v[m].y - d.y * v[m].x;
        }
        bc[k0 - r0 + t] = acc;
      }
      __syncthreads();
    }
  }
  cl.sync();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) xout[perm[r0 + i]] = bc[i];
}

template <typename T>
int lu_solve_h(const T* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
               cudaStream_t s, long long* launches) {
  static std::atomic<int> cmax{kMaxCluster};
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(trisolve_h_cluster_kernel<T>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmem);
    if (cudaFuncSetAttribute(trisolve_h_cluster_kernel<T>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      cmax = 8;
    }
  });
  if (b == x) return BEM2D_ERR_ARG;  // the scatter at the end needs distinct buffers
  for (;;) {
    const int nk = (n + kNB - 1) / kNB;
    const int C = std::max(1, std::min(cmax.load(), nk));
    const int rpb = ((nk + C - 1) / C) * kNB;
    const size_t smem = sizeof(T) * ((size_t)rpb + 3 * kNB);
    if (smem > kClusterSmem) return BEM2D_ERR_ARG;
    cudaError_t e = launch_cluster(trisolve_h_cluster_kernel<T>, C, 256, smem, s, LU, lda, n,
                                   (const int*)w.perm, (const T*)w.dinv, b, x, rpb);
    if (e == cudaSuccess) break;
    cudaGetLastError();
    if (cmax == 8) return BEM2D_ERR_CUDA;
    cmax = 8;
  }
  ++*launches;
  return BEM2D_OK;
}

template int lu_solve_h<double2>(const double2*, long long, int, const LuWork&, const double2*,
                                 double2*, cudaStream_t, long long*);
template int lu_solve_h<float2>(const float2*, long long, int, const LuWork&, const float2*,
                                float2*, cudaStream_t, long long*);

template int lu_factor<double2>(double2*, long long, int, const LuWork&, cudaStream_t, long long*);
template int lu_factor<float2>(float2*, long long, int, const LuWork&, cudaStream_t, long long*);
template int lu_solve<double2>(const double2*, long long, int, const LuWork&, const double2*,
                               double2*, cudaStream_t, long long*);
template int lu_solve<float2>(const float2*, long long, int, const LuWork&, const float2*, float2*,
                              cudaStream_t, long long*);

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
