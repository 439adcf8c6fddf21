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

// Wait (bounded: `limit` polls) until *seq == want (acquire); returns false
// on timeout.  Spins without sleeping first: the expected wait is one L2
// round trip.
__device__ __forceinline__ bool wait_seq(const int* seq, int want, int* status,
                                         unsigned limit = kSpinLimit) {
  unsigned it = 0;
  while (ld_acquire(seq) != want) {
    if (++it > limit || (it > 1024 && *(volatile int*)status != 0)) {
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
             int* __restrict__ ipiv, int* info, int* status, PanelSlots<T> sl, int nwait,
             unsigned spin) {
  typedef typename CTraits<T>::R R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // [rpb][kNB] block's panel rows
  T* prow = P + (size_t)rpb * kNB;        // [kNB] pivot row
  T* lcol = prow + kNB;                   // [rpb] multipliers
  __shared__ int s_p, s_bw, s_ok;
  __shared__ R s_pv;

  const int b = blockIdx.x;
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
    // (c) wait for every block's candidate (nwait = the grid size; a larger
    // value waits for slots nobody posts: the timeout check), agree on the
    // pivot
    R v = -1;
    int i = INT_MAX;
    if ((int)threadIdx.x < nwait) {
      const char* q = sl.slot(par, threadIdx.x);
      if (!wait_seq(reinterpret_cast<const int*>(q), epoch, status, spin)) {
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
      if (threadIdx.x == 0 && !wait_seq(reinterpret_cast<const int*>(kr), epoch, status, spin))
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

// Row swaps ipiv[k0 .. k0 + np) (LAPACK order) on columns [c0, c1).
template <typename T>
__global__ void laswp_cols_kernel(T* __restrict__ A, long long lda, const int* __restrict__ ipiv,
                                  int k0, int np, int c0, int c1) {
  const int j = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c1) return;
  T* col = A + (size_t)j * lda;
  for (int s = 0; s < np; ++s) {
    const int p = ipiv[k0 + s];
    if (p != k0 + s) {
      const T t = col[k0 + s];
      col[k0 + s] = col[p];
      col[p] = t;
    }
  }
}
template <typename T>
static void laswp_cols(T* A, long long lda, const int* ipiv, int k0, int np, int c0, int c1,
                       cudaStream_t s, long long* launches) {
  if (c1 <= c0 || np <= 0) return;
  laswp_cols_kernel<T><<<(c1 - c0 + 127) / 128, 128, 0, s>>>(A, lda, ipiv, k0, np, c0, c1);
  ++*launches;
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
  // U12 = L11^{-1} A12 for 32 columns per CTA, by blocks of 8 rows: warp w
  // holds rows 8w..8w+7 of its lane's column in registers; block b is
  // solved by warp b alone (8 steps in registers), then one __syncthreads
  // and every warp below subtracts L[w-block, b-block] x_b: 8 barriers
  // instead of one per row.
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // [kNB][kNB] column-major
  T* X = L + kNB * kNB;                   // [kNB][32]: X[r*32 + c]
  const T zero = CTraits<T>::make(0, 0);
  const int cb = c0 + blockIdx.x * 32;
  const int nc = min(32, c0 + ncols - cb);
  for (int v = threadIdx.x; v < kNB * kNB; v += blockDim.x) {
    const int s = v >> 6, r = v & 63;
    L[s * kNB + r] = (s < nb && r < nb) ? A[(size_t)(k0 + s) * lda + k0 + r] : zero;
  }
  for (int v = threadIdx.x; v < kNB * 32; v += blockDim.x) {
    const int c = v >> 6, r = v & 63;
    X[r * 32 + c] = (c < nc && r < nb) ? A[(size_t)(cb + c) * lda + k0 + r] : zero;
  }
  __syncthreads();
  const int c = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = X[(8 * w + i) * 32 + c];
  const int nbk = (nb + 7) >> 3;
  for (int b = 0; b < nbk; ++b) {
    if (w == b) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = i + 1; j < 8; ++j) x[j] = cfms(x[j], L[(8 * b + i) * kNB + 8 * b + j], x[i]);
#pragma unroll
      for (int i = 0; i < 8; ++i) X[(8 * b + i) * 32 + c] = x[i];
    }
    __syncthreads();
    if (w > b) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const T xb = X[(8 * b + j) * 32 + c];
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = cfms(x[i], L[(8 * b + j) * kNB + 8 * w + i], xb);
      }
    }
  }
  __syncthreads();
  for (int v = threadIdx.x; v < nb * nc; v += blockDim.x) {
    const int cc = v / nb, r = v - cc * nb;
    A[(size_t)(cb + cc) * lda + k0 + r] = X[r * 32 + cc];
  }
}

// C[M x N] -= A[M x K] B[K x N], K <= kNB, column-major operands.
constexpr int kGB = 64;
constexpr int kTensorMinN = 256;  // update size from which complex64 uses tcgen05
constexpr int kOuterNB = 256;     // outer block width of the complex64 LU
constexpr int kOuterMinN = 8192;  // smaller matrices: the extra launches cost more
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
// The panel's H rows are split over the C CTAs of one cluster (rpb rows
// each, at most kPanelRPT per thread) and held column-major in shared
// memory; thread t owns rows t, t + 256, ... and is the only thread that
// touches them, so the per-column update needs no intra-CTA barrier.
// Candidates are pushed, not pulled: per column
//   1. each thread: arg-max |re|+|im| over its rows >= kc, warp shuffles, one
//      __syncthreads, warp 0 merges the warps and writes the CTA's candidate
//      (value, row index, the whole row) into slot [parity][rank] of EVERY
//      CTA's shared memory (DSMEM stores); warp 1 of the owner of row kc
//      writes row kc into every CTA's krow[parity];
//   2. one cluster barrier (release/acquire): all C candidates and row kc
//      are now local to every CTA;
//   3. every warp picks the pivot from the C local slots (ties to the smaller
//      row, as izamax); the thread owning the pivot row takes row kc, the
//      thread owning row kc takes the pivot row (the row swap), and every
//      thread scales its rows below kc and applies the rank-1 update with the
//      pivot row read from the local slot.
// One __syncthreads and one cluster barrier per column, no DSMEM load on the
// critical path.  Slots are double-buffered by column parity: a CTA can only
// write the slots of column c + 1 after every CTA has left column c - 1.
constexpr int kPanelRPT = 4;        // panel rows per thread at most
constexpr int kMaxClusterPanel = 16;

template <typename T>
struct PanelSmem {
  // offsets in units of T, after the [kNB][ldp] panel
  static __host__ __device__ size_t slots(int ldp) { return (size_t)kNB * ldp; }
  static __host__ __device__ size_t krow(int ldp) {
    return slots(ldp) + (size_t)2 * kMaxClusterPanel * kNB;
  }
  static __host__ __device__ size_t total(int ldp) { return krow(ldp) + 2 * kNB; }
};

template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
panel_cluster_kernel(T* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
                     int* __restrict__ ipiv, int* info) {
  typedef typename CTraits<T>::R R;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ldp = rpb | 1;  // odd column stride
  T* P = reinterpret_cast<T*>(smem_raw);          // [kNB][ldp] panel rows, column-major
  T* slot = P + PanelSmem<T>::slots(ldp);         // [2][kMaxClusterPanel][kNB] candidate rows
  T* krow = P + PanelSmem<T>::krow(ldp);          // [2][kNB] row kc
  __shared__ R sval[2][kMaxClusterPanel];
  __shared__ int sidx[2][kMaxClusterPanel];
  __shared__ R wv[kPanelThreads / 32];
  __shared__ int wi[kPanelThreads / 32];
  __shared__ int s_ipiv[kNB];  // pivots, written to global memory at the end
  __shared__ int s_info;
  const int r0 = k0 + rank * rpb;
  const int r1 = min(r0 + rpb, n);
  const int nr = max(r1 - r0, 0);
  const int lw = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int nw = (int)(blockDim.x >> 5);
  for (int c = 0; c < nb; ++c)
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x)
      P[c * ldp + lr] = A[(size_t)(k0 + c) * lda + r0 + lr];
  if (threadIdx.x == 0) s_info = 0;
  __syncthreads();
  cl.sync();  // every CTA of the cluster is running before any DSMEM access
  for (int c = 0; c < nb; ++c) {
    const int kc = k0 + c, par = c & 1;
    // 1. local candidate, pushed to every CTA
    T vc[kPanelRPT];
    R best = -1;
    int bidx = INT_MAX;
#pragma unroll
    for (int i = 0; i < kPanelRPT; ++i) {
      const int lr = threadIdx.x + i * kPanelThreads;
      if (lr < nr) {
        vc[i] = P[c * ldp + lr];
        if (r0 + lr >= kc) argmax_merge(best, bidx, cabs1(vc[i]), r0 + lr);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R v2 = __shfl_xor_sync(0xffffffffu, best, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, bidx, o);
      argmax_merge(best, bidx, v2, i2);
    }
    if (ln == 0) {
      wv[lw] = best;
      wi[lw] = bidx;
    }
    __syncthreads();
    if (lw == 0) {
      R v = ln < nw ? wv[ln] : R(-1);
      int i = ln < nw ? wi[ln] : INT_MAX;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        argmax_merge(v, i, v2, i2);
      }
      if (ln < C) {
        *cl.map_shared_rank(&sval[par][rank], ln) = v;
        *cl.map_shared_rank(&sidx[par][rank], ln) = i;
      }
      if (i != INT_MAX) {
        const int lr = i - r0;
        const T a0 = P[ln * ldp + lr], a1 = P[(ln + 32) * ldp + lr];
        T* dst = slot + ((size_t)par * kMaxClusterPanel + rank) * kNB;
        for (int q = 0; q < C; ++q) {
          T* d = cl.map_shared_rank(dst, q);
          d[ln] = a0;
          d[ln + 32] = a1;
        }
      }
    } else if (lw == 1 && kc >= r0 && kc < r1) {
      const int lr = kc - r0;
      const T a0 = P[ln * ldp + lr], a1 = P[(ln + 32) * ldp + lr];
      T* dst = krow + (size_t)par * kNB;
      for (int q = 0; q < C; ++q) {
        T* d = cl.map_shared_rank(dst, q);
        d[ln] = a0;
        d[ln + 32] = a1;
      }
    }
    // 2. every candidate and row kc local to every CTA
    cl.sync();
    // 3. pivot (every warp, from local slots), swap, scale, update
    R v = -1;
    int p = INT_MAX, from = 0;
    if (ln < C) {
      v = sval[par][ln];
      p = sidx[par][ln];
      from = ln;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, p, o);
      const int f2 = __shfl_xor_sync(0xffffffffu, from, o);
      if (v2 > v || (v2 == v && i2 < p)) {
        v = v2;
        p = i2;
        from = f2;
      }
    }
    const bool zero = !(v > 0) || p == INT_MAX || p < kc || p >= n;
    if (threadIdx.x == 0) {
      s_ipiv[c] = zero ? kc : p;
      if (zero && s_info == 0) s_info = kc + 1;
    }
    if (zero) continue;  // LAPACK: no swap and no elimination for a zero pivot
    const T* prow = slot + ((size_t)par * kMaxClusterPanel + from) * kNB;
    const T* kr = krow + (size_t)par * kNB;
    const T inv = crcp(prow[c]);
#pragma unroll
    for (int i = 0; i < kPanelRPT; ++i) {
      const int lr = threadIdx.x + i * kPanelThreads;
      if (lr >= nr) break;
      const int gr = r0 + lr;
      if (gr < kc) continue;
      if (gr == kc) {
        if (p != kc)  // row kc becomes the pivot row
          for (int cc = 0; cc < nb; ++cc) P[cc * ldp + lr] = prow[cc];
        continue;
      }
      T a = vc[i];
      if (gr == p) {  // the pivot row takes row kc
        for (int cc = 0; cc < nb; ++cc) P[cc * ldp + lr] = kr[cc];
        a = kr[c];
      }
      const T l = cmul(a, inv);
      P[c * ldp + lr] = l;
      for (int cc0 = c + 1; cc0 < nb; cc0 += 8) {
        T pv[8], pr[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (cc0 + u < nb) {
            pv[u] = P[(cc0 + u) * ldp + lr];
            pr[u] = prow[cc0 + u];
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (cc0 + u < nb) P[(cc0 + u) * ldp + lr] = cfms(pv[u], l, pr[u]);
      }
    }
  }
  cl.sync();  // no CTA leaves while another may still write its shared memory
  if (rank == 0) {
    for (int c = threadIdx.x; c < nb; c += blockDim.x) ipiv[k0 + c] = s_ipiv[c];
    if (threadIdx.x == 0 && s_info && *info == 0) *info = s_info;
  }
  for (int c = 0; c < nb; ++c)
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x)
      A[(size_t)(k0 + c) * lda + r0 + lr] = P[c * ldp + lr];
}

// ---- row-resident complex64 panel -------------------------------------------
// Complex64 panels of up to 16 x 416 rows.  Thread t of CTA r owns rows t and
// t + blockDim of its CTA's slice, stored row-major in shared memory (stride
// 66 complex, 16-byte aligned rows) and is the only thread that ever changes
// them.  Row exchanges are done by renaming: each row carries the index
// (label) of the matrix row it currently represents; the pivot search runs
// over (|re|+|im|, label) with ties to the smaller label (izamax order), and
// at column c the pivot row takes label kc while the row labelled kc takes
// the pivot's label - the permutation LAPACK applies with physical swaps, so
// ipiv is the same.  At the end every row is written to the matrix row
// named by its label.
// A candidate is one 64-bit key: the bits of |re|+|im| (non-negative floats
// order like their bit patterns) above (2^23 - 1 - label) and the local row,
// so the arg-max is a plain maximum (one 64-bit shuffle per step).
// Per column: warp maxima and one __syncthreads form the CTA key; warp 0
// stages the candidate row (columns c..63) at a fixed place; one cluster
// barrier; the warps read every CTA's key and staged row (one DSMEM round
// trip) into local shared memory; a second __syncthreads; every warp picks
// the pivot from the local keys, and each thread scales its rows and
// applies the rank-1 update (16-byte shared-memory accesses, eight column
// pairs per batch).  The update streams the CTA's rows through shared
// memory, so the slices are kept short (64 rows per CTA while 16 CTAs
// suffice) and the CTA has one thread per row.
constexpr int kRowsMaxThreads = 256;
constexpr int kRowsRPT = 2;     // rows per thread
constexpr int kRowsLd = 66;     // complex64 per smem row (528 bytes)
constexpr int kRowsMaxRpb = 416;
constexpr int kRowsMinRpb = 64;
constexpr int kLabelBits = 23;  // labels (matrix rows) below 2^23

__host__ __device__ constexpr size_t panel_rows_smem(int rpb) {
  return sizeof(float2) * ((size_t)rpb * kRowsLd + (size_t)(2 + kMaxClusterPanel) * kNB);
}

__device__ __forceinline__ unsigned long long pivot_key(float a, int label, int lr) {
  return ((unsigned long long)__float_as_uint(a) << 32) |
         ((unsigned long long)((1u << kLabelBits) - 1u - (unsigned)label) << 9) | (unsigned)lr;
}

__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long k) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
    k = k2 > k ? k2 : k;
  }
  return k;
}

__global__ void __launch_bounds__(kRowsMaxThreads, 1)
panel_rows_kernel(float2* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
                  int* __restrict__ ipiv, int* info) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int T = (int)blockDim.x, nw = T >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* P = reinterpret_cast<float2*>(smem_raw);   // [rpb][kRowsLd]
  float2* cand = P + (size_t)rpb * kRowsLd;           // [2][kNB] this CTA's candidate row
  float2* stage = cand + 2 * kNB;                     // [kMaxClusterPanel][kNB] all candidates
  __shared__ unsigned long long ckey[2];
  __shared__ unsigned long long skey[kMaxClusterPanel];
  __shared__ unsigned long long wkey[kRowsMaxThreads / 32];
  __shared__ int s_ipiv[kNB];  // pivots, written to global memory at the end
  __shared__ int s_info;
  const int lw = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int r0 = k0 + rank * rpb;
  const int nr = max(min(rpb, n - r0), 0);
  int label[kRowsRPT];
#pragma unroll
  for (int i = 0; i < kRowsRPT; ++i) {
    const int lr = threadIdx.x + i * T;
    label[i] = lr < nr ? r0 + lr : INT_MAX;
  }
  // load: 16 columns of a row in flight per thread
  for (int lr = threadIdx.x; lr < nr; lr += T) {
    const float2* src = A + (size_t)k0 * lda + r0 + lr;
    for (int c0 = 0; c0 < kNB; c0 += 16) {
      float2 v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        v[u] = c0 + u < nb ? src[(size_t)(c0 + u) * lda] : make_float2(0.f, 0.f);
#pragma unroll
      for (int u = 0; u < 16; ++u) P[lr * kRowsLd + c0 + u] = v[u];
    }
  }
  if (threadIdx.x == 0) s_info = 0;
  __syncthreads();
  cl.sync();  // every CTA of the cluster is running before any DSMEM access
  for (int c = 0; c < nb; ++c) {
    const int kc = k0 + c, par = c & 1;
    // 1. CTA candidate key
    unsigned long long key = 0;
    float2 vc[kRowsRPT];
#pragma unroll
    for (int i = 0; i < kRowsRPT; ++i) {
      const int lr = threadIdx.x + i * T;
      vc[i] = make_float2(0.f, 0.f);
      if (label[i] != INT_MAX) {
        vc[i] = P[lr * kRowsLd + c];
        const float a = cabs1(vc[i]);
        if (label[i] >= kc && a >= 0.f) {  // NaN never wins, as in izamax
          const unsigned long long k2 = pivot_key(a, label[i], lr);
          key = k2 > key ? k2 : key;
        }
      }
    }
    key = warp_max_key(key);
    if (ln == 0) wkey[lw] = key;
    __syncthreads();
    // 2. warp 0: the CTA key and its row, staged at a fixed place
    if (lw == 0) {
      key = warp_max_key(ln < nw ? wkey[ln] : 0ull);
      if (key) {
        const float2* src = P + (size_t)(key & 511ull) * kRowsLd;
        if (c + ln < kNB) cand[par * kNB + c + ln] = src[c + ln];
        if (c + 32 + ln < kNB) cand[par * kNB + c + 32 + ln] = src[c + 32 + ln];
      }
      if (ln == 0) ckey[par] = key;
    }
    cl.sync();
    // 3. every CTA's key and staged row into local shared memory
    for (int q = lw; q < C; q += nw) {
      const float2* src = cl.map_shared_rank(cand, q) + par * kNB;
      const unsigned long long kq = *cl.map_shared_rank(&ckey[par], q);
      if (c + ln < kNB) stage[q * kNB + c + ln] = src[c + ln];
      if (c + 32 + ln < kNB) stage[q * kNB + c + 32 + ln] = src[c + 32 + ln];
      if (ln == 0) skey[q] = kq;
    }
    __syncthreads();
    // 4. the pivot (every warp, from local keys)
    const unsigned long long mine = ln < C ? skey[ln] : 0ull;
    const unsigned long long best = warp_max_key(mine);
    const float v = __uint_as_float((unsigned)(best >> 32));
    const int p = (int)((1u << kLabelBits) - 1u - (unsigned)((best >> 9) & ((1u << kLabelBits) - 1u)));
    const bool zero = best == 0ull || !(v > 0.f) || p < kc || p >= n;
    if (threadIdx.x == 0) {
      // no global store inside the loop: the release of the next cluster
      // barrier would wait for it
      s_ipiv[c] = zero ? kc : p;
      if (zero && s_info == 0) s_info = kc + 1;
    }
    if (zero) continue;  // LAPACK neither swaps nor eliminates
    const int q = __ffsll((long long)__ballot_sync(0xffffffffu, mine == best)) - 1;
    const float2* prow = stage + q * kNB;
    const float4* pr4 = reinterpret_cast<const float4*>(prow);
    const float2 inv = crcp(prow[c]);
    const int j0 = c >> 1;
#pragma unroll
    for (int i = 0; i < kRowsRPT; ++i) {
      if (label[i] == p)
        label[i] = kc;
      else if (label[i] == kc)
        label[i] = p;
      if (label[i] <= kc || label[i] == INT_MAX) continue;
      const int lr = threadIdx.x + i * T;
      float4* row = reinterpret_cast<float4*>(P + (size_t)lr * kRowsLd);
      const float2 l = cmul(vc[i], inv);
      {  // the pair holding column c
        const float4 w = row[j0];
        float2 a = make_float2(w.x, w.y), b = make_float2(w.z, w.w);
        if (c & 1) {
          b = l;
        } else {
          a = l;
          b = cfms(b, l, prow[c + 1]);
        }
        row[j0] = make_float4(a.x, a.y, b.x, b.y);
      }
      for (int jb = j0 + 1; jb < kNB / 2; jb += 8) {
        float4 w[8], pq[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (jb + u < kNB / 2) {
            w[u] = row[jb + u];
            pq[u] = pr4[jb + u];
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (jb + u < kNB / 2) {
            const float2 a = cfms(make_float2(w[u].x, w[u].y), l, make_float2(pq[u].x, pq[u].y));
            const float2 b = cfms(make_float2(w[u].z, w[u].w), l, make_float2(pq[u].z, pq[u].w));
            row[jb + u] = make_float4(a.x, a.y, b.x, b.y);
          }
        }
      }
    }
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
  if (rank == 0) {
    for (int c = threadIdx.x; c < nb; c += T) ipiv[k0 + c] = s_ipiv[c];
    if (threadIdx.x == 0 && s_info && *info == 0) *info = s_info;
  }
#pragma unroll
  for (int i = 0; i < kRowsRPT; ++i) {
    if (label[i] == INT_MAX) continue;
    const int lr = threadIdx.x + i * T;
    for (int cc = 0; cc < nb; ++cc) A[(size_t)(k0 + cc) * lda + label[i]] = P[lr * kRowsLd + cc];
  }
}

// ---- register-window complex64 panel ----------------------------------------
// Complex64 panels of up to 16 x 256 rows.  Two threads per row, each
// holding every other column pair of it in registers (thread h of a row holds
// pairs 2i + h, i = 0..15, as float4 r[16]).  Columns are processed in
// blocks of four (two pairs, one per thread of the row): inside a block the
// column index is a compile-time constant (the loop is unrolled), so every
// register index is static; after a block its finished pairs go to shared
// memory (Fin) and each thread's window shifts by one, so r[i] holds pair
// 2(b + i) + h in block b.  Rows are exchanged by renaming, as in the
// shared-memory panels (same ipiv).
// Reductions use the warp reduce instructions: the maximum of (bits of
// |re|+|im|) + 1 (0 = no candidate; non-negative floats order like their
// bits), then the minimum label among the lanes holding that maximum.
// Per column: one __syncthreads for the warp maxima, one for the CTA
// candidate, whose two threads stage its row (columns c..63) in shared
// memory; one cluster barrier; the threads pull every CTA's key and staged
// row (one DSMEM round trip); a third __syncthreads; every warp picks the
// pivot and each thread updates its registers.
constexpr int kWinMaxRows = 256;
constexpr int kWinMaxThreads = 2 * kWinMaxRows;

__host__ __device__ constexpr size_t panel_win_smem(int rpb) {
  return sizeof(float2) * ((size_t)rpb * kRowsLd + (size_t)(2 + kMaxClusterPanel) * kNB);
}

__device__ __forceinline__ float2 crcp_fast(float2 a) {
  // 1/a = conj(a) / |a|^2 with the components scaled by 1/max(|re|,|im|)
  const float sc = fmaxf(fabsf(a.x), fabsf(a.y));
  const float rs = __frcp_rn(sc);
  const float ar = a.x * rs, ai = a.y * rs;
  const float rd = __frcp_rn(fmaf(ar, ar, ai * ai)) * rs;
  return make_float2(ar * rd, -ai * rd);
}

__device__ __forceinline__ float4 cfms2(float4 w, float2 l, float4 q) {
  const float2 a = cfms(make_float2(w.x, w.y), l, make_float2(q.x, q.y));
  const float2 b = cfms(make_float2(w.z, w.w), l, make_float2(q.z, q.w));
  return make_float4(a.x, a.y, b.x, b.y);
}

__global__ void __launch_bounds__(kWinMaxThreads, 1)
panel_win_kernel(float2* __restrict__ A, long long lda, int n, int k0, int nb, int rpb,
                 int* __restrict__ ipiv, int* info) {
  constexpr int kW = kNB / 4;  // pairs per thread
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int T = (int)blockDim.x, nw = T >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* Fin = reinterpret_cast<float2*>(smem_raw);    // [rpb][kRowsLd] finished pairs
  float4* cand4 = reinterpret_cast<float4*>(Fin + (size_t)rpb * kRowsLd);  // [2][32]
  float4* stage4 = cand4 + 2 * (kNB / 2);                // [kMaxClusterPanel][32]
  __shared__ unsigned ckv[2], ckl[2];
  __shared__ unsigned skv[kMaxClusterPanel], skl[kMaxClusterPanel];
  __shared__ unsigned wkv[kWinMaxThreads / 32], wkl[kWinMaxThreads / 32];
  __shared__ int s_ipiv[kNB];
  __shared__ int s_info;
  const int lw = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int lr = threadIdx.x >> 1, h = threadIdx.x & 1;
  const int r0 = k0 + rank * rpb;
  const int nr = max(min(rpb, n - r0), 0);
  const bool active = lr < nr;
  unsigned label = active ? (unsigned)(r0 + lr) : 0xffffffffu;
  float4 r[kW];
#pragma unroll
  for (int i = 0; i < kW; ++i) {
    const int c0 = 4 * i + 2 * h;
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (active && c0 < nb) a = A[(size_t)(k0 + c0) * lda + label];
    if (active && c0 + 1 < nb) b = A[(size_t)(k0 + c0 + 1) * lda + label];
    r[i] = make_float4(a.x, a.y, b.x, b.y);
  }
  if (threadIdx.x == 0) s_info = 0;
  __syncthreads();
  cl.sync();  // every CTA of the cluster is running before any DSMEM access
  for (int b = 0; 4 * b < nb; ++b) {
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const int c = 4 * b + cc;
      if (c < nb) {
        const int hc = cc >> 1;         // the thread of a row holding column c (static)
        const bool hi = (cc & 1) != 0;  // static
        const unsigned kc = (unsigned)(k0 + c);
        const int par = c & 1;
        // 1. warp and CTA candidates
        const float2 vv = hi ? make_float2(r[0].z, r[0].w) : make_float2(r[0].x, r[0].y);
        const float a = cabs1(vv);
        const unsigned vb =
            (active && h == hc && label >= kc && a >= 0.f) ? __float_as_uint(a) + 1u : 0u;
        unsigned m = __reduce_max_sync(0xffffffffu, vb);
        unsigned lab = __reduce_min_sync(0xffffffffu, (vb == m && m) ? label : 0xffffffffu);
        if (ln == 0) {
          wkv[lw] = m;
          wkl[lw] = lab;
        }
        __syncthreads();
        // every warp forms the CTA candidate from the warp maxima (no second
        // barrier: the next column rewrites them only after the cluster
        // barrier below, which every thread reaches after reading them)
        unsigned cand;
        {
          const unsigned wv = ln < nw ? wkv[ln] : 0u;
          const unsigned wl = ln < nw ? wkl[ln] : 0xffffffffu;
          m = __reduce_max_sync(0xffffffffu, wv);
          lab = __reduce_min_sync(0xffffffffu, (wv == m && m) ? wl : 0xffffffffu);
          cand = m ? lab : 0xfffffffeu;
          if (lw == 0 && ln == 0) {
            ckv[par] = m;
            ckl[par] = lab;
          }
        }
        if (label == cand) {  // this row is the CTA candidate: stage pairs >= c/2
          float4* dst = cand4 + par * (kNB / 2) + 2 * b + h;
#pragma unroll
          for (int i = 0; i < kW; ++i)
            if (i < kW - b && (i > 0 || h >= hc)) dst[2 * i] = r[i];
        }
        // 2. every CTA's candidate visible
        cl.sync();
        // 3. pull all keys and staged rows: loads first, then stores, so
        //    that a thread's DSMEM loads (up to four ranks) are in flight at
        //    once; with no more ranks than warps, warp q pulls rank q
        if (C <= nw) {
          if (lw < C) {
            const int j = ln;
            float4 t4 = make_float4(0.f, 0.f, 0.f, 0.f);
            unsigned tv = 0u, tl = 0u;
            if (j >= (c >> 1)) t4 = cl.map_shared_rank(cand4, lw)[par * (kNB / 2) + j];
            if (j == 0) {
              tv = *cl.map_shared_rank(&ckv[par], lw);
              tl = *cl.map_shared_rank(&ckl[par], lw);
            }
            if (j >= (c >> 1)) stage4[lw * (kNB / 2) + j] = t4;
            if (j == 0) {
              skv[lw] = tv;
              skl[lw] = tl;
            }
          }
        } else {
        for (int q0 = 0; q0 < C; q0 += 4 * nw) {
          constexpr int kPer = 4;
          const int j = ln;  // absolute pair index
          float4 t4[kPer];
          unsigned tv[kPer], tl[kPer];
#pragma unroll
          for (int u = 0; u < kPer; ++u) {
            const int q = q0 + lw + u * nw;
            if (q < C) {
              if (j >= (c >> 1)) t4[u] = cl.map_shared_rank(cand4, q)[par * (kNB / 2) + j];
              if (j == 0) {
                tv[u] = *cl.map_shared_rank(&ckv[par], q);
                tl[u] = *cl.map_shared_rank(&ckl[par], q);
              }
            }
          }
#pragma unroll
          for (int u = 0; u < kPer; ++u) {
            const int q = q0 + lw + u * nw;
            if (q < C) {
              if (j >= (c >> 1)) stage4[q * (kNB / 2) + j] = t4[u];
              if (j == 0) {
                skv[q] = tv[u];
                skl[q] = tl[u];
              }
            }
          }
        }
        }
        __syncthreads();
        // 4. the pivot, from the local keys (every warp)
        const unsigned kv = ln < C ? skv[ln] : 0u;
        const unsigned kl = ln < C ? skl[ln] : 0xffffffffu;
        const unsigned bm = __reduce_max_sync(0xffffffffu, kv);
        const unsigned p = __reduce_min_sync(0xffffffffu, (kv == bm && bm) ? kl : 0xffffffffu);
        const bool zero = bm <= 1u || p < kc || p >= (unsigned)n;  // bm == 1: |pivot| = 0
        if (threadIdx.x == 0) {
          s_ipiv[c] = zero ? (int)kc : (int)p;
          if (zero && s_info == 0) s_info = (int)kc + 1;
        }
        // the row's column-c value, from the thread holding it
        const float2 v = make_float2(__shfl_sync(0xffffffffu, vv.x, (ln & ~1) | hc),
                                     __shfl_sync(0xffffffffu, vv.y, (ln & ~1) | hc));
        if (!zero) {
          const int q = __ffs(__ballot_sync(0xffffffffu, kv == bm && kl == p)) - 1;
          const float4* pr = stage4 + q * (kNB / 2) + 2 * b + h;  // pr[2i]: this thread's pair i
          if (label == p)
            label = kc;
          else if (label == kc)
            label = p;
          if (active && label > kc) {
            const float4 pc = stage4[q * (kNB / 2) + (c >> 1)];
            const float2 piv = hi ? make_float2(pc.z, pc.w) : make_float2(pc.x, pc.y);
            const float2 l = cmul(v, crcp_fast(piv));
            // window position 0 without divergence between the two threads
            // of a row: the update of the whole pair (pr[0] is the pivot
            // row's pair of this thread; for h == hc it is pc, for h < hc a
            // stale slot whose result is discarded), then a select: the
            // pair holding column c keeps its finished column c - 1 (hi) and
            // takes the multiplier l at column c; pair 2b + 1 right of column
            // c takes the update; a finished pair left of c stays
            const float4 x = cfms2(r[0], l, pr[0]);
            if (h == hc)
              r[0] = hi ? make_float4(r[0].x, r[0].y, l.x, l.y) : make_float4(l.x, l.y, x.z, x.w);
            else if (h > hc)
              r[0] = x;
#pragma unroll
            for (int i = 1; i < kW; ++i)
              if (i < kW - b) r[i] = cfms2(r[i], l, pr[2 * i]);
          }
        }
      }
    }
    // block b done: pair 2b + h is final; shift the window by one
    if (active) reinterpret_cast<float4*>(Fin + (size_t)lr * kRowsLd)[2 * b + h] = r[0];
#pragma unroll
    for (int i = 0; i < kW - 1; ++i) r[i] = r[i + 1];
    r[kW - 1] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
  if (rank == 0) {
    for (int c = threadIdx.x; c < nb; c += T) ipiv[k0 + c] = s_ipiv[c];
    if (threadIdx.x == 0 && s_info && *info == 0) *info = s_info;
  }
  __syncthreads();  // Fin complete
  if (active) {
    const float2* fr = Fin + (size_t)lr * kRowsLd;
    for (int c = h; c < nb; c += 2) A[(size_t)(k0 + c) * lda + label] = fr[c];
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

// ---- tournament pivoting for tall complex64 panels --------------------------
// A complex64 panel taller than the register-window cluster holds (16 x 256
// rows) is factored with tournament pivoting (TSLU: Grigori, Demmel and
// Xiang, "CALU: a communication optimal LU factorization algorithm", SIAM J.
// Matrix Anal. Appl. 32, 2011):
//   1. select: G blocks of R rows, one CTA each, run partial pivoting on
//      their own rows in shared memory (no exchange between CTAs) and name
//      the nb rows they pivoted on;
//   2. the G nb candidate rows, with their original values, are gathered and
//      factored with partial pivoting by the register-window cluster kernel:
//      its nb pivot rows are the panel's, its top nb rows are L11 \ U11;
//   3. every other row a of the panel becomes L21 = a U11^{-1} (substitution
//      across the columns, one warp per row), and the panel is written back
//      in pivot order; the pivot sequence is returned as LAPACK row
//      interchanges (ipiv), so the rest of the factorisation is unchanged.
// One exchange between CTAs per panel instead of one per column.  The pivots
// can differ from partial pivoting's (its growth is as small in practice);
// the complex64 factor is the preconditioner of the FP64 refinement, whose
// backward-error test decides the result.
constexpr int kTsluMaxRows = 384;  // rows of one select CTA (one row per thread)
constexpr int kTsluMinRows = 256;
constexpr int kTsluMaxCand = kMaxClusterPanel * kWinMaxRows;  // 4096
constexpr int kTsluFinalCand = 1024;  // capacity of the second candidates' buffer
// candidates left for the final factorisation (a cluster of four CTAs);
// measured on the graded L-shape (N = 16384): LU 127 ms against 140 ms when
// the rounds go on to 256 candidates and one CTA
constexpr int kTsluLastCand = 1024;
constexpr int kTsluMaxH = 64 * kTsluMaxRows;                  // tallest panel (24576)

// Scratch of the tournament, behind the panel exchange slots in
// LuWork::scratch.
struct TsluScratch {
  float2* Cb;    // [kTsluMaxCand][kNB] candidates of rounds 1, 3, ... (original values)
  float2* Cb2;   // [kTsluFinalCand][kNB] candidates of rounds 2, 4, ...
  float2* P;     // [H][kNB] the factored panel
  int* sel;      // [kTsluMaxCand] a round's picks (rows of its input)
  int* mapX;     // [kTsluMaxCand] rows of A of a round's candidates
  int* mapY;     // [kTsluMaxCand] (alternating with mapX)
  int* ipc;      // [kNB] the final candidates' interchanges
  int* infc;     // [1] their first zero pivot
  int* moved;    // [2 kNB + 1] count, then (position, row) pairs beyond the pivots
};
static size_t slots_region() {
  return ((size_t)2 * (kMaxPanelBlocks + 1) * (kSlotHead + sizeof(double2) * kNB) + 511) / 256 *
         256;
}
static size_t tslu_bytes(int n) {
  if (n <= kTsluMaxCand) return 0;
  return sizeof(float2) * (size_t)(kTsluMaxCand + kTsluFinalCand + n) * kNB +
         sizeof(int) * ((size_t)3 * kTsluMaxCand + 4 * kNB + 64) + 2048;
}
static TsluScratch tslu_scratch(void* base, int n) {
  auto al = [](char* q) { return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(q) + 255) / 256 * 256); };
  char* p = al(static_cast<char*>(base));
  TsluScratch t;
  t.Cb = reinterpret_cast<float2*>(p);
  p = al(p + sizeof(float2) * (size_t)kTsluMaxCand * kNB);
  t.Cb2 = reinterpret_cast<float2*>(p);
  p = al(p + sizeof(float2) * (size_t)kTsluFinalCand * kNB);
  t.P = reinterpret_cast<float2*>(p);
  p = al(p + sizeof(float2) * (size_t)n * kNB);
  t.sel = reinterpret_cast<int*>(p);
  t.mapX = t.sel + kTsluMaxCand;
  t.mapY = t.mapX + kTsluMaxCand;
  t.ipc = t.mapY + kTsluMaxCand;
  t.infc = t.ipc + kNB;
  t.moved = t.infc + 32;
  return t;
}

size_t lu_scratch_bytes(int n) { return slots_region() + tslu_bytes(n); }

// One tournament round: grid G, R threads (one row each, R a multiple of
// 32, at most kTsluMaxRows).  Block b runs partial pivoting on rows r0 ..
// r0 + R - 1 (r0 = k0 + b R) of columns k0 .. k0 + nb - 1 and writes the
// rows it pivoted on (absolute indices) to cand[b nb + c], -1 for steps not
// taken.  Each thread holds its row in registers as a window over the
// columns: in block q of four columns, a[i] is column 4 q + i, so every
// register index is static while the loop over blocks stays a loop (the
// window shifts by four after each block).  Per column: the warp's best row
// (reduce by shuffles) stages itself in shared memory, one barrier, every
// warp picks the block's best from the warp bests and updates its rows from
// the staged row.  The staging area alternates between two buffers, so one
// barrier per column suffices.
__global__ void __launch_bounds__(kTsluMaxRows, 1)
tslu_select_kernel(const float2* __restrict__ A, long long lda, int n, int k0, int nb, int R,
                   int* __restrict__ cand) {
  constexpr int kW = kTsluMaxRows / 32;
  __shared__ __align__(16) float2 stage[2][kW][kNB];
  __shared__ unsigned wv[2][kW], wi[2][kW];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = (int)blockDim.x >> 5;
  const int r0 = k0 + blockIdx.x * R;
  const int nr = max(0, min(R, n - r0));
  bool active = t < nr;
  float2 a[kNB];
#pragma unroll
  for (int c = 0; c < kNB; ++c)
    a[c] = (active && c < nb) ? A[(size_t)(k0 + c) * lda + r0 + t] : make_float2(0.f, 0.f);
  int* out = cand + (size_t)blockIdx.x * nb;
  const int npiv = min(nb, nr);
  int taken = 0;
  for (int q = 0; 4 * q < npiv && taken == 4 * q; ++q) {
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const int col = 4 * q + cc, par = cc & 1;
      if (col < npiv && taken == col) {  // uniform over the block
        // keys: bits of |re| + |im| plus one (non-negative floats order like
        // their bits; 0 = not a candidate, NaN counts as zero); the warp's
        // best key, then the smallest row holding it (LAPACK's izamax)
        float v = cabs1(a[cc]);
        if (!(v >= 0.f)) v = 0.f;
        const unsigned key = active ? __float_as_uint(v) + 1u : 0u;
        const unsigned m = __reduce_max_sync(0xffffffffu, key);
        const unsigned lab = __reduce_min_sync(0xffffffffu, (key == m && m) ? (unsigned)t : 0xffffffffu);
        if (lane == 0) {
          wv[par][wid] = m;
          wi[par][wid] = lab;
        }
        const int lim = kNB - 4 * q;  // window positions still holding columns
        if (m && (unsigned)t == lab) {  // the warp's best row: stage columns col ..
          float4* st4 = reinterpret_cast<float4*>(stage[par][wid]);
#pragma unroll
          for (int j = cc & ~1; j < kNB; j += 2) {
            if (j >= lim) break;
            st4[j >> 1] = make_float4(a[j].x, a[j].y, a[j + 1].x, a[j + 1].y);
          }
        }
        __syncthreads();
        const unsigned kv = lane < nw ? wv[par][lane] : 0u;
        const unsigned bm = __reduce_max_sync(0xffffffffu, kv);
        const unsigned bl = __reduce_min_sync(0xffffffffu,
                                              (kv == bm && bm) ? wi[par][lane] : 0xffffffffu);
        const int p = bm ? (int)bl : -1;  // an active row (one is left while col < nr)
        if (p >= 0 && p < nr) {
          if (t == 0) out[col] = r0 + p;
          if (t == p) active = false;  // the pivot row is not updated from here on
          if (active) {
            const float4* pr4 = reinterpret_cast<const float4*>(stage[par][p >> 5]);
            const float4 pc = pr4[cc >> 1];
            const float2 pv = (cc & 1) ? make_float2(pc.z, pc.w) : make_float2(pc.x, pc.y);
            if (pv.x != 0.f || pv.y != 0.f) {
              const float2 l = cmul(a[cc], crcp_fast(pv));
              if (!(cc & 1)) a[cc + 1] = cfms(a[cc + 1], l, make_float2(pc.z, pc.w));
#pragma unroll
              for (int j = (cc & ~1) + 2; j < kNB; j += 2) {
                if (j >= lim) break;
                const float4 u = pr4[j >> 1];
                a[j] = cfms(a[j], l, make_float2(u.x, u.y));
                a[j + 1] = cfms(a[j + 1], l, make_float2(u.z, u.w));
              }
            }
          }
          taken = col + 1;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < kNB - 4; ++i) a[i] = a[i + 4];
#pragma unroll
    for (int i = kNB - 4; i < kNB; ++i) a[i] = make_float2(0.f, 0.f);
  }
  for (int j = taken + t; j < nb; j += blockDim.x) out[j] = -1;  // steps not taken
}

// Cb (Gc x nb, column-major, ld Gc) = rows src[j] of S (column-major, ld
// lds; zero rows for -1); optionally map[j] = idx[src[j]].
// grid (ceil(Gc / 256), nb), 256 threads.
__global__ void tslu_gather_kernel(const float2* __restrict__ S, long long lds, int k0, int nb,
                                   const int* __restrict__ src, int Gc, float2* __restrict__ Cb,
                                   const int* __restrict__ idx, int* __restrict__ map) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (j >= Gc || c >= nb) return;
  const int r = src[j];
  Cb[(size_t)c * Gc + j] = r >= 0 ? S[(size_t)(k0 + c) * lds + r] : make_float2(0.f, 0.f);
  if (map && c == 0) map[j] = (r >= 0 && idx) ? idx[r] : r;
}

// The panel's interchanges from the final candidates' factorisation (ipc,
// infc): ipiv[k0 + c] (LAPACK), and the rows that end beyond the pivots at
// positions other than their own: moved[0] = count, then (position, row)
// pairs.  Positions relative to k0 live in shared memory (2 H ints).  One
// CTA of 1024 threads.
__global__ void __launch_bounds__(1024)
tslu_perm_kernel(int n, int k0, int nb, const int* __restrict__ candF, int Gc,
                 const int* __restrict__ ipc, const int* __restrict__ infc, int* __restrict__ ipiv,
                 int* info, int* __restrict__ moved) {
  extern __shared__ int sh[];
  const int H = n - k0;
  int* pos = sh;       // [H] position of row k0 + i
  int* at = sh + H;    // [H] row at position k0 + i
  __shared__ int cw[kTsluMaxCand];
  for (int i = threadIdx.x; i < H; i += blockDim.x) {
    pos[i] = i;
    at[i] = i;
  }
  Gc = min(Gc, kTsluMaxCand);  // the caller passes at most kTsluMaxCand
  for (int j = threadIdx.x; j < Gc; j += blockDim.x) cw[j] = candF[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < nb; ++c) {  // the candidates' interchanges: cw[c] = pivot row c
      const int q = ipc[c];
      if (q != c && q >= 0 && q < Gc) {
        const int tmp = cw[c];
        cw[c] = cw[q];
        cw[q] = tmp;
      }
    }
    for (int c = 0; c < nb; ++c) {
      const int r = cw[c] - k0;
      if (r < 0 || r >= H) {  // a zero column: no interchange (info is set)
        ipiv[k0 + c] = k0 + c;
        continue;
      }
      const int p = pos[r], rt = at[c];
      ipiv[k0 + c] = k0 + p;
      at[p] = rt;
      pos[rt] = p;
      at[c] = r;
      pos[r] = c;
    }
    int m = 0;
    for (int c = 0; c < nb; ++c) {
      const int p = ipiv[k0 + c] - k0;
      if (p >= nb && at[p] != p) {
        bool seen = false;
        for (int u = 0; u < m; ++u) seen |= moved[1 + 2 * u] == k0 + p;
        if (!seen) {
          moved[1 + 2 * m] = k0 + p;
          moved[2 + 2 * m] = k0 + at[p];
          ++m;
        }
      }
    }
    moved[0] = m;
    if (*infc && *info == 0) *info = k0 + *infc;
  }
}

// P (H x nb, column-major, ld H = n - k0): the factored panel in its final
// row order.  Positions k0 .. k0 + nb - 1: rows 0 .. nb - 1 of the
// candidates' factor (L11 \ U11, Cf: ld Gc); position i beyond: the row r
// there (i itself unless listed in `moved`), x U11 = A(r, :) solved for x =
// L21(i).  A warp per position (lane j holds columns j and j + 32), each CTA
// looping over positions with stride.
__global__ void __launch_bounds__(256)
tslu_rows_kernel(const float2* __restrict__ A, long long lda, int n, int k0, int nb,
                 const float2* __restrict__ Cf, int Gc, const int* __restrict__ moved,
                 float2* __restrict__ P) {
  __shared__ float2 U[kNB * (kNB + 1)];  // U[c (kNB + 1) + r] = U11(c, r): row c of U11
  __shared__ float2 dv[kNB];
  __shared__ int mv[2 * kNB + 1];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int c = e / nb, r = e - c * nb;  // coalesced: consecutive rows of column c
    U[r * (kNB + 1) + c] = Cf[(size_t)c * Gc + r];
  }
  for (int e = threadIdx.x; e < 2 * kNB + 1; e += blockDim.x) mv[e] = moved[e];
  __syncthreads();
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    const float2 d = U[c * (kNB + 1) + c];
    dv[c] = (d.x != 0.f || d.y != 0.f) ? crcp(d) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int H = n - k0, lane = threadIdx.x & 31, m = mv[0];
  const int j0 = lane, j1 = lane + 32;
  for (int i = blockIdx.x * 8 + (threadIdx.x >> 5); i < H; i += gridDim.x * 8) {
    if (i < nb) {
      for (int c = lane; c < nb; c += 32) P[(size_t)c * H + i] = Cf[(size_t)c * Gc + i];
      continue;
    }
    int f = -1;  // the row moved to position k0 + i, if any
    for (int u = lane; u < m; u += 32)
      if (mv[1 + 2 * u] == k0 + i) f = mv[2 + 2 * u];
    f = __reduce_max_sync(0xffffffffu, f);
    const int r = f >= 0 ? f : k0 + i;
    float2 a0 = j0 < nb ? A[(size_t)(k0 + j0) * lda + r] : make_float2(0.f, 0.f);
    float2 a1 = j1 < nb ? A[(size_t)(k0 + j1) * lda + r] : make_float2(0.f, 0.f);
    for (int c = 0; c < nb; ++c) {
      const float2 src = c < 32 ? a0 : a1;
      const float2 ac = make_float2(__shfl_sync(0xffffffffu, src.x, c & 31),
                                    __shfl_sync(0xffffffffu, src.y, c & 31));
      const float2 x = cmul(ac, dv[c]);
      if (j0 == c) a0 = x;
      if (j1 == c) a1 = x;
      if (j0 > c && j0 < nb) a0 = cfms(a0, x, U[c * (kNB + 1) + j0]);
      if (j1 > c && j1 < nb) a1 = cfms(a1, x, U[c * (kNB + 1) + j1]);
    }
    if (j0 < nb) P[(size_t)j0 * H + i] = a0;
    if (j1 < nb) P[(size_t)j1 * H + i] = a1;
  }
}

static int num_sms_lu() {
  static const int v = [] {
    int dev = 0, c = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    return c > 0 ? c : 1;
  }();
  return v;
}

// Tournament-pivoted panel of columns k0 .. k0 + nb - 1 (rows k0 .. n - 1).
// false: not applicable (taller than the tournament holds, scratch too
// small, or the cluster launch refused); A and ipiv are then untouched.
static bool tslu_panel(float2* A, long long lda, int n, int k0, int nb, const LuWork& w, int cmax,
                       cudaStream_t s, long long* launches) {
  const int H = n - k0;
  if (H > kTsluMaxH || tslu_bytes(n) == 0 ||
      w.scratch_bytes < slots_region() + tslu_bytes(n))
    return false;
  const int gmax = kTsluMaxCand / nb;
  const int R0 = std::max(kTsluMinRows, ((H + gmax - 1) / gmax + 31) / 32 * 32);
  if (R0 > kTsluMaxRows) return false;
  const TsluScratch ts = tslu_scratch(static_cast<char*>(w.scratch) + slots_region(), n);
  // rounds: blocks of the current candidates (the panel's rows first), one
  // CTA each, until at most kTsluLastCand are left; a launch the GPU refuses
  // leaves the panel to the other kernels (A is only read until the end)
  const float2* src = A;
  long long lds = lda;
  int koff = k0, rows = H, round = 0, R = R0;
  int* mapPrev = nullptr;
  int* mapNext = ts.mapX;
  float2* Cf = ts.Cb;
  int Gf = 0;
  cudaGetLastError();
  for (;;) {
    const int G = (rows + R - 1) / R;
    Gf = G * nb;
    Cf = (round & 1) ? ts.Cb2 : ts.Cb;
    if (Gf > ((round & 1) ? kTsluFinalCand : kTsluMaxCand)) return false;
    tslu_select_kernel<<<G, R, 0, s>>>(src, lds, koff + rows, koff, nb, R, ts.sel);
    if (cudaGetLastError() != cudaSuccess) return false;
    tslu_gather_kernel<<<dim3((Gf + 255) / 256, nb), 256, 0, s>>>(src, lds, koff, nb, ts.sel, Gf,
                                                                  Cf, mapPrev, mapNext);
    *launches += 2;
    if (Gf <= kTsluLastCand || G == 1) break;
    src = Cf;
    lds = Gf;
    koff = 0;
    rows = Gf;
    R = kTsluMinRows;
    mapPrev = mapNext;
    mapNext = (mapNext == ts.mapX) ? ts.mapY : ts.mapX;
    ++round;
  }
  const int* candF = mapNext;
  const int ld = Gf;
  if (Gf > kTsluMaxCand || sizeof(int) * (2 * (size_t)H + kTsluMaxCand) > 220 * 1024)
    return false;  // the permutation kernel's shared memory
  // the final candidates: partial pivoting in one cluster (one CTA for up to
  // 256 rows)
  int C = std::max(1, (Gf + kWinMaxRows - 1) / kWinMaxRows);
  if (C > cmax) return false;
  const int rpb = (Gf + C - 1) / C;
  const int threads = std::max(64, (2 * rpb + 31) / 32 * 32);
  cudaMemsetAsync(ts.infc, 0, sizeof(int), s);
  if (launch_cluster(panel_win_kernel, C, threads, panel_win_smem(rpb), s, Cf, (long long)ld, Gf,
                     0, nb, rpb, ts.ipc, ts.infc) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  tslu_perm_kernel<<<1, 1024, sizeof(int) * 2 * (size_t)H, s>>>(n, k0, nb, candF, Gf, ts.ipc,
                                                                ts.infc, w.ipiv, w.info, ts.moved);
  const int rgrid = std::min((H + 7) / 8, 4 * num_sms_lu());
  tslu_rows_kernel<<<rgrid, 256, 0, s>>>(A, lda, n, k0, nb, Cf, ld, ts.moved, ts.P);
  cudaMemcpy2DAsync(A + (size_t)k0 * lda + k0, sizeof(float2) * lda, ts.P, sizeof(float2) * H,
                    sizeof(float2) * H, nb, cudaMemcpyDeviceToDevice, s);
  *launches += 2;  // + the cluster launch the caller counts
  return true;
}

constexpr int kMaxCluster = 16;
constexpr size_t kClusterSmem = 220 * 1024;

template <typename T>
static size_t panel_cluster_smem(int rpb) {
  return sizeof(T) * PanelSmem<T>::total(rpb | 1);
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

size_t lu_pack_bytes(int n) {
  return tc_pack_bytes(n, n, n >= kOuterMinN ? kOuterNB : kNB);
}

// SMs left to the panels while a look-ahead update runs beside them
constexpr int kLookaheadFreeSMs = 40;
#ifndef BEM2D_LOOKAHEAD_MIN_N
#define BEM2D_LOOKAHEAD_MIN_N 8192
#endif
bool lu_lookahead(int n) { return n >= BEM2D_LOOKAHEAD_MIN_N; }
int lu_lookahead_ctas() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, v - kLookaheadFreeSMs);
}

size_t lu_aux_bytes(int n, size_t elem) {
  const size_t nk = (n + kNB - 1) / kNB;
  return sizeof(int) * (size_t)n + 2 * nk * kNB * kNB * elem + 256;
}

// C -= Am Bm (M x N, inner dimension K; all three column-major with leading
// dimension ld inside the matrix being factored).  complex64 updates of at
// least kTensorMinN rows and columns run on the tensor cores, the rest on the
// CUDA cores in slices of K = 64.
template <typename T>
static int update_sub(T* C, const T* Am, const T* Bm, long long ld, int M, int N, int K,
                      const LuWork& w, cudaStream_t s, long long* launches) {
  if (M <= 0 || N <= 0 || K <= 0) return BEM2D_OK;
  if constexpr (sizeof(T) == sizeof(float2)) {
    // tall and narrow updates (the columns inside an outer block), and short
    // wide ones (the rows of an outer block right of it) too
    if ((M >= kTensorMinN && N >= kTensorMinN) || (M >= 4 * kTensorMinN && N >= kNB) ||
        (N >= 4 * kTensorMinN && M >= kNB)) {
      ++*launches;
      if (w.pack && tc_pack_bytes(M, N, K) <= w.pack_bytes) {
        *launches += 2;  // + the two packing kernels
        return launch_tc_cgemm_sub(reinterpret_cast<float2*>(C), ld,
                                   reinterpret_cast<const float2*>(Am), ld,
                                   reinterpret_cast<const float2*>(Bm), ld, M, N, K, w.pack,
                                   w.pack_bytes, w.status, s, w.tc_ctas, w.tc_passes)
                   ? BEM2D_ERR_CUDA
                   : BEM2D_OK;
      }
      --*launches;
    }
  }
  dim3 g((M + kGB - 1) / kGB, (N + kGB - 1) / kGB);
  for (int k = 0; k < K; k += kNB) {
    gemm_sub_kernel<T><<<g, 256, sizeof(T) * 2 * kNB * kGB, s>>>(
        Am + (size_t)k * ld, ld, Bm + k, ld, C, ld, M, N, std::min(kNB, K - k));
    ++*launches;
  }
  return BEM2D_OK;
}

template <typename T>
static void trsm_rows(T* A, long long lda, int k0, int nb, int c0, int nc, cudaStream_t s,
                      long long* launches) {
  if (nc <= 0) return;
  trsm_kernel<T><<<(nc + 31) / 32, 256, sizeof(T) * (kNB * kNB + kNB * 32), s>>>(A, lda, k0, nb,
                                                                                c0, nc);
  ++*launches;
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
    cudaFuncSetAttribute(panel_win_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(panel_win_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)panel_win_smem(kWinMaxRows));
    cudaFuncSetAttribute(panel_rows_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(panel_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)panel_rows_smem(kRowsMaxRpb));
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
    cudaFuncSetAttribute(tslu_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(int) * 2 * kTsluMaxH));
  });
  // complex64 matrices are factored in outer blocks of kOuterNB columns:
  // inside a block each 64-column panel updates only the block's columns;
  // the columns right of the block receive one rank-kOuterNB update (K =
  // kOuterNB on the tensor cores), which reads and writes the trailing
  // matrix once per block instead of once per panel.
  const int outer = (sizeof(T) == sizeof(float2) && n >= kOuterMinN) ? kOuterNB : kNB;
  // look-ahead (complex64, from BEM2D_LOOKAHEAD_MIN_N on; a block is an
  // outer block, or a single panel below kOuterMinN): block b's update of the columns
  // beyond block b + 1 runs on w.aux while block b + 1's panels run here;
  // until that update is done, block b + 1 applies its row swaps to its own
  // columns only (the update reads block b's L21 and writes the columns
  // beyond), then to the rest
  const bool la = sizeof(T) == sizeof(float2) && lu_lookahead(n) && w.aux && w.ev_u12 &&
                  w.ev_far && w.pack2 && w.pack2_bytes >= lu_pack_bytes(n);
  LuWork w2 = w;  // the far updates' work: second packing buffer, fewer CTAs
  if (la) {
    w2.pack = w.pack2;
    w2.pack_bytes = w.pack2_bytes;
    w2.tc_ctas = w.aux_ctas;
  }
  bool far_pending = false;
  for (int K0 = 0; K0 < n; K0 += outer) {
  const int bend = std::min(n, K0 + outer);
  for (int k0 = K0; k0 < bend; k0 += kNB) {
    const int nb = std::min(kNB, n - k0);
    const int H = n - k0;
    // cluster panel.  complex64: about one row per thread (256 rows per
    // CTA; the update is cheap on the FP32 pipe, fewer CTAs make the
    // per-column barrier cheaper).  complex128: 64 rows per CTA, as many CTAs
    // as allowed, since the rank-1 updates are bound by the FP64 pipe.  More
    // CTAs when the rows do not fit in shared memory; at most 16 (8
    // portable) CTAs and kPanelRPT rows per thread.
    const int rows_target = sizeof(T) == sizeof(float2) ? kPanelThreads : 64;
    bool done = false;
    if (sizeof(T) == sizeof(float2)) {  // register-window panel
      const int min_rpb = std::min(kWinMaxRows, w.min_rows > 0 ? w.min_rows : kRowsMinRpb);
      for (int cmax : {cluster16 ? kMaxClusterPanel : 8, 8}) {
        int C = std::max(1, std::min(cmax, (H + min_rpb - 1) / min_rpb));
        while ((H + C - 1) / C > kWinMaxRows) ++C;
        if (C > cmax) continue;
        const int rpb = (H + C - 1) / C;
        const int threads = std::max(64, (2 * rpb + 31) / 32 * 32);
        cudaError_t e = launch_cluster(panel_win_kernel, C, threads, panel_win_smem(rpb), s,
                                       reinterpret_cast<float2*>(A), lda, n, k0, nb, rpb,
                                       w.ipiv, w.info);
        if (e == cudaSuccess) {
          done = true;
          break;
        }
        cudaGetLastError();
        if (cmax > 8) cluster16 = false;
      }
    }
    if (!done && sizeof(T) == sizeof(float2)) {  // taller: shared-memory rows panel
      for (int cmax : {cluster16 ? kMaxClusterPanel : 8, 8}) {
        int C = std::max(1, std::min(cmax, (H + kRowsMinRpb - 1) / kRowsMinRpb));
        while ((H + C - 1) / C > kRowsMaxRpb) ++C;
        if (C > cmax) continue;
        const int rpb = (H + C - 1) / C;
        const int threads = rpb <= kRowsMaxThreads ? (rpb + 31) / 32 * 32 : kRowsMaxThreads;
        cudaError_t e = launch_cluster(panel_rows_kernel, C, threads, panel_rows_smem(rpb), s,
                                       reinterpret_cast<float2*>(A), lda, n, k0, nb, rpb,
                                       w.ipiv, w.info);
        if (e == cudaSuccess) {
          done = true;
          break;
        }
        cudaGetLastError();
        if (cmax > 8) cluster16 = false;
      }
    }
    if (!done && sizeof(T) == sizeof(float2)) {
      // taller still: tournament pivoting (measured against the shared-memory
      // rows panel above: ~200 us per 64 columns for it up to 16 x 416 rows,
      // ~260 us for the tournament there; beyond, the grid panel: ~370 us)
      done = tslu_panel(reinterpret_cast<float2*>(A), lda, n, k0, nb, w,
                        cluster16 ? kMaxClusterPanel : 8, s, launches);
    }
    for (int cmax : {cluster16 ? kMaxClusterPanel : 8, 8}) {
      if (done) break;
      int C = std::max(1, std::min(cmax, (H + rows_target - 1) / rows_target));
      while (C < cmax && panel_cluster_smem<T>((H + C - 1) / C) > kClusterSmem) ++C;
      const int rpb = (H + C - 1) / C;
      const size_t smem = panel_cluster_smem<T>(rpb);
      if (smem > kClusterSmem || rpb > kPanelRPT * kPanelThreads) continue;
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
      unsigned spin = kSpinLimit;
      void* args[] = {(void*)&A,      (void*)&lda,    (void*)&n,      (void*)&k0,
                      (void*)&nb,     (void*)&rpb,    (void*)&w.ipiv, (void*)&w.info,
                      (void*)&w.status, (void*)&sl,   (void*)&nblk,   (void*)&spin};
      cudaError_t e = cudaLaunchCooperativeKernel((void*)panel_kernel<T>, dim3(nblk),
                                                  dim3(kPanelThreads), args, smem, s);
      if (e != cudaSuccess) return BEM2D_ERR_CUDA;
    }
    ++*launches;
    if (la) {  // the block's own columns; the rest after the far update
      laswp_cols(A, lda, w.ipiv, k0, nb, K0, k0, s, launches);
      laswp_cols(A, lda, w.ipiv, k0, nb, k0 + nb, bend, s, launches);
    } else if (n > nb) {
      laswp_kernel<T><<<(n - nb + 127) / 128, 128, 0, s>>>(A, lda, n, w.ipiv, k0, nb);
      ++*launches;
    }
    // columns of the block right of this panel
    const int c0 = k0 + nb, ncb = bend - c0;
    if (ncb > 0) {
      trsm_rows(A, lda, k0, nb, c0, ncb, s, launches);
      int rc = update_sub(A + (size_t)c0 * lda + c0, A + (size_t)k0 * lda + c0,
                          A + (size_t)c0 * lda + k0, lda, n - c0, ncb, nb, w, s, launches);
      if (rc) return rc;
    }
  }
  if (la) {  // the block's swaps on the columns outside it
    if (far_pending && cudaStreamWaitEvent(s, w.ev_far, 0) != cudaSuccess) return BEM2D_ERR_CUDA;
    far_pending = false;
    laswp_cols(A, lda, w.ipiv, K0, bend - K0, 0, K0, s, launches);
    laswp_cols(A, lda, w.ipiv, K0, bend - K0, bend, n, s, launches);
  }
  // columns right of the block: U12 = L11^{-1} A12 block row by block row,
  // then A22 -= L21 U12 with K = the block width
  const int nc = n - bend;
  if (nc > 0) {
    for (int j0 = K0; j0 < bend; j0 += kNB) {
      trsm_rows(A, lda, j0, kNB, bend, nc, s, launches);
      const int r1 = j0 + kNB;
      if (r1 < bend) {
        int rc = update_sub(A + (size_t)bend * lda + r1, A + (size_t)j0 * lda + r1,
                            A + (size_t)bend * lda + j0, lda, bend - r1, nc, kNB, w, s, launches);
        if (rc) return rc;
      }
    }
    if (la) {
      // the next block's columns here; the columns beyond it on w.aux
      const int next = std::min(n, bend + outer);
      int rc = update_sub(A + (size_t)bend * lda + bend, A + (size_t)K0 * lda + bend,
                          A + (size_t)bend * lda + K0, lda, nc, next - bend, bend - K0, w, s,
                          launches);
      if (rc) return rc;
      if (next < n) {
        if (cudaEventRecord(w.ev_u12, s) != cudaSuccess ||
            cudaStreamWaitEvent(w.aux, w.ev_u12, 0) != cudaSuccess)
          return BEM2D_ERR_CUDA;
        rc = update_sub(A + (size_t)next * lda + bend, A + (size_t)K0 * lda + bend,
                        A + (size_t)next * lda + K0, lda, nc, n - next, bend - K0, w2, w.aux,
                        launches);
        if (rc) return rc;
        if (cudaEventRecord(w.ev_far, w.aux) != cudaSuccess) return BEM2D_ERR_CUDA;
        far_pending = true;
      }
    } else {
      int rc = update_sub(A + (size_t)bend * lda + bend, A + (size_t)K0 * lda + bend,
                          A + (size_t)bend * lda + K0, lda, nc, nc, bend - K0, w, s, launches);
      if (rc) return rc;
    }
  }
  }
  if (far_pending && cudaStreamWaitEvent(s, w.ev_far, 0) != cudaSuccess) return BEM2D_ERR_CUDA;
  // solve aids: permutation and diagonal-block inverses
  const int nk = (n + kNB - 1) / kNB;
  perm_kernel<<<1, 1024, sizeof(int) * n, s>>>(n, w.ipiv, w.perm);
  dinv_kernel<T><<<nk, 128, sizeof(T) * kNB * kNB, s>>>(A, lda, n, reinterpret_cast<T*>(w.dinv));
  *launches += 2;
  return BEM2D_OK;
}

// ---- triangular solves ----------------------------------------------------
// The solves are templated on the arithmetic type T and the factor's
// storage type TS (TS = complex64, T = complex128: the complex64 factor
// applied exactly in FP64, a fixed operator, as GMRES-IR needs).
template <typename T, typename TS>
__device__ __forceinline__ T cvt(TS v) {
  return CTraits<T>::make(v.x, v.y);
}
// x = U^{-1} L^{-1} P b in one cluster launch.  CTA r owns rows
// [r rpb, (r+1) rpb) of b in shared memory (rpb a multiple of 64).  Step k of
// the forward sweep: the owner of block k forms y_k = L_kk^{-1} b_k from the
// stored inverse; one cluster barrier; every CTA reads y_k over DSMEM and
// updates its rows below the block.  The backward sweep is the mirror with
// U_kk^{-1}.  One cluster barrier per block step.  bin and xout may be the
// same vector (every read of bin precedes the first write of xout), so
// neither is declared __restrict__.
template <typename T, typename TS = T>
__global__ void __launch_bounds__(256)
trisolve_cluster_kernel(const TS* __restrict__ LU, long long lda, int n,
                        const int* __restrict__ perm, const TS* __restrict__ dinv,
                        const T* bin, T* xout, int rpb) {
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
      const TS* Di = dinv + (size_t)(2 * kb + (fwd ? 0 : 1)) * kNB * kNB;
      const T* bk = bc + (k0 - r0);
      const int r = threadIdx.x & 63, g = threadIdx.x >> 6;
      T acc = CTraits<T>::make(0, 0);
      if (r < nb) {
        T l[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) l[u] = cvt<T>(Di[(g * 16 + u) * kNB + r]);
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
      const TS* col = LU + (size_t)(k0 + g * 16) * lda + r;
      T l[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        l[u] = (g * 16 + u < nb) ? cvt<T>(col[(size_t)u * lda]) : CTraits<T>::make(0, 0);
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

// ---- wavefront triangular solves (large n) -----------------------------------
// One cooperative launch per triangle.  The 64-row blocks are dealt to the G
// CTAs round-robin (block b to CTA b % G); each CTA keeps its blocks' entries
// of the right-hand side in shared memory.  Step k (ascending going forward,
// descending going back): the owner of block k, which has already applied
// every earlier step to that block, forms y_k = D_k^{-1} x_k from the stored
// inverse of the diagonal block, writes y_k to the output and to a slot in
// global memory and posts the slot's flag (release); every other CTA that
// still has blocks beyond k waits for the flag (acquire, bounded), reads y_k
// and subtracts L[rows, k] y_k (U[rows, k] y_k going back) from those blocks.
// There is no grid-wide barrier: a CTA waits only for the block it needs
// next, and it loads the factor entries of that step and, if it owns the
// next block, that block's inverse before it waits, so the chain of owners
// costs about one L2 round trip and two 64 x 64 products per step.  The
// factor streams through every SM at once.
constexpr int kWaveThreads = 256;
constexpr int kWaveMinN = 8192;  // below: the single-cluster solve (fewer launches)

template <typename T, bool FWD, typename TS = T>
__global__ void __launch_bounds__(kWaveThreads)
trisolve_wave_kernel(const TS* __restrict__ LU, long long lda, int n, const TS* __restrict__ dinv,
                     const int* __restrict__ perm, const T* bin, T* xout, T* ybuf, int* flags,
                     int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const T zero = CTraits<T>::make(0, 0);
  const int G = gridDim.x, g = blockIdx.x;
  const int nk = (n + kNB - 1) / kNB;
  const int nown = (nk - g + G - 1) / G;  // this CTA's blocks: g, g + G, ...
  T* xs = reinterpret_cast<T*>(smem_raw);  // [nown][kNB]
  T* ys = xs + (size_t)nown * kNB;          // [kNB] y of the current step
  T* ps = ys + kNB;                         // [4][kNB] partial sums
  __shared__ int s_ok;
  const int r = threadIdx.x & (kNB - 1), q = threadIdx.x >> 6;  // row, 16-column group
  for (int v = threadIdx.x; v < nown * kNB; v += blockDim.x) {
    const int row = (g + (v / kNB) * G) * kNB + (v % kNB);
    xs[v] = row < n ? (FWD ? bin[perm[row]] : bin[row]) : zero;
  }
  if (threadIdx.x == 0) s_ok = 1;
  __syncthreads();
  if (nown == 0) return;
  const int first = g, last = g + (nown - 1) * G;  // owned block range
  // entries of the diagonal-block inverse of block k for thread (r, q)
  auto load_dinv = [&](int kb, T* d) {
    const TS* Di = dinv + (size_t)(2 * kb + (FWD ? 0 : 1)) * kNB * kNB;
#pragma unroll
    for (int u = 0; u < 16; ++u) d[u] = cvt<T>(Di[(q * 16 + u) * kNB + r]);
  };
  // factor entries of block row `blk` in the columns of block kb
  auto load_l = [&](int blk, int kb, T* l) {
    const int row = blk * kNB + r, c0 = kb * kNB + q * 16;
    const TS* col = LU + (size_t)c0 * lda + row;
#pragma unroll
    for (int u = 0; u < 16; ++u)
      l[u] = (row < n && c0 + u < n) ? cvt<T>(col[(size_t)u * lda]) : zero;
  };
  // first owned block strictly beyond kb in the sweep direction, or -1
  auto next_owned = [&](int kb) -> int {
    if (FWD) {
      if (kb >= last) return -1;
      const int b = kb < first ? first : first + ((kb - first) / G + 1) * G;
      return b <= last ? b : -1;
    }
    if (kb <= first) return -1;
    const int b = kb > last ? last : first + ((kb - first - 1) / G) * G;
    return b >= first ? b : -1;
  };
  T dpre[16], lpre[16];
  int kb = FWD ? 0 : nk - 1;
  if (kb % G == g) load_dinv(kb, dpre);
  for (int s = 0; s < nk; ++s, kb += FWD ? 1 : -1) {
    if (FWD ? kb > last : kb < first) break;  // nothing of this CTA left to update
    const int jb = next_owned(kb);
    if (jb >= 0) load_l(jb, kb, lpre);
    const int kn = FWD ? kb + 1 : kb - 1;  // the next step's block
    if (kb % G == g) {
      // owner: y = D_k^{-1} x_k, published through ybuf / flags[kb]
      const T* xk = xs + (size_t)((kb - first) / G) * kNB;
      T acc = zero;
#pragma unroll
      for (int u = 0; u < 16; ++u) acc = cfma(dpre[u], xk[q * 16 + u], acc);
      ps[q * kNB + r] = acc;
      __syncthreads();
      if ((int)threadIdx.x < kNB) {
        const int t = threadIdx.x;
        T v = ps[t];
        v.x += ps[kNB + t].x + ps[2 * kNB + t].x + ps[3 * kNB + t].x;
        v.y += ps[kNB + t].y + ps[2 * kNB + t].y + ps[3 * kNB + t].y;
        ys[t] = v;
        if (kb * kNB + t < n) {
          xout[kb * kNB + t] = v;
          ybuf[kb * kNB + t] = v;
        }
      }
      block_publish(&flags[kb], 1);
      if (kn >= 0 && kn < nk && kn % G == g) load_dinv(kn, dpre);
    } else {
      if (kn >= 0 && kn < nk && kn % G == g) load_dinv(kn, dpre);  // before the wait
      if (threadIdx.x == 0 && !wait_seq(&flags[kb], 1, status)) s_ok = 0;
      __syncthreads();
      if (!s_ok) return;
      if ((int)threadIdx.x < kNB)
        ys[threadIdx.x] = kb * kNB + (int)threadIdx.x < n ? __ldcg(&ybuf[kb * kNB + threadIdx.x])
                                                          : zero;
    }
    __syncthreads();
    // update the owned blocks beyond kb: the first with the prefetched
    // entries, the others loading theirs
    for (int blk = jb; blk >= 0 && blk >= first && blk <= last; blk += FWD ? G : -G) {
      T l[16];
      if (blk == jb) {
#pragma unroll
        for (int u = 0; u < 16; ++u) l[u] = lpre[u];
      } else {
        load_l(blk, kb, l);
      }
      T acc = zero;
#pragma unroll
      for (int u = 0; u < 16; ++u) acc = cfma(l[u], ys[q * 16 + u], acc);
      ps[q * kNB + r] = acc;
      __syncthreads();
      if ((int)threadIdx.x < kNB) {
        const int t = threadIdx.x;
        T* xv = xs + (size_t)((blk - first) / G) * kNB + t;
        T v = *xv;
        v.x -= ps[t].x + ps[kNB + t].x + ps[2 * kNB + t].x + ps[3 * kNB + t].x;
        v.y -= ps[t].y + ps[kNB + t].y + ps[2 * kNB + t].y + ps[3 * kNB + t].y;
        *xv = v;
      }
      __syncthreads();
    }
  }
}

template <typename T, typename TS = T>
static int lu_solve_wave(const TS* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
                         cudaStream_t s, long long* launches) {
  const int nk = (n + kNB - 1) / kNB;
  // scratch: forward result v [n], y slots [nk * kNB], flags [2 * nk]
  const size_t need = sizeof(T) * ((size_t)n + (size_t)nk * kNB) + sizeof(int) * 2 * nk;
  if (w.scratch_bytes < need) return BEM2D_ERR_ARG;
  T* v = static_cast<T*>(w.scratch);
  T* ybuf = v + n;
  int* flags = reinterpret_cast<int*>(ybuf + (size_t)nk * kNB);
  static const int nsm = [] {
    int dev = 0, c = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    return std::max(c, 1);
  }();
  const int G = std::min(nk, nsm);
  const size_t smem = sizeof(T) * ((size_t)((nk + G - 1) / G) * kNB + 5 * kNB);
  if (smem > 48 * 1024) return BEM2D_ERR_ARG;
  cudaMemsetAsync(flags, 0, sizeof(int) * 2 * nk, s);
  const TS* dinv = reinterpret_cast<const TS*>(w.dinv);
  const int* perm = w.perm;
  int* fl = flags;
  int* status = w.status;
  T* vo = v;
  void* af[] = {(void*)&LU, (void*)&lda, (void*)&n, (void*)&dinv, (void*)&perm, (void*)&b,
                (void*)&vo, (void*)&ybuf, (void*)&fl, (void*)&status};
  if (cudaLaunchCooperativeKernel((void*)trisolve_wave_kernel<T, true, TS>, dim3(G),
                                  dim3(kWaveThreads), af, smem, s) != cudaSuccess)
    return BEM2D_ERR_CUDA;
  const T* vin = v;
  int* fb = flags + nk;
  void* ab[] = {(void*)&LU, (void*)&lda, (void*)&n, (void*)&dinv, (void*)&perm, (void*)&vin,
                (void*)&x, (void*)&ybuf, (void*)&fb, (void*)&status};
  if (cudaLaunchCooperativeKernel((void*)trisolve_wave_kernel<T, false, TS>, dim3(G),
                                  dim3(kWaveThreads), ab, smem, s) != cudaSuccess)
    return BEM2D_ERR_CUDA;
  *launches += 2;
  return BEM2D_OK;
}

template <typename T>
int lu_solve(const T* LU, long long lda, int n, const LuWork& w, const T* b, T* x,
             cudaStream_t s, long long* launches) {
  if (n >= kWaveMinN) return lu_solve_wave(LU, lda, n, w, b, x, s, launches);
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

// x = A^{-1} b with a complex64 factor, the arithmetic in complex128.
int lu_solve_mixed(const float2* LU, long long lda, int n, const LuWork& w, const double2* b,
                   double2* x, cudaStream_t s, long long* launches) {
  if (n >= kWaveMinN) return lu_solve_wave<double2, float2>(LU, lda, n, w, b, x, s, launches);
  static std::atomic<int> cmax{kMaxCluster};
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(trisolve_cluster_kernel<double2, float2>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmem);
    if (cudaFuncSetAttribute(trisolve_cluster_kernel<double2, float2>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      cmax = 8;
    }
  });
  for (;;) {
    const int nk = (n + kNB - 1) / kNB;
    const int C = std::max(1, std::min(cmax.load(), nk));
    const int rpb = ((nk + C - 1) / C) * kNB;
    const size_t smem = sizeof(double2) * ((size_t)rpb + kNB + 4 * (size_t)std::max(rpb, kNB));
    if (smem > kClusterSmem) return BEM2D_ERR_ARG;
    cudaError_t e = launch_cluster(trisolve_cluster_kernel<double2, float2>, C, 256, smem, s, LU,
                                   lda, n, (const int*)w.perm, (const float2*)w.dinv, b, x, rpb);
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

// Timeout check of the grid panel's bounded waits: one panel of the
// complex64 matrix A (n x 64, n >= 256, lda) on two cooperative blocks whose
// waits expect three candidates, so each waits for a slot that is never
// posted; every wait gives up after `polls` polls, sets *w.status and the
// kernel returns.  The caller reads *w.status after synchronising.
int lu_panel_timeout_probe(float2* A, long long lda, int n, const LuWork& w, unsigned polls,
                           cudaStream_t s) {
  if (n < 256 || lda < n || polls < 1) return BEM2D_ERR_ARG;
  PanelSlots<float2> sl;
  sl.base = static_cast<char*>(w.scratch);
  cudaMemsetAsync(w.info, 0, sizeof(int), s);
  cudaMemsetAsync(w.status, 0, sizeof(int), s);
  cudaMemsetAsync(sl.base, 0, slots_bytes(sizeof(float2)), s);
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(panel_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
  });
  int nblk = 2, k0 = 0, nb = kNB;
  int rpb = (n + nblk - 1) / nblk;
  const size_t smem = sizeof(float2) * ((size_t)rpb * kNB + kNB + rpb);
  if (smem > 200 * 1024) return BEM2D_ERR_ARG;
  int nwait = nblk + 1;
  unsigned spin = polls;
  void* args[] = {(void*)&A,      (void*)&lda,    (void*)&n,      (void*)&k0,
                  (void*)&nb,     (void*)&rpb,    (void*)&w.ipiv, (void*)&w.info,
                  (void*)&w.status, (void*)&sl,   (void*)&nwait,  (void*)&spin};
  return cudaLaunchCooperativeKernel((void*)panel_kernel<float2>, dim3(nblk),
                                     dim3(kPanelThreads), args, smem, s) == cudaSuccess
             ? BEM2D_OK
             : BEM2D_ERR_CUDA;
}

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

// ---- explicit inverse of a complex64 factor ---------------------------------
// W = U^{-1} L^{-1} from the factor P A = L U of lu_factor<float2>, so that
// A^{-1} x = W (P x) and A^{-H} x = P^T (W^H x).  Blocked substitution on
// the identity, 64 rows at a time inside outer blocks of 256 rows (64 when
// the packing buffer only holds rank-64 operands):
//   forward  Y_k = L_kk^{-1} Y_k, then the outer block's rows below k, and
//            after the outer block the rows below it (Y stays lower
//            triangular: only the columns left of the block are touched);
//   backward W_k = U_kk^{-1} W_k, then the outer block's rows above k, and
//            after the outer block the rows above it.
// The diagonal-block inverses are lu_factor's (w.dinv); the updates run on
// the tensor cores (the trailing-update kernel).  About 2.7 N^3
// complex flops; an inverse pays for itself once an iteration needs more
// than a few dozen solves with the factor (a product with W streams N^2
// entries; the substitution is a chain of 2 N / 64 dependent steps).

// Xb (rows r0 .. r0 + bs - 1 of X, column-major, ld ldx) = D Xb, D a 64 x 64
// column-major block (zero beyond bs).  grid ceil(ncols / 16), 256 threads.
__global__ void __launch_bounds__(256)
block_apply_kernel(const float2* __restrict__ D, float2* __restrict__ X, long long ldx, int bs,
                   int ncols) {
  __shared__ float2 Ds[kNB * kNB];  // Ds[k * 64 + r] = D(r, k)
  __shared__ float2 T[kNB * 17];    // T[k * 17 + c] = X(r0 + k, c0 + c)
  const int c0 = blockIdx.x * 16;
  for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) Ds[e] = D[e];
  for (int e = threadIdx.x; e < kNB * 16; e += blockDim.x) {
    const int c = e / kNB, k = e - c * kNB;  // coalesced along k (rows)
    T[k * 17 + c] = (k < bs && c0 + c < ncols) ? X[(size_t)(c0 + c) * ldx + k]
                                                : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int c = threadIdx.x & 15, rb = threadIdx.x >> 4;  // rows rb + 16 q
  float2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int k = 0; k < bs; ++k) {
    const float2 t = T[k * 17 + c];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = cfma(Ds[k * kNB + rb + 16 * q], t, acc[q]);
  }
  if (c0 + c >= ncols) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = rb + 16 * q;
    if (r < bs) X[(size_t)(c0 + c) * ldx + r] = acc[q];
  }
}

__global__ void identity_c64_kernel(int n, float2* __restrict__ X, long long ldx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) X[(size_t)i * ldx + i] = make_float2(1.f, 0.f);
}

int lu_inverse_c64(const float2* LU, long long lda, int n, const LuWork& w, float2* W,
                   long long ldw, cudaStream_t s, long long* launches) {
  if (n <= 0) return BEM2D_OK;
  if (!w.pack || !w.dinv) return BEM2D_ERR_ARG;
  if (tc_pack_bytes(n, n, kNB) > w.pack_bytes) return BEM2D_ERR_ARG;
  // outer blocks of kOuterNB rows where the packing buffer holds rank-256
  // operands (one pass over the rest of W per outer block, not per 64 rows)
  const int ob = tc_pack_bytes(n, n, kOuterNB) <= w.pack_bytes ? kOuterNB : kNB;
  auto upd = [&](float2* C, const float2* Am, const float2* Bm, int M, int N, int K) -> int {
    if (M <= 0 || N <= 0 || K <= 0) return BEM2D_OK;
    if (launch_tc_cgemm_sub(C, ldw, Am, lda, Bm, ldw, M, N, K, w.pack, w.pack_bytes, w.status, s))
      return BEM2D_ERR_CUDA;
    *launches += 3;
    return BEM2D_OK;
  };
  if (cudaMemset2DAsync(W, sizeof(float2) * ldw, 0, sizeof(float2) * n, n, s) != cudaSuccess)
    return BEM2D_ERR_CUDA;
  identity_c64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, W, ldw);
  ++*launches;
  const float2* dinv = static_cast<const float2*>(w.dinv);
  int rc = 0;
  for (int R0 = 0; R0 < n; R0 += ob) {  // forward: Y = L^{-1} (lower triangular)
    const int R1 = std::min(n, R0 + ob);
    for (int k0 = R0; k0 < R1; k0 += kNB) {
      const int kb = k0 / kNB, bs = std::min(kNB, n - k0), nc = k0 + bs;
      block_apply_kernel<<<(nc + 15) / 16, 256, 0, s>>>(dinv + (size_t)(2 * kb) * kNB * kNB,
                                                        W + k0, ldw, bs, nc);
      ++*launches;
      // the rest of this outer block's rows
      if ((rc = upd(W + nc, LU + (size_t)k0 * lda + nc, W + k0, R1 - nc, nc, bs))) return rc;
    }
    // the rows below the outer block, columns 0 .. R1 - 1 (Y is zero beyond)
    if ((rc = upd(W + R1, LU + (size_t)R0 * lda + R1, W + R0, n - R1, R1, R1 - R0))) return rc;
  }
  const int nob = (n + ob - 1) / ob;
  for (int q = nob - 1; q >= 0; --q) {  // backward: W = U^{-1} Y
    const int R0 = q * ob, R1 = std::min(n, R0 + ob);
    for (int k0 = ((R1 - 1) / kNB) * kNB; k0 >= R0; k0 -= kNB) {
      const int kb = k0 / kNB, bs = std::min(kNB, n - k0);
      block_apply_kernel<<<(n + 15) / 16, 256, 0, s>>>(dinv + (size_t)(2 * kb + 1) * kNB * kNB,
                                                       W + k0, ldw, bs, n);
      ++*launches;
      if ((rc = upd(W + R0, LU + (size_t)k0 * lda + R0, W + k0, k0 - R0, n, bs))) return rc;
    }
    if ((rc = upd(W, LU + (size_t)R0 * lda, W + R0, R0, n, R1 - R0))) return rc;
  }
  return cudaPeekAtLastError() == cudaSuccess ? BEM2D_OK : BEM2D_ERR_CUDA;
}

// dst[i] = (complex64) (scale src[perm[i]]): P x of an FP64 vector.
__global__ void gather_to_c64_kernel(int n, const double2* __restrict__ src,
                                     const int* __restrict__ perm, double scale,
                                     float2* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = src[perm[i]];
  dst[i] = make_float2((float)(v.x * scale), (float)(v.y * scale));
}
// dst[perm[i]] = src[i]: P^T y (complex64).
__global__ void scatter_c64_kernel(int n, const float2* __restrict__ src,
                                   const int* __restrict__ perm, float2* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}
void launch_gather_to_c64(int n, const double2* src, const int* perm, double scale, float2* dst,
                          cudaStream_t s) {
  gather_to_c64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, src, perm, scale, dst);
}
void launch_scatter_c64(int n, const float2* src, const int* perm, float2* dst, cudaStream_t s) {
  scatter_c64_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, src, perm, dst);
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

// *flag |= 1 if any entry of the rows x cols column-major block is NaN or
// infinite: one coalesced pass (rows fastest), one atomic per warp that saw
// a non-finite value.
__global__ void nonfinite_kernel(const double2* __restrict__ A, long long ld, int rows, int cols,
                                 int* flag) {
  bool bad = false;
  for (int j = blockIdx.y; j < cols; j += gridDim.y)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
      const double2 a = A[(size_t)j * ld + i];
      bad |= !(isfinite(a.x) && isfinite(a.y));
    }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

void launch_nonfinite_scan(const double2* A, long long ld, int rows, int cols, int* flag,
                           cudaStream_t s) {
  const int bx = std::min(8, (rows + 255) / 256);
  const int by = std::min(cols, 1024);
  nonfinite_kernel<<<dim3(bx, by), 256, 0, s>>>(A, ld, rows, cols, flag);
}

}  // namespace bem2d_gpu
