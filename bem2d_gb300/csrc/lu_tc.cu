// Trailing update of the complex64 LU on the 5th-generation tensor cores:
// C -= A B (complex64, column-major, arbitrary leading dimensions), as
// tcgen05.mma kind::tf32 with FP32 accumulators in tensor memory.
//
// Complex arithmetic as two real products.  The complex M x K operand A is
// read as a real (2M) x K matrix A' whose rows 2i and 2i + 1 hold re and im
// of row i (that is how complex column-major data lies in memory).  With the
// real and imaginary parts B_r, B_i of B (K x N):
//   D1 = A' B_r,  D2 = A' B_i,
//   re C_i = D1[2i] - D2[2i+1],   im C_i = D2[2i] + D1[2i+1].
// One CTA owns a tile of 64 complex rows (128 real rows = the MMA's M) and
// 64 complex columns (the MMA's N); D1 and D2 take 64 tensor-memory columns
// each.  K is staged 32 at a time (64 KB of shared memory), so three CTAs
// share an SM and one CTA's epilogue overlaps another's staging and MMAs.
//
// Accuracy (3xTF32): every FP32 operand x is split into hi = x with its low
// 13 mantissa bits cleared (exactly a TF32 value) and lo = x - hi; each
// product is accumulated as hi*hi + hi*lo + lo*hi, which keeps about 21 bits
// per product - the accuracy of the FP32 update it replaces, so the LU keeps
// the quality the FP64 refinement expects.
//
// Operands are staged by the CTA's threads (global -> split -> shared memory)
// in the K-major, non-swizzled canonical layout: core matrices of 8 rows x
// 16 bytes; 128 bytes from one core matrix to the next along K (leading
// byte offset), 1024 bytes from one group of 8 rows to the next (stride
// byte offset).  One thread issues the MMAs; tcgen05.commit signals an
// mbarrier that the others wait on (bounded: on timeout the status flag is
// set and the tile is left unchanged).  The epilogue reads D1/D2 with
// tcgen05.ld (warp w reads lanes 32w..32w+31 = real rows), combines rows
// 2i/2i+1 with one shuffle and updates C in place.
#include <cuda_runtime.h>

#include "common.cuh"

namespace bem2d_gpu {
namespace {

constexpr int kTcBM = 64;   // complex rows per tile (128 real rows = MMA M)
constexpr int kTcBN = 64;   // complex columns per tile (MMA N)
constexpr int kTcBK = 32;   // K per staged chunk
constexpr int kTcThreads = 128;
constexpr int kCoreBytes = 128;                      // 8 rows x 16 bytes
constexpr int kTcSBO = (kTcBK / 4) * kCoreBytes;     // 1024
constexpr int kTcAbytes = 2 * kTcBM * kTcBK * 4;     // 16 KB per split part
constexpr int kTcBbytes = kTcBN * kTcBK * 4;         // 8 KB per part
constexpr int kTcSmem = 2 * kTcAbytes + 4 * kTcBbytes + 64;
constexpr unsigned kTcSpin = 1u << 24;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
// tcgen05 shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
  return (unsigned long long)((addr & 0x3FFFF) >> 4) |
         ((unsigned long long)(kCoreBytes >> 4) << 16) |
         ((unsigned long long)(kTcSBO >> 4) << 32) | (1ull << 46);
}
// byte offset of (row r, k) in the canonical layout
__device__ __forceinline__ int kmajor_off(int r, int k) {
  return (r >> 3) * kTcSBO + (k >> 2) * kCoreBytes + (r & 7) * 16 + (k & 3) * 4;
}
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

__device__ __forceinline__ void mma_tf32(unsigned d, unsigned a, unsigned b, unsigned idesc,
                                         unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(smem_desc(a)), "l"(smem_desc(b)), "r"(idesc), "r"(acc));
}

#define TC_LD16(dst, addr)                                                                  \
  asm volatile(                                                                             \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15}, [%16];"                                                                     \
      : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]), \
        "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]), "=r"(dst[11]), \
        "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])                          \
      : "r"(addr))

__global__ void __launch_bounds__(kTcThreads, 3)
tc_cgemm_sub_kernel(float2* __restrict__ C, long long ldc, const float2* __restrict__ A,
                    long long lda, const float2* __restrict__ B, long long ldb, int M, int N,
                    int K, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* Ahi = sm;
  unsigned char* Alo = sm + kTcAbytes;
  unsigned char* Brh = sm + 2 * kTcAbytes;
  unsigned char* Brl = Brh + kTcBbytes;
  unsigned char* Bih = Brl + kTcBbytes;
  unsigned char* Bil = Bih + kTcBbytes;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(Bil + kTcBbytes);
  unsigned* tslot = reinterpret_cast<unsigned*>(mbar + 1);
  const int t = threadIdx.x, w = t >> 5;
  const int i0 = blockIdx.x * kTcBM, n0 = blockIdx.y * kTcBN;
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
        smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = *tslot;
  // kind::tf32: D f32 (bits 4-5 = 1), A/B tf32 (bits 7-9, 10-12 = 2), both
  // K-major, N >> 3 at bit 17, M >> 4 at bit 24
  const unsigned idesc =
      (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(kTcBN >> 3) << 17) | ((128u >> 4) << 24);
  unsigned phase = 0;
  bool timeout = false;
  for (int kb = 0; kb < K; kb += kTcBK) {
    // Stage A: a warp covers 4 complex rows x 4 k, both components, so its
    // 32 stores fill one 128-byte line of core matrices (no bank conflict);
    // loads are batched 16 deep.
    {
      const int l = t & 31;
      const int ci = (l >> 2) & 1, kl = l & 3, il = l >> 3;
      const float* Af = reinterpret_cast<const float*>(A);
      for (int j0 = 0; j0 < kTcBM * kTcBK * 2 / kTcThreads; j0 += 16) {
        float v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int b = w + 4 * (j0 + u);
          const int i = (b & 15) * 4 + il, k = (b >> 4) * 4 + kl;
          v[u] = (i0 + i < M && kb + k < K) ? Af[2 * ((size_t)(kb + k) * lda + i0 + i) + ci] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int b = w + 4 * (j0 + u);
          const int i = (b & 15) * 4 + il, k = (b >> 4) * 4 + kl;
          const int off = kmajor_off(2 * i + ci, k);
          float h, lo;
          tf32_split(v[u], h, lo);
          *reinterpret_cast<float*>(Ahi + off) = h;
          *reinterpret_cast<float*>(Alo + off) = lo;
        }
      }
    }
    // Stage B: a warp covers 8 columns n x 4 k (one line per part)
    {
      const int l = t & 31;
      const int kl = l & 3, nl = l >> 2;
      for (int j0 = 0; j0 < kTcBN * kTcBK / kTcThreads; j0 += 16) {
        float2 v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int b = w + 4 * (j0 + u);
          const int n = (b & 7) * 8 + nl, k = (b >> 3) * 4 + kl;
          v[u] = (n0 + n < N && kb + k < K) ? B[(size_t)(n0 + n) * ldb + kb + k]
                                             : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int b = w + 4 * (j0 + u);
          const int n = (b & 7) * 8 + nl, k = (b >> 3) * 4 + kl;
          const int off = kmajor_off(n, k);
          float h, lo;
          tf32_split(v[u].x, h, lo);
          *reinterpret_cast<float*>(Brh + off) = h;
          *reinterpret_cast<float*>(Brl + off) = lo;
          tf32_split(v[u].y, h, lo);
          *reinterpret_cast<float*>(Bih + off) = h;
          *reinterpret_cast<float*>(Bil + off) = lo;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const unsigned d1 = tmem, d2 = tmem + kTcBN;
      for (int s = 0; s < kTcBK / 8; ++s) {
        const unsigned o = 256u * s;  // K = 8 tf32 = two core matrices
        const unsigned ah = smem_u32(Ahi) + o, al = smem_u32(Alo) + o;
        const unsigned acc = (kb == 0 && s == 0) ? 0u : 1u;
        mma_tf32(d1, ah, smem_u32(Brh) + o, idesc, acc);
        mma_tf32(d1, ah, smem_u32(Brl) + o, idesc, 1u);
        mma_tf32(d1, al, smem_u32(Brh) + o, idesc, 1u);
        mma_tf32(d2, ah, smem_u32(Bih) + o, idesc, acc);
        mma_tf32(d2, ah, smem_u32(Bil) + o, idesc, 1u);
        mma_tf32(d2, al, smem_u32(Bih) + o, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(mbar)));
    }
    unsigned done = 0;
    for (unsigned it = 0; it < kTcSpin && !done; ++it)
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          " selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(smem_u32(mbar)), "r"(phase));
    if (!done) timeout = true;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();  // the operands may be restaged
    if (__syncthreads_or(timeout)) {
      timeout = true;
      break;
    }
  }
  if (timeout) {
    if (t == 0) atomicExch(status, 1);
  } else {
    const int i = t >> 1, c = t & 1;  // real row t = 2i + c
    const unsigned lanes = tmem + ((unsigned)(w * 32) << 16);
    float* Cf = reinterpret_cast<float*>(C);
    const bool row_ok = i0 + i < M;
    for (int j0 = 0; j0 < kTcBN; j0 += 16) {
      float cv[16];  // the C values first, all loads in flight
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int n = n0 + j0 + u;
        cv[u] = (row_ok && n < N) ? Cf[2 * ((size_t)n * ldc + i0 + i) + c] : 0.f;
      }
      unsigned d1[16], d2[16];
      TC_LD16(d1, lanes + j0);
      TC_LD16(d2, lanes + kTcBN + j0);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const float p2 = __shfl_xor_sync(0xffffffffu, __uint_as_float(d2[u]), 1);
        const float o = __uint_as_float(d1[u]) + (c ? p2 : -p2);
        const int n = n0 + j0 + u;
        if (row_ok && n < N) Cf[2 * ((size_t)n * ldc + i0 + i) + c] = cv[u] - o;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

#undef TC_LD16

}  // namespace

int launch_tc_cgemm_sub(float2* C, long long ldc, const float2* A, long long lda,
                        const float2* B, long long ldb, int M, int N, int K, int* status,
                        cudaStream_t s) {
  static const cudaError_t attr = cudaFuncSetAttribute(
      tc_cgemm_sub_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (attr != cudaSuccess) return BEM2D_ERR_CUDA;
  if (M <= 0 || N <= 0 || K <= 0) return BEM2D_OK;
  dim3 grid((M + kTcBM - 1) / kTcBM, (N + kTcBN - 1) / kTcBN);
  tc_cgemm_sub_kernel<<<grid, kTcThreads, kTcSmem, s>>>(C, ldc, A, lda, B, ldb, M, N, K, status);
  return cudaPeekAtLastError() == cudaSuccess ? BEM2D_OK : BEM2D_ERR_CUDA;
}

}  // namespace bem2d_gpu
