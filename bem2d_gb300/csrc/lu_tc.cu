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
// each.
//
// Accuracy (3xTF32): every FP32 operand x is split into hi = x with its low
// 13 mantissa bits cleared (exactly a TF32 value) and lo = x - hi; each
// product is accumulated as hi*hi + hi*lo + lo*hi, which keeps about 21 bits
// per product - the accuracy of the FP32 update it replaces, so the LU keeps
// the quality the FP64 refinement expects.
//
// Operands are packed once per update (pack_a_kernel, pack_b_kernel): split
// into hi/lo and laid out, per tile and per chunk of 16 along K, exactly as
// the MMA reads them from shared memory - the K-major, non-swizzled
// canonical layout (core matrices of 8 rows x 16 bytes, 128 bytes from one
// core matrix to the next along K, 512 bytes from one group of 8 rows to the
// next).  The update kernel then stages each chunk with two bulk copies
// (cp.async.bulk, completion counted in bytes on an mbarrier) into one of two
// shared-memory stages, so the copy of chunk c + 1 overlaps the MMAs of
// chunk c.  One thread issues the copies and the MMAs; tcgen05.commit
// signals an mbarrier when a stage's MMAs are done (the stage may then be
// refilled) and, at the end, that the accumulators are complete.  Every wait
// is bounded: on timeout the status flag is set and the tile is left
// unchanged.  The epilogue reads D1/D2 with tcgen05.ld (warp w reads lanes
// 32w..32w+31 = real rows), combines rows 2i/2i+1 with one shuffle and
// updates C in place.
#include <cuda_runtime.h>

#include "common.cuh"

namespace bem2d_gpu {
namespace {

constexpr int kTcBM = 64;   // complex rows per tile (128 real rows = MMA M)
constexpr int kTcBN = 64;   // complex columns per tile (MMA N)
constexpr int kTcBK = 16;   // K per chunk (two MMAs of K = 8)
constexpr int kTcThreads = 128;
constexpr int kCoreBytes = 128;                   // 8 rows x 16 bytes
constexpr int kTcSBO = (kTcBK / 4) * kCoreBytes;  // 512
constexpr int kTcApart = 2 * kTcBM * kTcBK * 4;   // 8 KB: 128 real rows x 16
constexpr int kTcBpart = kTcBN * kTcBK * 4;       // 4 KB: 64 rows x 16
constexpr int kTcChunkA = 2 * kTcApart;           // hi, lo
constexpr int kTcChunkB = 4 * kTcBpart;           // re hi, re lo, im hi, im lo
constexpr int kTcStage = kTcChunkA + kTcChunkB;   // 32 KB
constexpr int kTcSmem = 2 * kTcStage + 64;
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
// byte offset of (row r, k) inside one packed chunk
__host__ __device__ __forceinline__ int kmajor_off(int r, int k) {
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

__device__ __forceinline__ void mbar_init(unsigned long long* m) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(m)));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)),
               "r"(bytes));
}
// bounded wait for phase `parity` of the mbarrier; false on timeout
__device__ __forceinline__ bool mbar_wait(unsigned long long* m, unsigned parity) {
  unsigned done = 0;
  for (unsigned it = 0; it < kTcSpin && !done; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(m)), "r"(parity));
  return done != 0;
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes,
                                          unsigned long long* m) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(m))
      : "memory");
}

#define TC_LD16(dst, addr)                                                                  \
  asm volatile(                                                                             \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
      "%14,%15}, [%16];"                                                                     \
      : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]), \
        "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]), "=r"(dst[11]), \
        "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])                          \
      : "r"(addr))

// ---- packing ---------------------------------------------------------------
// A (M x K complex) -> Apk[mt][kc] = {hi, lo} chunks of kTcApart bytes each.
// grid: (ceil(M / 64) * 64 / 128 x nkc * 16), 128 threads
__global__ void pack_a_kernel(const float2* __restrict__ A, long long lda, int M, int K, int nkc,
                              unsigned char* __restrict__ Apk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // complex row
  const int k = blockIdx.y;                             // 0 .. nkc * 16 - 1
  const int mt = i / kTcBM, il = i - mt * kTcBM;
  const int kc = k / kTcBK, kl = k - kc * kTcBK;
  if (i >= ((M + kTcBM - 1) / kTcBM) * kTcBM) return;
  const float2 v = (i < M && k < K) ? A[(size_t)k * lda + i] : make_float2(0.f, 0.f);
  unsigned char* chunk = Apk + ((size_t)mt * nkc + kc) * kTcChunkA;
  float h, l;
  tf32_split(v.x, h, l);
  *reinterpret_cast<float*>(chunk + kmajor_off(2 * il, kl)) = h;
  *reinterpret_cast<float*>(chunk + kTcApart + kmajor_off(2 * il, kl)) = l;
  tf32_split(v.y, h, l);
  *reinterpret_cast<float*>(chunk + kmajor_off(2 * il + 1, kl)) = h;
  *reinterpret_cast<float*>(chunk + kTcApart + kmajor_off(2 * il + 1, kl)) = l;
}

// B (K x N complex) -> Bpk[nt][kc] = {re hi, re lo, im hi, im lo} chunks.
// grid: (ceil(N / 64) * 64 x ceil(nkc * 16 / 64)), 64 threads
__global__ void pack_b_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int nkc,
                              unsigned char* __restrict__ Bpk) {
  const int n = blockIdx.x;                             // complex column
  const int k = blockIdx.y * blockDim.x + threadIdx.x;  // 0 .. nkc * 16 - 1
  if (k >= nkc * kTcBK) return;
  const int nt = n / kTcBN, nl = n - nt * kTcBN;
  const int kc = k / kTcBK, kl = k - kc * kTcBK;
  const float2 v = (k < K && n < N) ? B[(size_t)n * ldb + k] : make_float2(0.f, 0.f);
  unsigned char* chunk = Bpk + ((size_t)nt * nkc + kc) * kTcChunkB;
  const int off = kmajor_off(nl, kl);
  float h, l;
  tf32_split(v.x, h, l);
  *reinterpret_cast<float*>(chunk + off) = h;
  *reinterpret_cast<float*>(chunk + kTcBpart + off) = l;
  tf32_split(v.y, h, l);
  *reinterpret_cast<float*>(chunk + 2 * kTcBpart + off) = h;
  *reinterpret_cast<float*>(chunk + 3 * kTcBpart + off) = l;
}

// ---- the update --------------------------------------------------------------
// grid (ceil(M / 64), ceil(N / 64)), 128 threads, kTcSmem bytes of shared memory
__global__ void __launch_bounds__(kTcThreads, 3)
tc_cgemm_sub_kernel(float2* __restrict__ C, long long ldc, const unsigned char* __restrict__ Apk,
                    const unsigned char* __restrict__ Bpk, int M, int N, int nkc, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned long long* full = reinterpret_cast<unsigned long long*>(sm + 2 * kTcStage);
  unsigned long long* done = full + 2;
  unsigned* tslot = reinterpret_cast<unsigned*>(done + 2);
  int* s_ok = reinterpret_cast<int*>(tslot + 1);
  const int t = threadIdx.x, w = t >> 5;
  const int mt = blockIdx.x, nt = blockIdx.y;
  const int i0 = mt * kTcBM, n0 = nt * kTcBN;
  const unsigned char* asrc = Apk + (size_t)mt * nkc * kTcChunkA;
  const unsigned char* bsrc = Bpk + (size_t)nt * nkc * kTcChunkB;
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
        smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    mbar_init(&full[0]);
    mbar_init(&full[1]);
    mbar_init(&done[0]);
    mbar_init(&done[1]);
    asm volatile("fence.mbarrier_init.release.cluster;");
    *s_ok = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = *tslot;
  // kind::tf32: D f32 (bits 4-5 = 1), A/B tf32 (bits 7-9, 10-12 = 2), both
  // K-major, N >> 3 at bit 17, M >> 4 at bit 24
  const unsigned idesc =
      (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(kTcBN >> 3) << 17) | ((128u >> 4) << 24);
  if (t == 0) {
    // chunk c goes to stage c & 1: A (hi, lo) and B (four parts) are each
    // one contiguous block in the packed operands
    auto issue = [&](int c) {
      unsigned char* st = sm + (c & 1) * kTcStage;
      mbar_expect_tx(&full[c & 1], kTcStage);
      bulk_copy(st, asrc + (size_t)c * kTcChunkA, kTcChunkA, &full[c & 1]);
      bulk_copy(st + kTcChunkA, bsrc + (size_t)c * kTcChunkB, kTcChunkB, &full[c & 1]);
    };
    issue(0);
    if (nkc > 1) issue(1);
    const unsigned d1 = tmem, d2 = tmem + kTcBN;
    for (int c = 0; c < nkc; ++c) {
      const int s = c & 1;
      const unsigned ph = (c >> 1) & 1;
      if (!mbar_wait(&full[s], ph)) {
        *s_ok = 0;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const unsigned base = smem_u32(sm + s * kTcStage);
      const unsigned ah = base, al = base + kTcApart;
      const unsigned brh = base + kTcChunkA, brl = brh + kTcBpart;
      const unsigned bih = brh + 2 * kTcBpart, bil = brh + 3 * kTcBpart;
#pragma unroll
      for (int ks = 0; ks < kTcBK / 8; ++ks) {
        const unsigned o = 256u * ks;  // K = 8 tf32 = two core matrices
        const unsigned acc = (c == 0 && ks == 0) ? 0u : 1u;
        mma_tf32(d1, ah + o, brh + o, idesc, acc);
        mma_tf32(d1, ah + o, brl + o, idesc, 1u);
        mma_tf32(d1, al + o, brh + o, idesc, 1u);
        mma_tf32(d2, ah + o, bih + o, idesc, acc);
        mma_tf32(d2, ah + o, bil + o, idesc, 1u);
        mma_tf32(d2, al + o, bih + o, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&done[s])));
      if (c + 2 < nkc) {  // refill this stage once its MMAs have read it
        if (!mbar_wait(&done[s], ph)) {
          *s_ok = 0;
          break;
        }
        issue(c + 2);
      }
    }
  }
  __syncthreads();
  // the last commit covers every MMA of the tile
  bool ok = *s_ok != 0;
  if (ok) ok = mbar_wait(&done[(nkc - 1) & 1], ((nkc - 1) >> 1) & 1);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (__syncthreads_or(!ok)) {
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
      unsigned dv1[16], dv2[16];
      TC_LD16(dv1, lanes + j0);
      TC_LD16(dv2, lanes + kTcBN + j0);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const float p2 = __shfl_xor_sync(0xffffffffu, __uint_as_float(dv2[u]), 1);
        const float o = __uint_as_float(dv1[u]) + (c ? p2 : -p2);
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

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

size_t tc_pack_bytes(int M, int N, int K) {
  const size_t nkc = (size_t)(K + kTcBK - 1) / kTcBK;
  const size_t mt = (size_t)(M + kTcBM - 1) / kTcBM, nt = (size_t)(N + kTcBN - 1) / kTcBN;
  return align256(mt * nkc * kTcChunkA) + align256(nt * nkc * kTcChunkB);
}

int launch_tc_cgemm_sub(float2* C, long long ldc, const float2* A, long long lda,
                        const float2* B, long long ldb, int M, int N, int K, void* pack,
                        size_t pack_bytes, int* status, cudaStream_t s) {
  static const cudaError_t attr = cudaFuncSetAttribute(
      tc_cgemm_sub_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (attr != cudaSuccess) return BEM2D_ERR_CUDA;
  if (M <= 0 || N <= 0 || K <= 0) return BEM2D_OK;
  if (!pack || tc_pack_bytes(M, N, K) > pack_bytes) return BEM2D_ERR_ARG;
  const int nkc = (K + kTcBK - 1) / kTcBK;
  const int mt = (M + kTcBM - 1) / kTcBM, nt = (N + kTcBN - 1) / kTcBN;
  unsigned char* Apk = static_cast<unsigned char*>(pack);
  unsigned char* Bpk = Apk + align256((size_t)mt * nkc * kTcChunkA);
  pack_a_kernel<<<dim3((mt * kTcBM + 127) / 128, nkc * kTcBK), 128, 0, s>>>(A, lda, M, K, nkc,
                                                                            Apk);
  pack_b_kernel<<<dim3(nt * kTcBN, (nkc * kTcBK + 63) / 64), 64, 0, s>>>(B, ldb, K, N, nkc, Bpk);
  tc_cgemm_sub_kernel<<<dim3(mt, nt), kTcThreads, kTcSmem, s>>>(C, ldc, Apk, Bpk, M, N, nkc,
                                                                status);
  return cudaPeekAtLastError() == cudaSuccess ? BEM2D_OK : BEM2D_ERR_CUDA;
}

}  // namespace bem2d_gpu
