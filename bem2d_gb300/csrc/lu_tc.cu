// Trailing update of the complex64 LU on the 5th-generation tensor cores:
// C -= A B (complex64, column-major, arbitrary leading dimensions), as
// tcgen05.mma kind::tf32 with FP32 accumulators in tensor memory.
//
// Complex arithmetic as one real product.  The complex M x K operand A is
// read as a real (2M) x K matrix A' whose rows 2i and 2i + 1 hold re and im
// of row i (that is how complex column-major data lies in memory).  The
// complex K x N operand B becomes the real N' x K operand [B_r; B_i] with
// N' = 2N (the real parts of the tile's columns, then the imaginary parts),
// so one MMA of N = 256 gives D = A' [B_r B_i] with
//   D1 = A' B_r (columns 0..127),  D2 = A' B_i (columns 128..255),
//   re C_i = D1[2i] - D2[2i+1],   im C_i = D2[2i] + D1[2i+1].
// A tile is 64 complex rows (128 real rows = the MMA's M) by 128 complex
// columns: 256 tensor-memory columns per accumulator.
//
// Accuracy (3xTF32): every FP32 operand x is split into hi = x rounded to
// the nearest TF32 value (10 mantissa bits) and lo = x - hi (exact); each
// product is accumulated as hi*hi + hi*lo + lo*hi, which keeps about 21 bits
// per product - the accuracy of the FP32 update it replaces, so the LU keeps
// the quality the FP64 refinement expects.  With passes = 1 (1xTF32) only
// hi*hi is issued: a third of the tensor work, products to about 2^-11
// relative, for systems whose condition number the refinement tolerates at
// that precision.
//
// Operands are packed once per update (pack_a_kernel, pack_b_kernel): split
// into hi/lo and laid out, per tile and per chunk of 16 along K, exactly as
// the MMA reads them from shared memory - the K-major, non-swizzled
// canonical layout (core matrices of 8 rows x 16 bytes, 128 bytes from one
// core matrix to the next along K, 512 bytes from one group of 8 rows to the
// next).  A chunk is then one contiguous block per operand: 16 KB of A'
// (hi, lo) and 32 KB of B (hi, lo).
//
// The update kernel is persistent (one CTA per SM, tiles in a static
// round-robin) and warp-specialised:
//   warp 0      producer: two bulk copies (cp.async.bulk, completion counted
//               in bytes on the stage's `full` mbarrier) per chunk into a
//               ring of four 48 KB shared-memory stages;
//   warp 1      MMA issuer: six MMAs per chunk (two K-steps of 8, 3xTF32);
//               tcgen05.commit frees the stage (`empty`) once its MMAs have
//               read it, and marks the tile's accumulator complete (`acc_full`);
//   warps 2-17  epilogue: tcgen05.ld of the accumulator (warp w reads TMEM
//               lanes 32 (w % 4) ..., four warps per lane quarter, one per
//               quarter of the columns), rows 2i / 2i + 1 combined with one
//               shuffle; each thread loads its 32 C values before it waits
//               for the tile's accumulator (the loads overlap the tile's
//               MMAs; the next tile's C is prefetched into L2 meanwhile), C
//               is written with coalesced 128-byte accesses; then `acc_empty`.
// The two accumulators alternate between tiles (512 TMEM columns), so the
// epilogue of one tile overlaps the MMAs of the next.  Every wait is bounded
// (2 s of device time): on timeout the status flag is set, every role stops,
// the producer waits (bounded) for its copies in flight and the MMA thread
// for its MMAs, and the tensor memory is released before the kernel returns.
#include <cuda_runtime.h>

#include "common.cuh"

namespace bem2d_gpu {
namespace {

constexpr int kTcBM = 64;    // complex rows per tile (128 real rows = MMA M)
constexpr int kTcBN = 128;   // complex columns per tile (MMA N = 256: re, im)
constexpr int kTcBK = 16;    // K per chunk (two MMAs of K = 8)
constexpr int kTcStages = 4;
constexpr int kTcThreads = 576;  // producer warp, MMA warp, 16 epilogue warps
constexpr int kTcEpiThreads = 512;
constexpr int kCoreBytes = 128;                   // 8 rows x 16 bytes
constexpr int kTcSBO = (kTcBK / 4) * kCoreBytes;  // 512
constexpr int kTcApart = 2 * kTcBM * kTcBK * 4;   // 8 KB: 128 real rows x 16
constexpr int kTcBpart = 2 * kTcBN * kTcBK * 4;   // 16 KB: 256 rows x 16
constexpr int kTcChunkA = 2 * kTcApart;           // hi, lo
constexpr int kTcChunkB = 2 * kTcBpart;           // hi, lo
constexpr int kTcStage = kTcChunkA + kTcChunkB;   // 48 KB
constexpr int kTcBarOff = kTcStages * kTcStage;   // 192 KB
constexpr int kTcSmem = kTcBarOff + 256;
constexpr unsigned kTcAcc = 2 * kTcBN;            // TMEM columns per accumulator
constexpr unsigned long long kTcWaitNs = 2000000000ull;  // 2 s

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
// hi = x rounded to 10 mantissa bits (ties away from zero), lo = x - hi
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
  lo = x - hi;
}

__device__ __forceinline__ void mma_tf32(unsigned d, unsigned a, unsigned b, unsigned idesc,
                                         unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(smem_desc(a)), "l"(smem_desc(b)), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(unsigned long long* m) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(m)));
}

__device__ __forceinline__ void mbar_init(unsigned long long* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)),
               "r"(bytes));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* m) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* m, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for phase `parity` of the mbarrier (try_wait suspends the
// thread for a short while between polls): false after kTcWaitNs of device
// time, or, if `abort` is given, as soon as another role has given up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* m, unsigned parity,
                                          const volatile int* abort) {
  if (mbar_test(m, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned it = 1;; ++it) {
    if (mbar_test(m, parity)) return true;
    if ((it & 15u) == 0u) {
      if (abort && *abort) return false;
      if (global_ns() - t0 > kTcWaitNs) return false;
    }
  }
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
                              int passes, unsigned char* __restrict__ Apk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // complex row
  const int k = blockIdx.y;                             // 0 .. nkc * 16 - 1
  const int mt = i / kTcBM, il = i - mt * kTcBM;
  const int kc = k / kTcBK, kl = k - kc * kTcBK;
  if (i >= ((M + kTcBM - 1) / kTcBM) * kTcBM) return;
  const float2 v = (i < M && k < K) ? A[(size_t)k * lda + i] : make_float2(0.f, 0.f);
  unsigned char* chunk = Apk + ((size_t)mt * nkc + kc) * kTcChunkA;
  float h, l;
  float h2, l2;
  tf32_split(v.x, h, l);
  tf32_split(v.y, h2, l2);
  *reinterpret_cast<float*>(chunk + kmajor_off(2 * il, kl)) = h;
  *reinterpret_cast<float*>(chunk + kmajor_off(2 * il + 1, kl)) = h2;
  if (passes > 1) {
    *reinterpret_cast<float*>(chunk + kTcApart + kmajor_off(2 * il, kl)) = l;
    *reinterpret_cast<float*>(chunk + kTcApart + kmajor_off(2 * il + 1, kl)) = l2;
  }
}

// B (K x N complex) -> Bpk[nt][kc] = {hi, lo} chunks of kTcBpart bytes, each
// with rows 0..127 = re and rows 128..255 = im of the tile's 128 columns.
// grid: (ceil(N / 128) * 128 x ceil(nkc * 16 / 64)), 64 threads
__global__ void pack_b_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int nkc,
                              int passes, unsigned char* __restrict__ Bpk) {
  const int n = blockIdx.x;                             // complex column
  const int k = blockIdx.y * blockDim.x + threadIdx.x;  // 0 .. nkc * 16 - 1
  if (k >= nkc * kTcBK) return;
  const int nt = n / kTcBN, nl = n - nt * kTcBN;
  const int kc = k / kTcBK, kl = k - kc * kTcBK;
  const float2 v = (k < K && n < N) ? B[(size_t)n * ldb + k] : make_float2(0.f, 0.f);
  unsigned char* chunk = Bpk + ((size_t)nt * nkc + kc) * kTcChunkB;
  const int ore = kmajor_off(nl, kl), oim = kmajor_off(kTcBN + nl, kl);
  float h, l;
  float h2, l2;
  tf32_split(v.x, h, l);
  tf32_split(v.y, h2, l2);
  *reinterpret_cast<float*>(chunk + ore) = h;
  *reinterpret_cast<float*>(chunk + oim) = h2;
  if (passes > 1) {
    *reinterpret_cast<float*>(chunk + kTcBpart + ore) = l;
    *reinterpret_cast<float*>(chunk + kTcBpart + oim) = l2;
  }
}

// ---- the update --------------------------------------------------------------
// grid: min(tiles, SMs) persistent CTAs, kTcThreads threads, kTcSmem bytes
// of shared memory (one CTA per SM).  Tile t: mt = t % mtiles, nt = t / mtiles.
__global__ void __launch_bounds__(kTcThreads, 1)
tc_cgemm_sub_kernel(float2* __restrict__ C, long long ldc, const unsigned char* __restrict__ Apk,
                    const unsigned char* __restrict__ Bpk, int M, int N, int nkc, int mtiles,
                    int ntiles, int passes, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned long long* full = reinterpret_cast<unsigned long long*>(sm + kTcBarOff);
  unsigned long long* empty = full + kTcStages;
  unsigned long long* acc_full = empty + kTcStages;
  unsigned long long* acc_empty = acc_full + 2;
  unsigned long long* fin = acc_empty + 2;
  unsigned* tslot = reinterpret_cast<unsigned*>(fin + 1);
  volatile int* s_abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const int ntl = mtiles * ntiles;
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
        smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 32) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&acc_full[a], 1);
      mbar_init(&acc_empty[a], kTcEpiThreads);
    }
    mbar_init(fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    *s_abort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = *tslot;
  // kind::tf32: D f32 (bits 4-5 = 1), A/B tf32 (bits 7-9, 10-12 = 2), both
  // K-major, N >> 3 at bit 17, M >> 4 at bit 24
  const unsigned idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((kTcAcc >> 3) << 17) |
                         ((128u >> 4) << 24);
  bool ok = true;
  if (w == 0) {
    if (lane == 0) {  // ---- producer
      int it = 0;
      for (int tile = blockIdx.x; tile < ntl && ok; tile += gridDim.x) {
        const int mt = tile % mtiles, nt = tile / mtiles;
        const unsigned char* asrc = Apk + (size_t)mt * nkc * kTcChunkA;
        const unsigned char* bsrc = Bpk + (size_t)nt * nkc * kTcChunkB;
        for (int c = 0; c < nkc; ++c, ++it) {
          const int s = it % kTcStages;
          const unsigned ph = (unsigned)(it / kTcStages) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, s_abort)) {
            ok = false;
            break;
          }
          unsigned char* st = sm + s * kTcStage;
          // 1xTF32: the hi halves only (the first half of each packed chunk)
          const unsigned abytes = passes > 1 ? kTcChunkA : kTcApart;
          const unsigned bbytes = passes > 1 ? kTcChunkB : kTcBpart;
          mbar_expect_tx(&full[s], abytes + bbytes);
          bulk_copy(st, asrc + (size_t)c * kTcChunkA, abytes, &full[s]);
          bulk_copy(st + kTcChunkA, bsrc + (size_t)c * kTcChunkB, bbytes, &full[s]);
        }
      }
      if (!ok) {
        *s_abort = 1;
        // let the copies in flight land before the CTA's shared memory goes
        for (int q = it - 1; q >= 0 && q >= it - kTcStages; --q)
          mbar_wait(&full[q % kTcStages], (unsigned)(q / kTcStages) & 1u, nullptr);
      }
    }
  } else if (w == 1) {
    if (lane == 0) {  // ---- MMA issuer
      int it = 0, j = 0;
      for (int tile = blockIdx.x; tile < ntl && ok; tile += gridDim.x, ++j) {
        const int a = j & 1;
        const unsigned aph = (unsigned)(j >> 1) & 1u;
        if (!mbar_wait(&acc_empty[a], aph ^ 1u, s_abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const unsigned d = tmem + (unsigned)a * kTcAcc;
        for (int c = 0; c < nkc; ++c, ++it) {
          const int s = it % kTcStages;
          const unsigned ph = (unsigned)(it / kTcStages) & 1u;
          if (!mbar_wait(&full[s], ph, s_abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const unsigned base = smem_u32(sm + s * kTcStage);
          const unsigned ah = base, al = base + kTcApart;
          const unsigned bh = base + kTcChunkA, bl = bh + kTcBpart;
#pragma unroll
          for (int ks = 0; ks < kTcBK / 8; ++ks) {
            const unsigned o = 256u * ks;  // K = 8 tf32 = two core matrices
            mma_tf32(d, ah + o, bh + o, idesc, (c == 0 && ks == 0) ? 0u : 1u);
            if (passes > 1) {
              mma_tf32(d, ah + o, bl + o, idesc, 1u);
              mma_tf32(d, al + o, bh + o, idesc, 1u);
            }
          }
          mma_commit(&empty[s]);  // the stage may be refilled once these MMAs read it
        }
        if (!ok) break;
        mma_commit(&acc_full[a]);
      }
      if (!ok) *s_abort = 1;
      // every MMA issued has completed before the tensor memory is released
      mma_commit(fin);
      if (!mbar_wait(fin, 0u, nullptr)) ok = false;
    }
  } else {  // ---- epilogue, warps 2-17
    // four warps per TMEM lane quarter (warp w may access lanes 32 (w % 4)
    // ..), one for each quarter of the tile's 128 columns
    const int ew = w - 2, q = w & 3, part = ew >> 2;
    const int tl = q * 32 + lane;
    const int i = tl >> 1, cc = tl & 1;  // real row tl = 2i + cc
    float* Cf = reinterpret_cast<float*>(C);
    // the next tile's C columns into L2 while this tile's MMAs run: thread
    // et covers 128 of the 512 bytes of column et / 4 of the tile
    auto prefetch = [&](int tile) {
      if (tile >= ntl) return;
      const int et = ew * 32 + lane;
      const int i0 = (tile % mtiles) * kTcBM, n = (tile / mtiles) * kTcBN + (et >> 2);
      const int l = et & 3;
      if (n >= N || l * 16 >= M - i0) return;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(Cf + 2 * ((size_t)n * ldc + i0) + 32 * l));
    };
    prefetch(blockIdx.x);
    int j = 0;
    for (int tile = blockIdx.x; tile < ntl; tile += gridDim.x, ++j) {
      prefetch(tile + gridDim.x);
      const int mt = tile % mtiles, nt = tile / mtiles;
      const int i0 = mt * kTcBM, n0 = nt * kTcBN + part * (kTcBN / 4);
      const bool row_ok = i0 + i < M;
      float* crow = Cf + 2 * ((size_t)i0 + i) + cc;
      // this thread's 32 C values, loaded while the tile's MMAs still run
      const int nlim = row_ok ? min(kTcBN / 4, N - n0) : 0;
      const long long cstep = 2 * ldc;
      float cv[kTcBN / 4];
      {
        const float* pc = crow + (size_t)n0 * cstep;
        if (nlim == kTcBN / 4) {  // full tile: no per-column predicates
#pragma unroll
          for (int u = 0; u < kTcBN / 4; ++u, pc += cstep) cv[u] = *pc;
        } else {
#pragma unroll
          for (int u = 0; u < kTcBN / 4; ++u, pc += cstep) cv[u] = u < nlim ? *pc : 0.f;
        }
      }
      const int a = j & 1;
      const unsigned aph = (unsigned)(j >> 1) & 1u;
      if (!mbar_wait(&acc_full[a], aph, s_abort)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const unsigned lanes = tmem + (unsigned)a * kTcAcc + ((unsigned)(q * 32) << 16) +
                             (unsigned)(part * (kTcBN / 4));
      float* pw = crow + (size_t)n0 * cstep;
#pragma unroll
      for (int h = 0; h < kTcBN / 4; h += 16) {
        unsigned d1[16], d2[16];
        TC_LD16(d1, lanes + h);
        TC_LD16(d2, lanes + kTcBN + h);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        float o[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const float p2 = __shfl_xor_sync(0xffffffffu, __uint_as_float(d2[u]), 1);
          o[u] = cv[h + u] - (__uint_as_float(d1[u]) + (cc ? p2 : -p2));
        }
        if (nlim == kTcBN / 4) {
#pragma unroll
          for (int u = 0; u < 16; ++u, pw += cstep) *pw = o[u];
        } else {
#pragma unroll
          for (int u = 0; u < 16; ++u, pw += cstep)
            if (h + u < nlim) *pw = o[u];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(&acc_empty[a]);
    }
    if (!ok) *s_abort = 1;
  }
  if (!ok) atomicExch(status, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

#undef TC_LD16

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

}  // namespace

size_t tc_pack_bytes(int M, int N, int K) {
  const size_t nkc = (size_t)(K + kTcBK - 1) / kTcBK;
  const size_t mt = (size_t)(M + kTcBM - 1) / kTcBM, nt = (size_t)(N + kTcBN - 1) / kTcBN;
  return align256(mt * nkc * kTcChunkA) + align256(nt * nkc * kTcChunkB);
}

int launch_tc_cgemm_sub(float2* C, long long ldc, const float2* A, long long lda,
                        const float2* B, long long ldb, int M, int N, int K, void* pack,
                        size_t pack_bytes, int* status, cudaStream_t s, int max_ctas,
                        int passes) {
  static const cudaError_t attr = cudaFuncSetAttribute(
      tc_cgemm_sub_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (attr != cudaSuccess) return BEM2D_ERR_CUDA;
  if (M <= 0 || N <= 0 || K <= 0) return BEM2D_OK;
  if (!pack || tc_pack_bytes(M, N, K) > pack_bytes) return BEM2D_ERR_ARG;
  if (passes != 1 && passes != 3) return BEM2D_ERR_ARG;
  const int nkc = (K + kTcBK - 1) / kTcBK;
  const int mt = (M + kTcBM - 1) / kTcBM, nt = (N + kTcBN - 1) / kTcBN;
  unsigned char* Apk = static_cast<unsigned char*>(pack);
  unsigned char* Bpk = Apk + align256((size_t)mt * nkc * kTcChunkA);
  pack_a_kernel<<<dim3((mt * kTcBM + 127) / 128, nkc * kTcBK), 128, 0, s>>>(A, lda, M, K, nkc,
                                                                            passes, Apk);
  pack_b_kernel<<<dim3(nt * kTcBN, (nkc * kTcBK + 63) / 64), 64, 0, s>>>(B, ldb, K, N, nkc,
                                                                        passes, Bpk);
  const int grid = std::min(mt * nt, max_ctas > 0 ? max_ctas : num_sms());
  tc_cgemm_sub_kernel<<<grid, kTcThreads, kTcSmem, s>>>(C, ldc, Apk, Bpk, M, N, nkc, mt, nt,
                                                        passes, status);
  return cudaPeekAtLastError() == cudaSuccess ? BEM2D_OK : BEM2D_ERR_CUDA;
}

}  // namespace bem2d_gpu
