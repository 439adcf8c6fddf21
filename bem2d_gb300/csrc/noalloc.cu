// bem2d_solve_system_noalloc: the complex128 dense solve x = A^{-1} b of
// bem2d_solve_system (BEM2D_PREC_FP64) for callers that must not allocate
// device memory.
//
// Who needs it: a solver called from inside a larger GPU application whose
// memory manager owns the device (a pool that reserves its budget up front
// and forbids direct cudaMalloc, or a process that already holds nearly all
// of the device's memory), and latency-critical loops in which cudaMalloc and
// cudaFree are unacceptable because they can synchronise the whole device.
// The regular entry points grow a per-context workspace with cudaMalloc on
// first use; this one never does.
//
// Where its memory comes from: every buffer the factorisation and the
// triangular solves use (the copy of A that is factored in place, the
// right-hand side, the pivots, the panel exchange slots, the permutation and
// the inverted diagonal blocks) lives in one file-scope __device__ array of
// kScratchBytes, sized for n <= BEM2D_NOALLOC_MAX_N.  That array is part of
// this library's device image: the CUDA runtime reserves it when the module
// is loaded, not this function.  Larger n is rejected with BEM2D_ERR_ARG and
// a message naming the limit; bem2d_noalloc_scratch_fits() reports whether
// the largest accepted n fits the array (a host-side check for the tests).
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress (which may load this
// module) and caches it; later calls reuse the cached address.  That first
// call should therefore come before any stream capture begins.
//
// Sharing: all calls on a device (from every context and thread) use the same
// array, and it keeps whatever the previous call left there.  The values that
// must start at zero (the zero-pivot flag, the wait-timeout flag and the panel
// exchange slots) are cleared by the factorisation at the start of every
// call; everything else is written before it is read.  Two calls whose GPU
// work overlaps (different streams, or different host threads without
// ordering between them) race on the array and give wrong results: callers
// must serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "common.cuh"

namespace bem2d_gpu {
namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxDevices = 64;
// n = 1024: A 16 MiB + b 16 KiB + x 16 KiB + pivots 4 KiB + panel slots
// 2.03 MiB + permutation and diagonal-block inverses 2.0 MiB = 20.07 MiB;
// 21 MiB leaves room for the 256-byte alignment of each part.
constexpr size_t kScratchBytes = (size_t)21 << 20;

static_assert(BEM2D_NOALLOC_MAX_N > 0, "BEM2D_NOALLOC_MAX_N must be positive");
static_assert((size_t)BEM2D_NOALLOC_MAX_N * BEM2D_NOALLOC_MAX_N * sizeof(double2) < kScratchBytes,
              "scratch array too small for BEM2D_NOALLOC_MAX_N");

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Byte offsets of the parts within the array for n unknowns.
struct Layout {
  size_t lu, vec, xv, ints, slots, aux, aux_bytes, total;
};

Layout layout(int n) {
  Layout L;
  L.lu = 0;
  L.vec = L.lu + round_up(sizeof(double2) * (size_t)n * n);
  L.xv = L.vec + round_up(sizeof(double2) * (size_t)n);
  L.ints = L.xv + round_up(sizeof(double2) * (size_t)n);
  L.slots = L.ints + round_up(sizeof(int) * ((size_t)n + 8));
  L.aux = L.slots + round_up(lu_scratch_bytes(n));
  L.aux_bytes = lu_aux_bytes(n, sizeof(double2));
  L.total = L.aux + round_up(L.aux_bytes);
  return L;
}

// Device address of the array on `device` (the current device), looked up
// once per device.
int scratch_on(bem2d_ctx* c, int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices)
    return ctx_fail(c, BEM2D_ERR_ARG, "device ordinal out of range for the no-allocation solve");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      char msg[256];
      std::snprintf(msg, sizeof msg, "cudaGetSymbolAddress of the solve scratch array: %s",
                    cudaGetErrorString(e));
      cudaGetLastError();
      return ctx_fail(c, BEM2D_ERR_CUDA, msg);
    }
    g_scratch_ptr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
  return BEM2D_OK;
}

int cuda_fail(bem2d_ctx* c, const char* what, cudaError_t e) {
  char msg[256];
  std::snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  return ctx_fail(c, BEM2D_ERR_CUDA, msg);
}

}  // namespace
}  // namespace bem2d_gpu

extern "C" int bem2d_solve_system_noalloc(bem2d_ctx* c, int n, const void* A, int64_t lda,
                                          const void* b, void* x, bem2d_solve_info* info) {
  using namespace bem2d_gpu;
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !b || !x) return ctx_fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (lda < n) return ctx_fail(c, BEM2D_ERR_ARG, "lda < n");
  if (n > BEM2D_NOALLOC_MAX_N) {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "n = %d exceeds the no-allocation solve limit BEM2D_NOALLOC_MAX_N = %d; "
                  "use bem2d_solve_system", n, BEM2D_NOALLOC_MAX_N);
    return ctx_fail(c, BEM2D_ERR_ARG, msg);
  }
  const Layout L = layout(n);
  if (L.total > kScratchBytes)
    return ctx_fail(c, BEM2D_ERR_ARG, "the LU work buffers do not fit the scratch array");
  const int device = ctx_device(c);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(c, "cudaSetDevice", e);
  unsigned char* base = nullptr;
  int rc = scratch_on(c, device, &base);
  if (rc) return rc;
  const cudaStream_t s = ctx_stream(c);

  double2* LU = reinterpret_cast<double2*>(base + L.lu);
  double2* v = reinterpret_cast<double2*>(base + L.vec);   // b
  double2* xv = reinterpret_cast<double2*>(base + L.xv);   // x
  int* ints = reinterpret_cast<int*>(base + L.ints);
  LuWork w;
  w.info = ints;
  w.status = ints + 1;
  w.ipiv = ints + 8;
  w.scratch = base + L.slots;
  w.scratch_bytes = lu_scratch_bytes(n);
  w.dinv = base + L.aux;
  w.perm = reinterpret_cast<int*>(base + L.aux + L.aux_bytes - 256 - sizeof(int) * (size_t)n);

  // A and b may be host or device memory: plain copies into the array.
  e = cudaMemcpy2DAsync(LU, sizeof(double2) * n, A, sizeof(double2) * lda, sizeof(double2) * n,
                        n, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(c, "copy of A into the scratch array", e);
  e = cudaMemcpyAsync(v, b, sizeof(double2) * n, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(c, "copy of b into the scratch array", e);

  // lu_factor zeroes the pivot flag, the timeout flag and the panel slots.
  bem2d_solve_info rep{0, 0, 0.0};
  int hinfo[2] = {0, 0};
  if ((rc = lu_factor<double2>(LU, n, n, w, s, ctx_launches(c))))
    return ctx_fail(c, rc, "LU launch failed");
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, "LU kernels", e);
  e = cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, "LU status read", e);
  if (hinfo[1]) return ctx_fail(c, BEM2D_ERR_TIMEOUT, "LU panel barrier timed out");
  rep.info = hinfo[0];
  if (info) *info = rep;
  if (hinfo[0]) {
    char msg[64];
    std::snprintf(msg, sizeof msg, "zero pivot at column %d", hinfo[0]);
    return ctx_fail(c, hinfo[0], msg);
  }
  if ((rc = lu_solve<double2>(LU, n, n, w, v, xv, s, ctx_launches(c))))
    return ctx_fail(c, rc, "triangular solve launch failed");
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, "triangular solve kernels", e);
  e = cudaMemcpyAsync(x, xv, sizeof(double2) * n, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(c, "copy of x out of the scratch array", e);
  e = cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, "solve status read", e);
  if (hinfo[1]) return ctx_fail(c, BEM2D_ERR_TIMEOUT, "triangular solve wait timed out");
  return BEM2D_OK;
}

// Host-side check that the parts for n = BEM2D_NOALLOC_MAX_N fit the array:
// 1 if they do (their byte total in *total), 0 if not.
extern "C" int bem2d_noalloc_scratch_fits(int64_t* total, int64_t* capacity) {
  using namespace bem2d_gpu;
  const Layout L = layout(BEM2D_NOALLOC_MAX_N);
  if (total) *total = (int64_t)L.total;
  if (capacity) *capacity = (int64_t)kScratchBytes;
  return L.total <= kScratchBytes ? 1 : 0;
}
