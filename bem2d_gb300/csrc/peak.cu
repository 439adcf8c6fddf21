// Measurement helper: sustained FMA throughput of the FP64 and FP32 pipes
// (a register-resident chain per thread, no memory traffic), used as the
// roofline denominator of the assembly kernels, which are bound by those
// pipes rather than by HBM or the tensor cores.
#include "common.cuh"

namespace bem2d_gpu {

template <typename R>
__global__ void fma_chain_kernel(R seed, int iters, R* out) {
  R a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + (R)(threadIdx.x + i);
  const R m = (R)0.999999, c = (R)1e-7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], m, c);
  }
  R s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == (R)-1) out[0] = s;  // keeps the chain live; never true
}

}  // namespace bem2d_gpu

using namespace bem2d_gpu;

extern "C" int bem2d_fma_peak(int precision, double* tflops) {
  if (!tflops) return BEM2D_ERR_ARG;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  void* out = nullptr;
  if (cudaMalloc(&out, 64) != cudaSuccess) return BEM2D_ERR_NOMEM;
  const int threads = 256, blocks = nsm * 8;
  const int iters = precision == BEM2D_PREC_FP64 ? 4096 : 65536;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (precision == BEM2D_PREC_FP64)
      fma_chain_kernel<double><<<blocks, threads>>>(1.0, iters, (double*)out);
    else
      fma_chain_kernel<float><<<blocks, threads>>>(1.0f, iters, (float*)out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return BEM2D_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3) / 1e12;
  return BEM2D_OK;
}
