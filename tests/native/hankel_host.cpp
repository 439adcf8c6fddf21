// Host build of the device Hankel evaluator (bem2d_gb300/csrc/hankel.cuh),
// exported for accuracy tests against mpmath / scipy.
#include "hankel.cuh"

extern "C" void hankel01_d_host(int n, const double* x, double* out) {
  for (int i = 0; i < n; ++i)
    bem2d_gpu::hankel01_d(x[i], out + 4 * i, out + 4 * i + 1, out + 4 * i + 2,
                          out + 4 * i + 3);
}
