// Host build of the device Hankel evaluators (bem2d_gb300/csrc/hankel.cuh,
// real argument; hankel_c.cuh, complex argument), exported for accuracy
// tests against mpmath / scipy.
#include "hankel_c.cuh"

extern "C" void hankel01_d_host(int n, const double* x, double* out) {
  for (int i = 0; i < n; ++i)
    bem2d_gpu::hankel01_d(x[i], out + 4 * i, out + 4 * i + 1, out + 4 * i + 2,
                          out + 4 * i + 3);
}

// z[2i], z[2i+1] = Re, Im of the i-th argument; out[4i..4i+3] = H0, H1.
extern "C" void hankel01_c_host(int n, const double* z, double* out) {
  for (int i = 0; i < n; ++i) {
    bem2d_gpu::cd h0, h1;
    bem2d_gpu::hankel01_c(bem2d_gpu::cd{z[2 * i], z[2 * i + 1]}, &h0, &h1);
    out[4 * i] = h0.re;
    out[4 * i + 1] = h0.im;
    out[4 * i + 2] = h1.re;
    out[4 * i + 3] = h1.im;
  }
}
