// Float-float kernel composition shared by the mixed-precision assembly
// kernels: the wavenumber constants and K(x, y) of the four integral
// operators (lib/bem2d_kernel.cpp:15-112) from J0, Y0, J1, Y1 at k|x - y|.
#pragma once

#include "bem2d_gpu.h"
#include "hankel_ff.cuh"

namespace bem2d_gpu {

struct KConstFF {
  ff k, invk, kq, eq, amp0;
};

inline KConstFF make_kconst(double k, double eta) {
  KConstFF kc;
  kc.k = ff_from_double(k);
  kc.invk = ff_from_double(1.0 / k);
  kc.kq = ff_from_double(0.25 * k);
  kc.eq = ff_from_double(0.25 * eta);
  kc.amp0 = ff_from_double(0.79788456080286535588);  // sqrt(2/pi)
  return kc;
}

// Kernel value of entry (x, y) from the Bessel values at k|x - y|.  cd: the
// normal factor over d (n_x . (x - y)/d for the adjoint double layer and the
// combined operator, n_y . (y - x)/d for the double layer); unused by SINGLE.
template <int KERNEL>
__device__ __forceinline__ ffc kernel_from_bessel(const BesselFF& b, ff cd, const KConstFF& kc) {
  ffc K;
  if (KERNEL == BEM2D_KERNEL_SINGLE) {
    // (i/4) (J0 + i Y0)
    K.re = ff_scale2(ff_neg(b.y0), 0.25f);
    K.im = ff_scale2(b.j0, 0.25f);
  } else {
    // -i (k/4) c (J1 + i Y1)
    const ff c = ff_mul(cd, kc.kq);
    K.re = ff_mul(c, b.y1);
    K.im = ff_neg(ff_mul(c, b.j1));
    if (KERNEL == BEM2D_KERNEL_COMBINED) {
      // + (eta/4) (J0 + i Y0)
      K.re = ff_add_fast(K.re, ff_mul(kc.eq, b.j0));
      K.im = ff_add_fast(K.im, ff_mul(kc.eq, b.y0));
    }
  }
  return K;
}

// Device copy of the e^{i x} reduction table of expi_ff (256 floats), made
// once per device (the current one); thread-safe.  nullptr if it could not
// be allocated.
const float* expi_table_dev();

}  // namespace bem2d_gpu
