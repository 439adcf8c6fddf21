// bem2d C++ API (GB300 build): basic types and constants.
// Same names as the reference library's lib/bem2d_defs.h so that programs
// written against it compile unchanged; shared pointers are std::shared_ptr.
#ifndef BEM2D_DEFS_H
#define BEM2D_DEFS_H

#include <complex>
#include <memory>
#include <vector>

namespace bem2d {

typedef std::complex<double> complex;
typedef std::vector<double> dvector;
typedef std::vector<complex> cvector;

// Wavenumber k = re + i im (this build supports im == 0).
struct freqtype {
  double re;
  double im;
};

typedef std::shared_ptr<cvector> pcvector;
typedef std::shared_ptr<dvector> pdvector;

const double PI = 3.14159265358979323846;

}  // namespace bem2d

#endif
