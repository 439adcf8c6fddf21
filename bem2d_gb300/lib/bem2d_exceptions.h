// bem2d C++ API (GB300 build): exception tags thrown by the library, named as
// in the reference (lib/bem2d_exceptions.h).  UnsupportedError (new) marks
// inputs this build does not evaluate (complex wavenumbers with arg k below
// -pi/3, user-defined element or curve classes, complex-valued bases, full
// spectra).
#ifndef BEM2D_EXCEPTIONS_H
#define BEM2D_EXCEPTIONS_H

#include <stdexcept>
#include <string>

namespace bem2d {

class ArrayMismatch {};
class LapackError {};
class IntervalException {};
class ParameterException {};
class SizeError {};

class UnsupportedError : public std::runtime_error {
 public:
  explicit UnsupportedError(const std::string& what) : std::runtime_error(what) {}
};

// A CUDA or device-side failure reported by the GPU library.
class GpuError : public std::runtime_error {
 public:
  GpuError(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

}  // namespace bem2d

#endif
