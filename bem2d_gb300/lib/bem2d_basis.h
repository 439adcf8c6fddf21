// bem2d C++ API (GB300 build): basis functions on the reference interval.
#ifndef BEM2D_BASIS_H
#define BEM2D_BASIS_H

#include "bem2d_defs.h"

namespace bem2d {

class Basis {
 public:
  virtual complex operator()(double t) const = 0;
  virtual ~Basis() {}
};

typedef std::shared_ptr<Basis> pBasis;

}  // namespace bem2d

#endif
