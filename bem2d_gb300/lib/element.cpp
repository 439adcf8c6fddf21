// bem2d C++ API (GB300 build): element constructors.
#include "bem2d_element.h"

namespace bem2d {

ConstElement::ConstElement(const Point& p1, const Point& p2, std::size_t index)
    : p1_(p1), p2_(p2), d_(p2 - p1) {
  set_index(index);
}

AnalyticCurveElement::AnalyticCurveElement(double t1, double t2, pCurve curve, std::size_t index)
    : curve_(curve), tstart_(t1), tend_(t2) {
  set_index(index);
}

}  // namespace bem2d
