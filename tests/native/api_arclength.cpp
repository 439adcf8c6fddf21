// Prints the element parameters AnalyticCurve assigns (this build's C++ API,
// host only): for each library curve, the equal-arc partition
// AnalyticCurve(n, curve) and the graded one AnalyticCurve(ppw, k, curve,
// closed, L, sigma).  One line per partition: a label, then t_start of every
// element and the last t_end.  Read by tests/test_cpp_api.py.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "bem2d.h"

static void dump(const std::string& label, bem2d::AnalyticCurve& ac) {
  bem2d::pGeometry g = ac.GetGeometry();
  std::printf("%s", label.c_str());
  const std::vector<bem2d::pElement>& el = g->elements();
  for (std::size_t i = 0; i < el.size(); ++i) {
    const bem2d::AnalyticCurveElement* e =
        dynamic_cast<const bem2d::AnalyticCurveElement*>(el[i].get());
    std::printf(" %.17g", e->tstart());
    if (i + 1 == el.size()) std::printf(" %.17g", e->tend());
  }
  std::printf("\n");
}

int main() {
  const double pi = 3.14159265358979323846;
  std::vector<std::pair<std::string, bem2d::pCurve> > curves;
  curves.push_back(std::make_pair(std::string("circle"), bem2d::pCurve(new bem2d::Circle)));
  curves.push_back(std::make_pair(std::string("kite"), bem2d::pCurve(new bem2d::Kite)));
  curves.push_back(std::make_pair(std::string("trefoil"), bem2d::pCurve(new bem2d::Trefoil)));
  curves.push_back(std::make_pair(std::string("ellipse"), bem2d::pCurve(new bem2d::Ellipse(1.5))));
  curves.push_back(std::make_pair(std::string("ellipsearc"),
                                  bem2d::pCurve(new bem2d::EllipseArc(2.0, 1.0, 0.3, 0.3 + 1.5 * pi))));
  curves.push_back(std::make_pair(std::string("invellipse"),
                                  bem2d::pCurve(new bem2d::InvEllipse(0.2))));
  bem2d::freqtype k = {6.0, 0.0};
  for (std::size_t c = 0; c < curves.size(); ++c) {
    bem2d::AnalyticCurve eq(13, curves[c].second, 1);
    dump(curves[c].first + " equal", eq);
    bem2d::AnalyticCurve gr(4, k, curves[c].second, 1, 3, 0.15);
    dump(curves[c].first + " graded", gr);
  }
  return 0;
}
