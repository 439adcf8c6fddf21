// bem2d C++ API (GB300 build): point-in-polygon test (even-odd ray rule).
#ifndef BEM2D_PNPOLY_H
#define BEM2D_PNPOLY_H

namespace bem2d {
int pnpoly(int nvert, double* vertx, double* verty, double testx, double testy);
}

#endif
