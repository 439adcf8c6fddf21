// bem2d C++ API (GB300 build): output of field values on a plotting grid.
#ifndef BEM2D_OUTPUTHANDLER_H
#define BEM2D_OUTPUTHANDLER_H

#include <string>
#include <vector>

#include "bem2d_defs.h"
#include "bem2d_point.h"

namespace bem2d {

class OutputHandler {
 public:
  virtual ~OutputHandler() {}
  virtual void WriteIncident(const cvector&) {}
  virtual void WriteScattered(const cvector&) {}
  virtual void WriteFull(const cvector&) {}
  virtual void WriteAll(const cvector&, const cvector&, const cvector&) {}
  const std::vector<Point>& mesh() const { return mesh_; }
  void set_real(bool real) { real_ = real; }

 protected:
  pdvector RealData(const cvector& vals);
  pdvector ImagData(const cvector& vals);
  pdvector TurnToRealImag(const cvector& vals);
  std::vector<Point> mesh_;
  bool real_ = true;
  bool isroot_ = true;
};

typedef std::shared_ptr<OutputHandler> pOutputHandler;

// gnuplot data + script files <name>inc, <name>scatt, <name>full (and
// their _gplot scripts): real or imaginary parts on the mesh
class GplotOutput : public OutputHandler {
 public:
  GplotOutput(int xpts, int ypts, double ax, double bx, double ay, double by, std::string name);
  void WriteIncident(const cvector& vals);
  void WriteScattered(const cvector& vals);
  void WriteFull(const cvector& vals);
  void WriteAll(const cvector& valsincident, const cvector& valsscattered,
                const cvector& valsfull);

 private:
  std::string name_;
  int xpts_, ypts_;
};

}  // namespace bem2d

#endif
