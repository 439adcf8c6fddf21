// bem2d C++ API (GB300 build): a boundary as a list of elements plus the basis
// functions on each element; FlatMap() numbers the unknowns (element-major,
// bases of one element in the order they were added).
#ifndef BEM2D_GEOMETRY_H
#define BEM2D_GEOMETRY_H

#include <cstddef>
#include <iostream>
#include <map>
#include <utility>
#include <vector>

#include "bem2d_basis.h"
#include "bem2d_element.h"
#include "bem2d_point.h"

namespace bem2d {

class Geometry;
typedef std::shared_ptr<Geometry> pGeometry;

class Geometry {
 public:
  typedef std::vector<std::map<std::size_t, pBasis> > basis_map;
  typedef std::vector<std::pair<pElement, pBasis> > flat_basis_map;

  // Elements as given; their links are kept.
  explicit Geometry(const std::vector<pElement>& elems);
  // Concatenation of several geometries, relinked as one closed chain
  // (index = position, next / prev cyclic).
  explicit Geometry(std::vector<pGeometry>& geoms);

  std::vector<pElement>& elements() { return elements_; }
  const std::vector<pElement>& elements() const { return elements_; }
  const basis_map elements_bases() { return elements_bases_; }

  // Adds basis b to every element (prints the element count, as the
  // reference does).
  void AddBasis(pBasis b);
  // Adds basis b to element i only.
  void AddBasis(std::size_t i, pBasis b);

  std::shared_ptr<flat_basis_map> FlatMap() const;
  std::size_t size() const { return size_; }
  const PointVector& points() const { return points_; }

 private:
  std::vector<pElement> elements_;
  basis_map elements_bases_;
  PointVector points_;
  int size_;
};

}  // namespace bem2d

#endif
