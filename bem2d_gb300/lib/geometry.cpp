// bem2d C++ API (GB300 build): Geometry.
#include "bem2d_geometry.h"

namespace bem2d {

Geometry::Geometry(const std::vector<pElement>& elems) : elements_(elems), size_(0) {
  elements_bases_.resize(elems.size());
  for (std::size_t i = 0; i < elements_.size(); ++i) points_.push_back(elements_[i]->First());
}

Geometry::Geometry(std::vector<pGeometry>& geoms) : size_(0) {
  for (std::size_t i = 0; i < geoms.size(); ++i)
    for (const pElement& e : geoms[i]->elements()) elements_.push_back(e);
  const int n = (int)elements_.size();
  elements_bases_.resize(n);
  for (int i = 0; i < n; ++i) {
    elements_[i]->set_index(i);
    elements_[i]->set_next(i + 1 < n ? i + 1 : 0);
    elements_[i]->set_prev(i > 0 ? i - 1 : n - 1);
  }
  for (int i = 0; i < n; ++i) points_.push_back(elements_[i]->First());
}

void Geometry::AddBasis(pBasis b) {
  std::cout << "Elems: " << elements_.size() << std::endl;
  for (std::size_t i = 0; i < elements_.size(); ++i) {
    elements_bases_[i].insert(std::make_pair((std::size_t)size_, b));
    size_++;
  }
}

void Geometry::AddBasis(std::size_t i, pBasis b) {
  elements_bases_[i].insert(std::make_pair((std::size_t)size_, b));
  size_++;
}

std::shared_ptr<Geometry::flat_basis_map> Geometry::FlatMap() const {
  std::shared_ptr<flat_basis_map> p(new flat_basis_map);
  for (std::size_t i = 0; i < elements_bases_.size(); ++i)
    for (const auto& kv : elements_bases_[i]) p->push_back(std::make_pair(elements_[i], kv.second));
  return p;
}

}  // namespace bem2d
