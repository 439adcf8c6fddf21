// Internal: the bridge from the C++ API to the C ABI (include/bem2d_gpu.h).
#ifndef BEM2D_GPU_GLUE_H
#define BEM2D_GPU_GLUE_H

#include <cstdint>
#include <vector>

#include "../../include/bem2d_gpu.h"
#include "bem2d_geometry.h"

namespace bem2d {
namespace detail {

// The process-wide context on device BEM2D_DEVICE (default 0), created on
// first use.
bem2d_ctx* ctx();
// Map a C-ABI status to the reference's exception tags.
void check(int rc, const char* what);

// A Geometry (or a flat basis map) lowered to the C-ABI tables.
struct PackedGeometry {
  std::vector<int32_t> kind;
  std::vector<double> param;
  std::vector<int64_t> index, next, prev;
  std::vector<int32_t> unk_elem, unk_kind;
  std::vector<double> unk_param;
  bem2d_geometry view() const;
};
PackedGeometry Pack(const Geometry::flat_basis_map& fm);
PackedGeometry Pack(const Geometry& g);

}  // namespace detail
}  // namespace bem2d

#endif
