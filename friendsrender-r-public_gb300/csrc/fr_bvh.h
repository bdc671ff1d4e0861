#pragma once
#include <vector>
#include "fr_layout.h"

namespace fr {

struct BVHResult {
  std::vector<BVHNodeW> nodes;  // node 0 is the root
  std::vector<int> tri_order;   // leaf order -> facet index
  int depth = 0;                // levels of the wide tree
};

// positions: num_tris x 9 floats.  pad_abs: absolute padding added to every
// child box on top of a 1e-6 relative one.
BVHResult build_bvh8(const float* positions, int num_tris, float pad_abs);

}  // namespace fr
