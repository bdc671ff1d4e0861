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

// A binary BVH node: inner (left/right node indices) or leaf (left < 0;
// triangles perm[first .. first + count)).
struct BinNode {
  float lo[3], hi[3];
  int left = -1, right = -1;
  int first = 0, count = 0;
};

// The 8-wide tree of a binary one (root `root`, leaf triangles through perm).
BVHResult collapse_bvh8(const std::vector<BinNode>& nodes, int root, const std::vector<int>& perm, float pad_abs);

// Device LBVH build (fr_bvh_gpu.cu): Morton codes of the triangle centroids in
// the scene box lo..hi, a stable radix sort, the binary radix tree (Karras
// 2012) with its boxes built bottom up, subtrees of at most 4 triangles as
// leaves; the tree comes back to the host and is collapsed as build_bvh8's.
// Returns 0, or -1 with *err set.
int build_bvh8_lbvh(const float* positions, int num_tris, const float lo[3], const float hi[3], float pad_abs,
                    BVHResult& out, const char** err);

}  // namespace fr
