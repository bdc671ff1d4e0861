// Host BVH builder: binned-SAH binary tree collapsed into 8-wide nodes.
//
// Replaces N_BVH<Triangle_ID, Ray, 8>::Build3 (SPPM/SPPM/bvh8.h:135-189).  The
// tree shape only decides which boxes a ray tests; the closest hit is fixed by
// the triangle test, so any valid tree gives the reference's hits.  Leaves
// hold up to 4 triangles; child boxes are padded so that the kernels' fused
// slab test never culls a box the ray actually meets.
#include "fr_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace fr {

namespace {

struct Box {
  float lo[3], hi[3];
  Box() {
    for (int a = 0; a < 3; ++a) { lo[a] = std::numeric_limits<float>::infinity(); hi[a] = -lo[a]; }
  }
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
  }
  float area() const {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct BNode {
  Box box;
  int left = -1, right = -1;  // children (binary), -1 for a leaf
  int first = 0, count = 0;   // leaf range in the permutation
};

constexpr int kBins = 16;
constexpr int kLeafMax = 4;

struct Builder {
  const float* pos;  // T x 9
  std::vector<Box> tb;
  std::vector<float> cen;  // T x 3
  std::vector<int> perm;
  std::vector<BNode> nodes;

  int build(int first, int count, int depth) {
    BNode n;
    Box cb;
    for (int i = first; i < first + count; ++i) {
      const int t = perm[i];
      n.box.grow(tb[t]);
      cb.grow(&cen[3 * t]);
    }
    const int id = (int)nodes.size();
    nodes.push_back(n);
    if (count <= 1) {
      nodes[id].first = first;
      nodes[id].count = count;
      return id;
    }
    int axis = 0;
    float ext = cb.hi[0] - cb.lo[0];
    for (int a = 1; a < 3; ++a)
      if (cb.hi[a] - cb.lo[a] > ext) { ext = cb.hi[a] - cb.lo[a]; axis = a; }
    int split = -1;
    float best = std::numeric_limits<float>::infinity();
    int mid = first + count / 2;
    if (ext > 0.0f) {
      Box bb[kBins];
      int bc[kBins] = {0};
      const float k = kBins / ext;
      auto bin_of = [&](int t) {
        int b = (int)((cen[3 * t + axis] - cb.lo[axis]) * k);
        return std::min(kBins - 1, std::max(0, b));
      };
      for (int i = first; i < first + count; ++i) {
        const int t = perm[i];
        const int b = bin_of(t);
        bb[b].grow(tb[t]);
        ++bc[b];
      }
      float ra[kBins];
      int rc[kBins];
      Box acc;
      int c = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        c += bc[b];
        ra[b] = acc.area();
        rc[b] = c;
      }
      acc = Box();
      c = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        acc.grow(bb[b]);
        c += bc[b];
        if (c == 0 || rc[b + 1] == 0) continue;
        const float cost = acc.area() * c + ra[b + 1] * rc[b + 1];
        if (cost < best) { best = cost; split = b; }
      }
      const float leaf_cost = n.box.area() * count;
      const float parent = n.box.area();
      if (count <= kLeafMax && (split < 0 || 0.5f * parent + best >= leaf_cost)) {
        nodes[id].first = first;
        nodes[id].count = count;
        return id;
      }
      if (split >= 0) {
        auto it = std::partition(perm.begin() + first, perm.begin() + first + count,
                                 [&](int t) { return bin_of(t) <= split; });
        mid = (int)(it - perm.begin());
      }
    }
    if (split < 0) {
      if (count <= kLeafMax) {
        nodes[id].first = first;
        nodes[id].count = count;
        return id;
      }
      // All centroids coincide along every axis: split the range in the middle.
      mid = first + count / 2;
    }
    const int l = build(first, mid - first, depth + 1);
    const int r = build(mid, first + count - mid, depth + 1);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }
};

}  // namespace

BVHResult build_bvh8(const float* positions, int num_tris, float pad_abs) {
  Builder b;
  b.pos = positions;
  b.tb.resize(num_tris);
  b.cen.resize(3 * (size_t)num_tris);
  b.perm.resize(num_tris);
  for (int t = 0; t < num_tris; ++t) {
    Box bx;
    for (int k = 0; k < 3; ++k) bx.grow(positions + 9 * (size_t)t + 3 * k);
    b.tb[t] = bx;
    for (int a = 0; a < 3; ++a) b.cen[3 * (size_t)t + a] = 0.5f * (bx.lo[a] + bx.hi[a]);
    b.perm[t] = t;
  }
  b.nodes.reserve(2 * (size_t)num_tris);
  const int root = b.build(0, num_tris, 0);

  std::vector<BinNode> bn(b.nodes.size());
  for (size_t i = 0; i < b.nodes.size(); ++i) {
    const BNode& n = b.nodes[i];
    for (int a = 0; a < 3; ++a) { bn[i].lo[a] = n.box.lo[a]; bn[i].hi[a] = n.box.hi[a]; }
    bn[i].left = n.left;
    bn[i].right = n.right;
    bn[i].first = n.first;
    bn[i].count = n.count;
  }
  return collapse_bvh8(bn, root, b.perm, pad_abs);
}

namespace {
float bin_area(const BinNode& n) {
  const float dx = n.hi[0] - n.lo[0], dy = n.hi[1] - n.lo[1], dz = n.hi[2] - n.lo[2];
  if (dx < 0 || dy < 0 || dz < 0) return 0.0f;
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}
}  // namespace

BVHResult collapse_bvh8(const std::vector<BinNode>& bnodes, int root, const std::vector<int>& perm, float pad_abs) {
  BVHResult out;
  // Collapse breadth first: each wide node takes up to 8 binary descendants,
  // opening the largest-area inner child first; its internal children get
  // consecutive node indices and its leaves consecutive triangle slots.
  struct Job { int bnode; int wide; int depth; };
  std::vector<Job> jobs;
  size_t head = 0;
  out.nodes.emplace_back();
  jobs.push_back({root, 0, 1});
  auto pad = [&](float v, bool up) {
    const float d = pad_abs + std::fabs(v) * 1e-6f;
    return up ? v + d : v - d;
  };
  int maxd = 1;
  while (head < jobs.size()) {
    const Job j = jobs[head++];
    maxd = std::max(maxd, j.depth);
    std::vector<int> kids;
    const BinNode& bn = bnodes[j.bnode];
    if (bn.left < 0) {
      kids.push_back(j.bnode);  // a root that is a leaf
    } else {
      kids.push_back(bn.left);
      kids.push_back(bn.right);
      while (kids.size() < 8) {
        int pick = -1;
        float pa = -1.0f;
        for (int k = 0; k < (int)kids.size(); ++k) {
          const BinNode& c = bnodes[kids[k]];
          if (c.left >= 0 && bin_area(c) > pa) { pa = bin_area(c); pick = k; }
        }
        if (pick < 0) break;
        const BinNode& c = bnodes[kids[pick]];
        const int l = c.left, r = c.right;
        kids[pick] = l;
        kids.push_back(r);
      }
    }
    BVHNodeW node;
    std::memset(&node, 0, sizeof(node));
    for (int c = 0; c < 8; ++c) {
      node.lox[c] = node.loy[c] = node.loz[c] = std::numeric_limits<float>::infinity();
      node.hix[c] = node.hiy[c] = node.hiz[c] = -std::numeric_limits<float>::infinity();
    }
    int ninternal = 0;
    for (int c = 0; c < (int)kids.size(); ++c)
      if (bnodes[kids[c]].left >= 0) ++ninternal;
    node.child_base = (uint32_t)out.nodes.size();
    node.tri_base = (uint32_t)out.tri_order.size();
    for (int i = 0; i < ninternal; ++i) out.nodes.emplace_back();
    int next_internal = 0;
    uint32_t tri_off = 0;
    for (int c = 0; c < (int)kids.size(); ++c) {
      const BinNode& k = bnodes[kids[c]];
      node.lox[c] = pad(k.lo[0], false); node.hix[c] = pad(k.hi[0], true);
      node.loy[c] = pad(k.lo[1], false); node.hiy[c] = pad(k.hi[1], true);
      node.loz[c] = pad(k.lo[2], false); node.hiz[c] = pad(k.hi[2], true);
      if (k.left >= 0) {
        node.imask |= 1u << c;
        node.meta[c] = 0x80;
        jobs.push_back({kids[c], (int)node.child_base + next_internal++, j.depth + 1});
      } else {
        node.meta[c] = (uint8_t)(0x80u | ((uint32_t)(k.count - 1) << 5) | tri_off);
        for (int t = 0; t < k.count; ++t) out.tri_order.push_back(perm[k.first + t]);
        tri_off += (uint32_t)k.count;
      }
    }
    out.nodes[j.wide] = node;
  }
  out.depth = maxd;
  return out;
}

}  // namespace fr
