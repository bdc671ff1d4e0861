// Device LBVH build of the scene BVH (no counterpart in the reference, whose
// Build3 / Build2 run on the host, bvh8.h:44-189).
//
//   k_lbvh_keys     per triangle: box, centroid, 30-bit Morton code of the
//                   centroid in the scene box
//   k_bit_flags / scan / k_bit_scatter
//                   stable radix sort of the codes, one bit per pass (the
//                   photon grid's exclusive scan ranks the ones)
//   k_lbvh_tree     binary radix tree (Karras, "Maximizing parallelism in the
//                   construction of BVHs, octrees, and k-d trees", HPG 2012):
//                   inner node i spans a range of sorted codes and splits it
//                   at the highest differing bit; equal codes are told apart
//                   by their sorted index
//   k_lbvh_boxes    boxes bottom up, the second child to finish computes its
//                   parent's box
// The tree comes back to the host, where subtrees of at most 4 triangles
// become leaves and the 8-wide collapse of the host builder lays out the
// nodes.  Any valid tree gives the reference's closest hits (the triangle test
// decides them), so the choice of builder changes the speed only.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "fr_bvh.h"
#include "fr_kernels.h"

namespace fr {
namespace {

constexpr int kLeafMaxTris = 4;

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits to every third bit
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_lbvh_keys(const float* pos, int n, float3 lo, float3 inv_ext, uint32_t* keys, uint32_t* idx,
                            float* boxes) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float* p = pos + 9 * (size_t)t;
  float b[6];
  for (int a = 0; a < 3; ++a) {
    b[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
    b[3 + a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
  }
  for (int k = 0; k < 6; ++k) boxes[6 * (size_t)t + k] = b[k];
  const float cx = (0.5f * (b[0] + b[3]) - lo.x) * inv_ext.x;
  const float cy = (0.5f * (b[1] + b[4]) - lo.y) * inv_ext.y;
  const float cz = (0.5f * (b[2] + b[5]) - lo.z) * inv_ext.z;
  const uint32_t qx = (uint32_t)fminf(fmaxf(cx * 1024.0f, 0.0f), 1023.0f);
  const uint32_t qy = (uint32_t)fminf(fmaxf(cy * 1024.0f, 0.0f), 1023.0f);
  const uint32_t qz = (uint32_t)fminf(fmaxf(cz * 1024.0f, 0.0f), 1023.0f);
  keys[t] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
  idx[t] = (uint32_t)t;
}

__global__ void k_bit_flags(const uint32_t* keys, int n, int bit, uint32_t* flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = (keys[i] >> bit) & 1u;
  if (i == n) flags[n] = 0u;
}

// Stable split by one bit: zeros keep their order in front, ones after them.
__global__ void k_bit_scatter(const uint32_t* keys, const uint32_t* idx, const uint32_t* ones_before, int n,
                              int bit, uint32_t* keys_out, uint32_t* idx_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t total_ones = ones_before[n];
  const uint32_t zeros = (uint32_t)n - total_ones;
  const uint32_t k = keys[i];
  const uint32_t dst = ((k >> bit) & 1u) ? zeros + ones_before[i] : (uint32_t)i - ones_before[i];
  keys_out[dst] = k;
  idx_out[dst] = idx[i];
}

// Common-prefix length of sorted codes i and j (Karras 2012, section 4), -1
// out of range; equal codes compare their indices.
__device__ __forceinline__ int delta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = keys[i], b = keys[j];
  return a != b ? __clz(a ^ b) : 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Inner node i of n - 1: its children (leaf k encoded as n - 1 + k), range
// and the parents of both children.
__global__ void k_lbvh_tree(const uint32_t* keys, int n, int* left, int* right, int* first, int* last,
                            int* parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0, k = l;
  do {
    k = (k + 1) >> 1;
    if (delta(keys, n, i, i + (s + k) * d) > dnode) s += k;
  } while (k > 1);
  const int g = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  const int lc = lo == g ? (n - 1) + g : g;
  const int rc = hi == g + 1 ? (n - 1) + g + 1 : g + 1;
  left[i] = lc;
  right[i] = rc;
  first[i] = lo;
  last[i] = hi;
  parent[lc] = i;
  parent[rc] = i;
}

// Boxes bottom up: node boxes (6 floats) for inner nodes 0..n-2, then leaves.
__global__ void k_lbvh_boxes(const uint32_t* idx, const float* tri_boxes, int n, const int* left, const int* right,
                             const int* parent, float* node_boxes, unsigned int* visits) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int leaf = (n - 1) + k;
  for (int a = 0; a < 6; ++a) node_boxes[6 * (size_t)leaf + a] = tri_boxes[6 * (size_t)idx[k] + a];
  if (n == 1) return;
  int node = parent[leaf];
  while (true) {
    __threadfence();
    if (atomicAdd(visits + node, 1u) == 0u) return;  // the other child finishes this node
    __threadfence();
    const float* bl = node_boxes + 6 * (size_t)left[node];
    const float* br = node_boxes + 6 * (size_t)right[node];
    float* bo = node_boxes + 6 * (size_t)node;
    for (int a = 0; a < 3; ++a) {
      bo[a] = fminf(__ldcg(bl + a), __ldcg(br + a));
      bo[3 + a] = fmaxf(__ldcg(bl + 3 + a), __ldcg(br + 3 + a));
    }
    if (node == 0) return;
    node = parent[node];
  }
}

int blocks(int n) { return (n + 255) / 256; }

}  // namespace

int build_bvh8_lbvh(const float* positions, int n, const float lo[3], const float hi[3], float pad_abs,
                    BVHResult& out, const char** err) {
  if (n <= 0) {
    *err = "no triangles";
    return -1;
  }
  std::vector<void*> bufs;
  bool ok = true;
  auto dalloc = [&](size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) ok = false;
    bufs.push_back(p);
    return p;
  };
  const size_t nn = (size_t)n;
  float* d_pos = (float*)dalloc(36 * nn);
  float* d_tbox = (float*)dalloc(24 * nn);
  uint32_t* keys[2] = {(uint32_t*)dalloc(4 * nn), (uint32_t*)dalloc(4 * nn)};
  uint32_t* idx[2] = {(uint32_t*)dalloc(4 * nn), (uint32_t*)dalloc(4 * nn)};
  uint32_t* flags = (uint32_t*)dalloc(4 * (nn + 1));
  uint32_t* ones = (uint32_t*)dalloc(4 * (nn + 1));
  int* d_left = (int*)dalloc(4 * nn);
  int* d_right = (int*)dalloc(4 * nn);
  int* d_first = (int*)dalloc(4 * nn);
  int* d_last = (int*)dalloc(4 * nn);
  int* d_parent = (int*)dalloc(4 * 2 * nn);
  float* d_boxes = (float*)dalloc(24 * 2 * nn);
  unsigned int* d_visits = (unsigned int*)dalloc(4 * nn);
  ScanTemp st{};
  const uint32_t words = scan_temp_words((uint32_t)nn + 1, st);
  uint32_t* sw = (uint32_t*)dalloc(4 * (size_t)words);
  auto release = [&]() {
    for (void* p : bufs) cudaFree(p);
  };
  if (!ok) {
    release();
    *err = "cudaMalloc failed";
    return -1;
  }
  for (int l = 0; l < st.levels; ++l) {
    st.level[l] = sw;
    sw += st.level_n[l] + 1;
  }
  cudaStream_t s = 0;
  cudaMemcpyAsync(d_pos, positions, 36 * nn, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(d_visits, 0, 4 * nn, s);
  const float3 flo = make_float3(lo[0], lo[1], lo[2]);
  const float3 inv = make_float3(1.0f / std::max(hi[0] - lo[0], 1e-20f), 1.0f / std::max(hi[1] - lo[1], 1e-20f),
                                 1.0f / std::max(hi[2] - lo[2], 1e-20f));
  k_lbvh_keys<<<blocks(n), 256, 0, s>>>(d_pos, n, flo, inv, keys[0], idx[0], d_tbox);
  int cur = 0;
  for (int bit = 0; bit < 30; ++bit) {
    k_bit_flags<<<blocks(n + 1), 256, 0, s>>>(keys[cur], n, bit, flags);
    launch_scan(flags, ones, (uint32_t)n + 1, st, s);
    k_bit_scatter<<<blocks(n), 256, 0, s>>>(keys[cur], idx[cur], ones, n, bit, keys[cur ^ 1], idx[cur ^ 1]);
    cur ^= 1;
  }
  if (n > 1) k_lbvh_tree<<<blocks(n - 1), 256, 0, s>>>(keys[cur], n, d_left, d_right, d_first, d_last, d_parent);
  k_lbvh_boxes<<<blocks(n), 256, 0, s>>>(idx[cur], d_tbox, n, d_left, d_right, d_parent, d_boxes, d_visits);
  std::vector<int> perm(nn), left(nn - 1 + (n == 1)), right(left.size()), first(left.size()), last(left.size());
  std::vector<float> boxes(12 * nn);
  cudaMemcpyAsync(perm.data(), idx[cur], 4 * nn, cudaMemcpyDeviceToHost, s);
  if (n > 1) {
    cudaMemcpyAsync(left.data(), d_left, 4 * (nn - 1), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(right.data(), d_right, 4 * (nn - 1), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(first.data(), d_first, 4 * (nn - 1), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(last.data(), d_last, 4 * (nn - 1), cudaMemcpyDeviceToHost, s);
  }
  cudaMemcpyAsync(boxes.data(), d_boxes, 24 * (2 * nn - 1), cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  release();
  if (e != cudaSuccess) {
    *err = cudaGetErrorString(e);
    return -1;
  }
  // Inner nodes 0..n-2, then leaf k at n-1+k; inner nodes over at most
  // kLeafMaxTris triangles become leaves over their sorted range.
  std::vector<BinNode> nodes(2 * nn - 1);
  for (size_t i = 0; i < nodes.size(); ++i) {
    BinNode& b = nodes[i];
    for (int a = 0; a < 3; ++a) { b.lo[a] = boxes[6 * i + a]; b.hi[a] = boxes[6 * i + 3 + a]; }
    if (i + 1 < nn) {
      const int cnt = last[i] - first[i] + 1;
      if (cnt <= kLeafMaxTris) {
        b.first = first[i];
        b.count = cnt;
      } else {
        b.left = left[i];
        b.right = right[i];
      }
    } else {
      b.first = (int)(i - (nn - 1));
      b.count = 1;
    }
  }
  out = collapse_bvh8(nodes, n > 1 ? 0 : 0, perm, pad_abs);
  return 0;
}

}  // namespace fr
