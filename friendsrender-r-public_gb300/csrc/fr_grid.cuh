// Cell coordinates and bucket hash of the photon grid, shared by every
// kernel that builds or queries it.
#pragma once
#include <cstdint>

namespace fr {

__device__ __forceinline__ int cell_of(float p, float o, float inv) { return (int)floorf((p - o) * inv); }

__device__ __forceinline__ uint32_t cell_hash(int x, int y, int z, uint32_t mask) {
  return (((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^ ((uint32_t)z * 83492791u)) & mask;
}

}  // namespace fr
