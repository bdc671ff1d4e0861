// Device vector math and the counter-based RNG.
//
// Every operator evaluates in the order of the reference's PTUtility::Vec3
// (SPPM/SPPM/Vec.h:179-243, 303-323): dot = (a0*b0 + a1*b1) + a2*b2,
// normalized() divides by sqrt(norm2()).  The kernels are compiled with
// --fmad=false and IEEE division and square root, so a float expression
// written here rounds exactly as the reference's does on the host.
#pragma once
#include <cstdint>
#include "fr_layout.h"

namespace fr {

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3(const float* p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ float norm(V3 a) { return sqrtf(norm2(a)); }
__device__ __forceinline__ V3 normalized(V3 a) {
  const float d = norm(a);
  return V3{a.x / d, a.y / d, a.z / d};
}
__device__ __forceinline__ float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Float thresholds for the reference's float-against-double comparisons.
// For a float g and a double constant d that is not a float, (double)g > d
// exactly when g > rd(d), and (double)g < d exactly when g < ru(d), where
// rd/ru round d down/up to a float.  Comparing in float keeps the decisions
// bit-identical without the FP64 pipe.
constexpr float kGt1e4 = 0x1.a36e2ep-14f;      // (double)g > 1e-4
constexpr float kGt1e5 = 0x1.4f8b58p-17f;      // (double)g > 1e-5
constexpr float kLt1e5 = 0x1.4f8b5ap-17f;      // (double)g < 1e-5
constexpr float kGt1e6 = 0x1.0c6f7ap-20f;      // (double)g > 1e-6
constexpr float kLt1e6 = 0x1.0c6f7cp-20f;      // (double)g < 1e-6
constexpr float kLt1e8 = 0x1.5798f0p-27f;      // (double)g < 1e-8
constexpr float kGt1e8 = 0x1.5798eep-27f;      // (double)g > 1e-8
constexpr float kGt0_999999 = 0x1.ffffdep-1f;  // (double)g > 0.999999
constexpr float kGt0_9 = 0x1.ccccccp-1f;       // (double)g > 0.9
constexpr float kGt0_99 = 0x1.fae146p-1f;      // (double)g > 0.99

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  A stream is keyed by the
// reference's integer seed; draw n is lane n%4 of block n/4; a draw is the
// top 24 bits scaled by 2^-24, exact in float.
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Rng {
  uint32_t key;
  uint32_t draw;
  uint32_t buf[4];

  __device__ __forceinline__ explicit Rng(uint32_t seed) : key(seed), draw(0) {}
  // Continue the stream at draw n (the buffered block is refilled on demand).
  __device__ __forceinline__ void seek(uint32_t n) {
    draw = n;
    if (n & 3u) philox4x32_10(n >> 2, 0u, 0u, 0u, key, kPhiloxKeyHi, buf);
  }
  __device__ __forceinline__ uint32_t next_u24() {
    const uint32_t lane = draw & 3u;
    if (lane == 0) philox4x32_10(draw >> 2, 0u, 0u, 0u, key, kPhiloxKeyHi, buf);
    ++draw;
    uint32_t v = buf[0];
    v = lane == 1 ? buf[1] : v;
    v = lane == 2 ? buf[2] : v;
    v = lane == 3 ? buf[3] : v;
    return v >> 8;
  }
  // RandomMT::genrand64_real1/2 (MT.h:30-37): the same value, [0, 1).
  __device__ __forceinline__ float next() { return (float)next_u24() * (1.0f / 16777216.0f); }
};

}  // namespace fr
