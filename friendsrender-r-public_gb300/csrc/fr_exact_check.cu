// Device check of fr_exact.cuh: every float-float path against the double
// expression it replaces, on seeded random inputs over and beyond the ranges
// the renderer passes.  A mismatch is counted only where the float-float path
// returned a value (elsewhere the double expression itself is the result).
#include <cuda_runtime.h>
#include <cstdint>
#include "fr_exact.cuh"
#include "fr_kernels.h"
#include "fr_math.cuh"

namespace fr {
namespace {

constexpr int kExactFunctions = 9;

__device__ __forceinline__ float unit(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// A float with a uniform exponent in [lo, hi], a random mantissa and sign s.
__device__ __forceinline__ float wide(uint32_t u, uint32_t v, int lo, int hi, bool sign) {
  const int e = lo + (int)(v % (uint32_t)(hi - lo + 1));
  const uint32_t bits = ((uint32_t)(e + 127) << 23) | (u & 0x7FFFFFu) | (sign && (v & 0x80000000u) ? 0x80000000u : 0u);
  return __uint_as_float(bits);
}

__global__ void k_check_exact(uint64_t samples, uint32_t seed, unsigned long long* mismatch,
                              unsigned long long* fast) {
  unsigned long long mm[kExactFunctions] = {}, fp[kExactFunctions] = {};
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < samples;
       i += (uint64_t)gridDim.x * blockDim.x) {
    for (int f = 0; f < kExactFunctions; ++f) {
      uint32_t r[4];
      philox4x32_10((uint32_t)i, (uint32_t)(i >> 32), (uint32_t)f, 0u, seed, 0x45584354u, r);
      const bool realistic = (r[3] & 1u) != 0;
      float got = 0.0f, want = 0.0f;
      bool ok = false;
      switch (f) {
        case 0: {  // pow_m2
          const float x = realistic ? unit(r[0]) : wide(r[0], r[1], -45, 45, true);
          ok = pow_m2_fast(x, got);
          want = pow_m2_d(x);
        } break;
        case 1: {  // ggx_cth
          const float e = unit(r[0]);
          const float a = realistic ? 0.01f + 0.99f * unit(r[1]) : unit(r[1]);
          const float den = realistic ? e * (a * a - 1.0f) + 1.0f : wide(r[2], r[1], -35, 35, false);
          ok = ggx_cth_fast(e, den, got);
          want = ggx_cth_d(e, den);
        } break;
        case 2: {  // ggx_pdf
          const float a = 0.01f + 0.99f * unit(r[0]);
          const float wm = unit(r[1]), wo = unit(r[2]);
          const float x = realistic ? 1.0f - (1.0f - a * a) * wm * wm : wide(r[2], r[3], -35, 35, true);
          const float f4 = realistic ? 4.0f * wo : wide(r[1], r[0], -45, 25, true);
          ok = ggx_pdf_fast(a * a, x, wm, f4, 3.14159f, got);
          want = ggx_pdf_d(a * a, x, wm, f4, 3.14159f);
        } break;
        case 3: {  // glass_cth
          const float e = unit(r[0]);
          const float a = realistic ? 0.01f + 0.5f * unit(r[1]) : unit(r[1]);
          ok = glass_cth_fast(e, a * a, got);
          want = glass_cth_d(e, a * a);
        } break;
        case 4: {  // glass_pdf
          const float A = realistic ? unit(r[0]) : wide(r[0], r[1], -45, 25, true);
          const float io = 1.0f + unit(r[1]);
          const float B = io * io * unit(r[2]);
          const float s = realistic ? 0.01f + 3.0f * unit(r[3]) : wide(r[3], r[2], -35, 35, true);
          const float alpha = 0.01f + unit(r[1] ^ r[2]);
          const float y = unit(r[0] ^ r[3]);
          ok = glass_pdf_fast(A, B, s, alpha, 3.14159f * (y * y), got);
          want = glass_pdf_d(A, B, s, alpha, 3.14159f * (y * y));
        } break;
        case 5: {  // metal_brdf
          const float c = realistic ? 1e-4f + unit(r[0]) : wide(r[0], r[1], -30, 10, true);
          ok = metal_brdf_fast(c, 1.0f, got);
          want = metal_brdf_d(c, 1.0f);
        } break;
        case 6: {  // conductor_lambda
          const float a = 0.01f + 0.99f * unit(r[0]);
          const float l = realistic ? fminf(0.9999f, unit(r[1])) : wide(r[1], r[2], -60, -1, false);
          const float inv = 1.0f / (l * l);
          ok = conductor_lambda_fast(a * a, inv, got);
          want = conductor_lambda_d(a * a, inv);
        } break;
        case 7: {  // conductor_tm3
          const float fc = realistic ? unit(r[0]) : wide(r[0], r[1], -40, -1, false);
          const float apb = 10.0f * unit(r[2]);
          const float f2 = fc * fc;
          ok = conductor_tm3_fast(apb * fc * fc, 1.0f - f2, f2, got);
          want = conductor_tm3_d(apb * fc * fc, 1.0f - f2, f2);
        } break;
        default: {  // sqrt_half
          const float x = realistic ? 10.0f * unit(r[0]) : __uint_as_float(r[0] & 0x7FFFFFFFu);
          if (!(x == x) || x > 3.0e38f) continue;
          ok = sqrt_half_fast(x, got);
          want = sqrt_half_d(x);
        } break;
      }
      if (ok) {
        ++fp[f];
        if (__float_as_uint(got) != __float_as_uint(want)) ++mm[f];
      }
    }
  }
  for (int f = 0; f < kExactFunctions; ++f) {
    if (mm[f]) atomicAdd(mismatch + f, mm[f]);
    if (fp[f]) atomicAdd(fast + f, fp[f]);
  }
}

}  // namespace

int check_exact_math(uint64_t samples, uint32_t seed, uint64_t* mismatches, uint64_t* fast_paths, const char** msg) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long) * 2 * kExactFunctions) != cudaSuccess) {
    *msg = "cudaMalloc failed";
    return -1;
  }
  cudaMemset(d, 0, sizeof(unsigned long long) * 2 * kExactFunctions);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_check_exact<<<sms * 4, 256>>>(samples, seed, d, d + kExactFunctions);
  unsigned long long h[2 * kExactFunctions];
  const cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    *msg = cudaGetErrorString(e);
    return -1;
  }
  for (int f = 0; f < kExactFunctions; ++f) {
    mismatches[f] = h[f];
    fast_paths[f] = h[kExactFunctions + f];
  }
  return 0;
}

}  // namespace fr
