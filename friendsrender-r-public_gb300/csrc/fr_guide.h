// Photon-emission guide: network dimensions, parameter and weight-tile
// layouts, and the device state shared by the host library and the kernels
// (the kernels and the method are described in fr_guide.cuh).
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>

namespace fr {

constexpr int kGuideIn = 5;
constexpr int kGuideHidden = 64;
constexpr int kGuideLobes = 8;
constexpr int kGuideOut = 5 * kGuideLobes;  // 40
constexpr int kGuideOutPad = 48;            // tensor-core N for the output layer

// Flat FP32 parameter array; weights row-major [out][in].
constexpr int kOffW1 = 0;                                // [64][5]
constexpr int kOffB1 = kOffW1 + kGuideHidden * kGuideIn; // [64]
constexpr int kOffW2 = kOffB1 + kGuideHidden;            // [64][64]
constexpr int kOffB2 = kOffW2 + kGuideHidden * kGuideHidden;
constexpr int kOffW3 = kOffB2 + kGuideHidden;            // [64][64]
constexpr int kOffB3 = kOffW3 + kGuideHidden * kGuideHidden;
constexpr int kOffW4 = kOffB3 + kGuideHidden;            // [48][64], rows 40-47 zero
constexpr int kOffB4 = kOffW4 + kGuideOutPad * kGuideHidden;
constexpr int kGuideParams = kOffB4 + kGuideOutPad;      // 11824

// BF16 weight tiles in the tensor cores' K-major core-matrix layout
// (fr_tc.cuh): W2, W3 (64 x 64), W4 (48 x 64) for the forward pass and their
// transposes W2^T, W3^T (64 x 64), W4^T (64 x 48) for the backward pass.
constexpr int kTileW2 = 0;
constexpr int kTileW3 = kTileW2 + 64 * 64 * 2;
constexpr int kTileW4 = kTileW3 + 64 * 64 * 2;
constexpr int kTileW2T = kTileW4 + 48 * 64 * 2;
constexpr int kTileW3T = kTileW2T + 64 * 64 * 2;
constexpr int kTileW4T = kTileW3T + 64 * 64 * 2;
constexpr int kTileBytes = kTileW4T + 64 * 48 * 2;      // 45056

constexpr float kGuideKappaMin = 0.5f;
constexpr float kGuideKappaMax = 2000.0f;
constexpr float kGuideInvTwoPi = 0.15915494309189535f;

constexpr int kErrGuide = 2;  // a tensor-core wait of the guide gave up

// A path's importance is summed in fixed point so that the sum does not
// depend on the order of the gather's additions: two 64-bit words per path,
// hi in units of 2^-8 and lo in units of 2^-40, each added with integer
// atomics.  A contribution v > 0 adds hi = floor(v * 2^8) and
// lo = rint(frac(v * 2^8) * 2^32); both steps are exact in float except the
// rounding of lo (below 2^-40).  Contributions above 2^40 are clamped (so
// 2^16 of them still fit in hi), and NaN or infinite ones add nothing.
constexpr float kImportanceMax = 1099511627776.0f;  // 2^40
__host__ __device__ inline void importance_split(float v, unsigned long long* hi, unsigned long long* lo) {
  *hi = *lo = 0ull;
  if (!(v > 0.0f) || !(v < INFINITY)) return;
  v = v < kImportanceMax ? v : kImportanceMax;
  const float s = v * 256.0f;
  const float h = floorf(s);
  *hi = (unsigned long long)h;
  *lo = (unsigned long long)rintf((s - h) * 4294967296.0f);
}
__host__ __device__ inline float importance_value(unsigned long long hi, unsigned long long lo) {
  return (float)((double)hi * (1.0 / 256.0) + (double)lo * (1.0 / 1099511627776.0));
}

struct GuideGPU {
  float* params;        // kGuideParams FP32 master weights (the training's)
  float* adam_m;        // Adam moments
  float* adam_v;
  uint8_t* tiles;       // kTileBytes BF16 weight tiles (the training's)
  // The network the emission samples: the training's weights as they were
  // before the last selection (copied by launch_guide_publish), so that the
  // emission of iteration s + 1 can run while iteration s's training does.
  float* emit_params;
  uint8_t* emit_tiles;
  float4* feat;         // per path: inputs x0..x3
  float4* dir;          // per path: input x4, emission direction
  unsigned long long* importance;  // per path {hi, lo}: flux deposited at hitpoints this iteration
  uint32_t* batch;      // training samples (path indices), in path order
  float* batch_w;       // their importance
  float4* batch_feat;   // their inputs and directions (copies of feat and dir, which
  float4* batch_dir;    // the next emission rewrites while the training runs)
  uint32_t* batch_count;
  uint32_t* select_part;  // per selection block: paths taken, then their first batch slot
  float* grad_part;     // per training CTA: kGuideParams gradient sums
  float* wsum_part;     // per training CTA: importance sum
  float* grad;          // kGuideParams gradient sums of the current step (fixed-order sum of grad_part)
  float* weight_sum;    // sum of the batch's importance
  uint32_t* adam_step;
  int* err;             // device error word
  float plain_fraction; // share of plain cosine sampling in the emission mixture
  int batch_cap;
  int steps;            // Adam steps per iteration on the iteration's samples
  int train_ctas;       // grid of the training kernel (grad_part rows)
  float lr;
};

}  // namespace fr
