// Learned photon-emission guide: a small MLP maps a point on a light (5
// inputs: scene-normalized position, light-surface barycentrics u, v) to a
// mixture of kGuideLobes von Mises-Fisher lobes over the emission direction
// (5 -> 64 -> 64 -> 64 -> 8 x {mean direction (3), concentration, weight}).
// Photons take their direction from a defensive mixture of plain cosine
// sampling (fraction f) and the guide, with the mixture's exact pdf in the
// photon's weight, so the estimate stays the unbiased SPPM one.
//
// The network is trained online, every iteration, on the photon paths that
// reached a hitpoint: loss -I * log q(d | x), I the path's deposited flux seen
// through the hitpoints (its visual importance), d and x its emission
// direction and point.  Layers 2-4 run on the tensor cores (tcgen05, BF16
// operands, FP32 accumulation); layer 1 (5 inputs) and the mixture in FP32.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>
#include "fr_guide.h"
#include "fr_math.cuh"
#include "fr_tc.cuh"

namespace fr {

// ---- shared pieces of the forward pass (training and guided emission)

__device__ __forceinline__ void st_bf16(uint8_t* tile, uint32_t r, uint32_t k, uint32_t K, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + tc::tile_offset(r, k, K)) = __float2bfloat16_rn(v);
}
// Eight values of row r, columns k0..k0+7 (k0 a multiple of 8): one 16-byte
// store, the eight being contiguous in the core-matrix layout.
__device__ __forceinline__ void st_bf16x8(uint8_t* tile, uint32_t r, uint32_t k0, uint32_t K, const float v[8]) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
  *reinterpret_cast<uint4*>(tile + tc::tile_offset(r, k0, K)) = *reinterpret_cast<const uint4*>(h);
}
__device__ __forceinline__ float ld_bf16(const uint8_t* tile, uint32_t r, uint32_t k, uint32_t K) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tile + tc::tile_offset(r, k, K)));
}

// Shared memory written by the generic proxy, then read by tcgen05.mma.
__device__ __forceinline__ void publish() {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// Waits for the tensor-core work committed since the last wait; false (and
// stays false) when the bounded wait gives up.  Every thread of the CTA calls it.
struct TcSync {
  uint64_t* bar;
  uint32_t phase;
  bool ok;
  __device__ __forceinline__ bool wait() {
    const bool w = ok && tc::mbar_wait(bar, phase & 1u);
    ++phase;
    ok = __syncthreads_and(w) != 0;
    tc::fence_after_sync();
    return ok;
  }
};

// Layer 1 (FP32) of this thread's sample into tile h1 (row t).  p1 holds W1
// and b1 at their parameter offsets.
__device__ __forceinline__ void guide_layer1(const float* p1, const float x[kGuideIn], uint8_t* h1, uint32_t t) {
  for (int j0 = 0; j0 < kGuideHidden; j0 += 8) {
    float h[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float z = p1[kOffB1 + j0 + j];
#pragma unroll
      for (int k = 0; k < kGuideIn; ++k) z += p1[kOffW1 + (j0 + j) * kGuideIn + k] * x[k];
      h[j] = fmaxf(z, 0.0f);
    }
    st_bf16x8(h1, t, j0, 64, h);
  }
}

// Hidden-layer epilogue: TMEM row t (64 columns) + bias, ReLU, into tile h.
__device__ __forceinline__ void guide_hidden_epilogue(uint32_t taddr, const float* bias, uint8_t* h, uint32_t t) {
#pragma unroll
  for (int c0 = 0; c0 < 64; c0 += 16) {
    float v[16];
    tc::tmem_ld16(taddr + c0, v);
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = fmaxf(v[k] + bias[c0 + k], 0.0f);
    st_bf16x8(h, t, c0, 64, v);
    st_bf16x8(h, t, c0 + 8, 64, v + 8);
  }
}

// Output-layer epilogue: TMEM row t (48 columns) + bias into the 40 outputs.
__device__ __forceinline__ void guide_output_epilogue(uint32_t taddr, const float* bias, float o[kGuideOut]) {
#pragma unroll
  for (int c0 = 0; c0 < kGuideOutPad; c0 += 16) {
    float v[16];
    tc::tmem_ld16(taddr + c0, v);
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (c0 + k < kGuideOut) o[c0 + k] = v[k] + bias[c0 + k];
  }
}

// Mixture parameters of one output row: unit mean directions, concentrations,
// normalized weights.
struct GuideMixture {
  V3 mu[kGuideLobes];
  float kappa[kGuideLobes], w[kGuideLobes];
  float lnorm[kGuideLobes];  // log of the vMF normalization kappa / (2 pi (1 - e^{-2 kappa}))
  float norm[kGuideLobes];  // |raw mean| (for the gradient)
  float kraw[kGuideLobes];  // raw concentration (for the gradient)
};

__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }

__device__ __forceinline__ void guide_mixture(const float o[kGuideOut], GuideMixture& g) {
  float amax = -3.0e38f;
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) amax = fmaxf(amax, o[5 * k + 4]);
  float wsum = 0.0f;
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) {
    const V3 m = v3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
    const float n = fmaxf(sqrtf(norm2(m)), 1e-6f);
    g.norm[k] = n;
    g.mu[k] = m * (1.0f / n);
    g.kraw[k] = o[5 * k + 3];
    g.kappa[k] = fminf(kGuideKappaMin + softplus(o[5 * k + 3]), kGuideKappaMax);
    g.lnorm[k] = logf(g.kappa[k] * kGuideInvTwoPi) - log1pf(-expf(-2.0f * g.kappa[k]));
    g.w[k] = expf(o[5 * k + 4] - amax);
    wsum += g.w[k];
  }
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) g.w[k] /= wsum;
}

// log of the von Mises-Fisher density kappa / (2 pi (1 - e^{-2 kappa})) * e^{kappa (mu.d - 1)}.
__device__ __forceinline__ float vmf_log_pdf(float kappa, float cosang) {
  return logf(kappa * kGuideInvTwoPi) - log1pf(-expf(-2.0f * kappa)) + kappa * (cosang - 1.0f);
}

__device__ __forceinline__ float guide_pdf(const GuideMixture& g, V3 d) {
  float p = 0.0f;
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) p += g.w[k] * expf(g.lnorm[k] + g.kappa[k] * (dot(g.mu[k], d) - 1.0f));
  return p;
}

// A direction from lobe k (Wood's method): cos theta = 1 + log(e1 + (1 - e1) e^{-2 kappa}) / kappa.
__device__ __forceinline__ V3 vmf_sample(V3 mu, float kappa, float e1, float e2) {
  const float c = fminf(1.0f, fmaxf(-1.0f, 1.0f + logf(e1 + (1.0f - e1) * expf(-2.0f * kappa)) / kappa));
  const float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
  float sp, cp;
  sincosf(6.283185307179586f * e2, &sp, &cp);
  const V3 a = fabsf(mu.x) > 0.9f ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f);
  const V3 t = normalized(cross(a, mu));
  const V3 b = cross(mu, t);
  return normalized(mu * c + t * (s * cp) + b * (s * sp));
}

// Gradient of -I * log q(d) with respect to the 40 raw outputs.
__device__ __forceinline__ void guide_loss_grad(const GuideMixture& g, V3 d, float I, float dout[kGuideOut]) {
  float lf[kGuideLobes], lmax = -3.0e38f;
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) {
    lf[k] = logf(g.w[k]) + (g.lnorm[k] + g.kappa[k] * (dot(g.mu[k], d) - 1.0f));  // + vmf_log_pdf
    lmax = fmaxf(lmax, lf[k]);
  }
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) {
    lf[k] = expf(lf[k] - lmax);
    s += lf[k];
  }
#pragma unroll
  for (int k = 0; k < kGuideLobes; ++k) {
    const float gam = lf[k] / s;  // posterior of lobe k
    const float kap = g.kappa[k];
    const float cs = dot(g.mu[k], d);
    // d log f / d kappa = 1/kappa - 2 e^{-2k} / (1 - e^{-2k}) + (mu.d - 1)
    const float e2k = expf(-2.0f * kap);
    float dk = 1.0f / kap - 2.0f * e2k / (1.0f - e2k) + (cs - 1.0f);
    const bool clamped = kGuideKappaMin + softplus(g.kraw[k]) > kGuideKappaMax;
    const float sig = 1.0f / (1.0f + expf(-g.kraw[k]));
    dout[5 * k + 3] = clamped ? 0.0f : -I * gam * dk * sig;
    dout[5 * k + 4] = -I * (gam - g.w[k]);
    // d log f / d mu = kappa d; through mu = m / |m|: (I - mu mu^T) / |m|.
    const V3 gm = d * (kap * gam * -I);
    const V3 proj = (gm - g.mu[k] * dot(g.mu[k], gm)) * (1.0f / g.norm[k]);
    dout[5 * k] = proj.x;
    dout[5 * k + 1] = proj.y;
    dout[5 * k + 2] = proj.z;
  }
}

}  // namespace fr
