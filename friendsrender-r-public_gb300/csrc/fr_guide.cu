// Training of the learned photon-emission guide (fr_guide.cuh) and the
// forward pass it shares with the guided emission kernel.
//
// One CTA of 128 threads works on tiles of 128 samples, thread t on sample
// t of the tile.  Layer 1 (5 inputs) runs in FP32 on the CUDA cores; layers
// 2-4 and every backward product on the tensor cores with tcgen05.mma (BF16
// operands in shared memory, FP32 accumulators in TMEM):
//   forward      Z_l = H_{l-1} W_l^T                      (M = 128 samples)
//   backward     dH_{l-1} = dZ_l W_l                      (B operand W_l^T)
//   weights      dW_l += dZ_l^T [H_{l-1} | 1]             (M = output units,
//                                                          K = 128 samples)
// The column of ones appended to H_{l-1} makes the bias gradient the last
// column of the weight-gradient accumulator.  Weight gradients accumulate in
// TMEM over all of a CTA's tiles and reach global memory once per CTA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "fr_guide.cuh"
#include "fr_kernels.h"
#include "fr_tc.cuh"

namespace fr {
namespace {

// Shared-memory plan of the training kernel (bytes).
constexpr int kSmW = 0;                             // weight tiles (kTileBytes)
constexpr int kSmH1 = kSmW + kTileBytes;            // H1, H2, H3: 128 x 64
constexpr int kSmH2 = kSmH1 + 128 * 64 * 2;
constexpr int kSmH3 = kSmH2 + 128 * 64 * 2;
constexpr int kSmDO = kSmH3 + 128 * 64 * 2;         // dZ4: 128 x 48
constexpr int kSmDH = kSmDO + 128 * 48 * 2;         // dZ3 / dZ2: 128 x 64
constexpr int kSmAT = kSmDH + 128 * 64 * 2;         // dZ^T: 128 (units, padded) x 128 (samples)
constexpr int kSmBT = kSmAT + 128 * 128 * 2;        // [H | 1]^T: 80 x 128
constexpr int kSmP1 = kSmBT + 80 * 128 * 2;         // W1, b1 (FP32)
constexpr int kSmB = kSmP1 + (kOffW2 - kOffW1) * 4; // b2, b3, b4 (FP32)
constexpr int kSmMisc = kSmB + (64 + 64 + 48) * 4;  // TMEM address, mbarrier, weight sum
constexpr int kTrainSmem = kSmMisc + 64;

// TMEM columns of the training kernel.
constexpr uint32_t kTmWork = 0, kTmG4 = 64, kTmG3 = 144, kTmG2 = 224, kTmG1 = 304, kTmCols = 512;

__global__ void __launch_bounds__(128) k_guide_train(GuideGPU g) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* W = sm + kSmW;
  uint8_t *H1 = sm + kSmH1, *H2 = sm + kSmH2, *H3 = sm + kSmH3, *DO = sm + kSmDO, *DH = sm + kSmDH;
  uint8_t *AT = sm + kSmAT, *BT = sm + kSmBT;
  float* p1 = reinterpret_cast<float*>(sm + kSmP1);
  float* bias = reinterpret_cast<float*>(sm + kSmB);  // b2 [0,64), b3 [64,128), b4 [128,176)
  uint32_t* tbase = reinterpret_cast<uint32_t*>(sm + kSmMisc);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kSmMisc + 8);
  float* wsum = reinterpret_cast<float*>(sm + kSmMisc + 16);  // one per warp
  const uint32_t t = threadIdx.x, warp = t >> 5;

  const uint32_t n_all = min(*g.batch_count, (uint32_t)g.batch_cap);
  const uint32_t tiles = (n_all + 127) / 128;
  if (blockIdx.x >= tiles) return;  // uniform per CTA

  // Weights and biases into shared memory; AT and BT start at zero.
  for (uint32_t e = t; e < (uint32_t)kTileBytes / 16; e += 128)
    reinterpret_cast<uint4*>(W)[e] = reinterpret_cast<const uint4*>(g.tiles)[e];
  for (uint32_t e = t; e < (uint32_t)kOffW2; e += 128) p1[e] = g.params[e];
  for (uint32_t e = t; e < 64; e += 128) {
    bias[e] = g.params[kOffB2 + e];
    bias[64 + e] = g.params[kOffB3 + e];
  }
  for (uint32_t e = t; e < 48; e += 128) bias[128 + e] = g.params[kOffB4 + e];
  for (uint32_t e = t; e < (128 * 128 * 2 + 80 * 128 * 2) / 16; e += 128) reinterpret_cast<uint4*>(AT)[e] = uint4{0, 0, 0, 0};
  if (t == 0) tc::mbar_init(bar, 1);
  if (warp == 0) tc::tmem_alloc(tbase, kTmCols);
  publish();
  const uint32_t tm = *tbase;
  const uint32_t lane_addr = tm + ((warp * 32u) << 16);
  const uint32_t aW2 = tc::smem_addr(W + kTileW2), aW3 = tc::smem_addr(W + kTileW3), aW4 = tc::smem_addr(W + kTileW4);
  const uint32_t aW2T = tc::smem_addr(W + kTileW2T), aW3T = tc::smem_addr(W + kTileW3T),
                 aW4T = tc::smem_addr(W + kTileW4T);
  const uint32_t aH1 = tc::smem_addr(H1), aH2 = tc::smem_addr(H2), aH3 = tc::smem_addr(H3);
  const uint32_t aDO = tc::smem_addr(DO), aDH = tc::smem_addr(DH), aAT = tc::smem_addr(AT), aBT = tc::smem_addr(BT);
  TcSync sy{bar, 0u, true};
  float my_wsum = 0.0f;
  bool first = true;

  for (uint32_t tile = blockIdx.x; tile < tiles && sy.ok; tile += gridDim.x) {
    const uint32_t j0 = tile * 128 + t;
    float x[kGuideIn] = {0.f, 0.f, 0.f, 0.f, 0.f};
    V3 d = v3(0.f, 0.f, 1.f);
    float I = 0.0f;
    if (j0 < n_all) {
      const float4 f = g.batch_feat[j0], dd = g.batch_dir[j0];
      x[0] = f.x; x[1] = f.y; x[2] = f.z; x[3] = f.w; x[4] = dd.x;
      d = v3(dd.y, dd.z, dd.w);
      I = g.batch_w[j0];
    }
    my_wsum += I;
    // ---- forward
    guide_layer1(p1, x, H1, t);
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aH1, aW2, 64, 64, false);
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    guide_hidden_epilogue(lane_addr + kTmWork, bias, H2, t);
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aH2, aW3, 64, 64, false);
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    guide_hidden_epilogue(lane_addr + kTmWork, bias + 64, H3, t);
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aH3, aW4, kGuideOutPad, 64, false);
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    float o[kGuideOut];
    guide_output_epilogue(lane_addr + kTmWork, bias + 128, o);
    // ---- loss gradient at the output, dZ4 and [H3 | 1]^T
    GuideMixture mix;
    guide_mixture(o, mix);
    float dout[kGuideOut];
    guide_loss_grad(mix, d, I, dout);
    for (int k = 0; k < kGuideOutPad; ++k) {
      const float v = k < kGuideOut ? dout[k] : 0.0f;
      st_bf16(DO, t, k, 48, v);
      st_bf16(AT, k, t, 128, v);
    }
    for (int k = kGuideOutPad; k < 64; ++k) st_bf16(AT, k, t, 128, 0.0f);
    for (int k = 0; k < 64; ++k) st_bf16(BT, k, t, 128, ld_bf16(H3, t, k, 64));
    st_bf16(BT, 64, t, 128, 1.0f);
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aDO, aW4T, 64, 48, false);     // dH3 = dZ4 W4
      tc::gemm_issue(tm + kTmG4, aAT, aBT, 80, 128, !first);      // dW4 += dZ4^T [H3 | 1]
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    // ---- layer 3: dZ3 = dH3 * relu'(Z3); [H2 | 1]^T
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(lane_addr + kTmWork + c0, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float dz = ld_bf16(H3, t, c0 + k, 64) > 0.0f ? v[k] : 0.0f;
        st_bf16(DH, t, c0 + k, 64, dz);
        st_bf16(AT, c0 + k, t, 128, dz);
      }
    }
    for (int k = 0; k < 64; ++k) st_bf16(BT, k, t, 128, ld_bf16(H2, t, k, 64));
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aDH, aW3T, 64, 64, false);     // dH2 = dZ3 W3
      tc::gemm_issue(tm + kTmG3, aAT, aBT, 80, 128, !first);      // dW3 += dZ3^T [H2 | 1]
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    // ---- layer 2: dZ2; [H1 | 1]^T
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(lane_addr + kTmWork + c0, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float dz = ld_bf16(H2, t, c0 + k, 64) > 0.0f ? v[k] : 0.0f;
        st_bf16(DH, t, c0 + k, 64, dz);
        st_bf16(AT, c0 + k, t, 128, dz);
      }
    }
    for (int k = 0; k < 64; ++k) st_bf16(BT, k, t, 128, ld_bf16(H1, t, k, 64));
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmWork, aDH, aW2T, 64, 64, false);     // dH1 = dZ2 W2
      tc::gemm_issue(tm + kTmG2, aAT, aBT, 80, 128, !first);      // dW2 += dZ2^T [H1 | 1]
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    // ---- layer 1: dZ1; [x | 1 | 0]^T (16 rows)
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(lane_addr + kTmWork + c0, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) st_bf16(AT, c0 + k, t, 128, ld_bf16(H1, t, c0 + k, 64) > 0.0f ? v[k] : 0.0f);
    }
    for (int k = 0; k < 16; ++k) st_bf16(BT, k, t, 128, k < kGuideIn ? x[k] : (k == kGuideIn ? 1.0f : 0.0f));
    publish();
    if (t == 0) {
      tc::gemm_issue(tm + kTmG1, aAT, aBT, 16, 128, !first);      // dW1 += dZ1^T [x | 1]
      tc::mma_commit(bar);
    }
    if (!sy.wait()) break;
    // The next tile rewrites rows 0-64 of BT (64: ones) and 0-63 of AT; AT
    // rows 64-127 and BT rows 65-79 stay zero.
    first = false;
  }
  // ---- gradient sums of this CTA to its own row of grad_part (thread t:
  // unit t); k_guide_adam (and k_guide_reduce) add the rows in CTA order, so the step's
  // gradient does not depend on which CTA finishes first.
  float* gp = g.grad_part + (size_t)blockIdx.x * kGuideParams;
  if (!first && sy.ok) {
    float v[16];
    for (int c0 = 0; c0 < 80; c0 += 16) {
      tc::tmem_ld16(lane_addr + kTmG4 + c0, v);
      for (int k = 0; k < 16; ++k) {
        const int c = c0 + k;
        if (t < (uint32_t)kGuideOut && c < 64) gp[kOffW4 + t * 64 + c] = v[k];
        if (t < (uint32_t)kGuideOut && c == 64) gp[kOffB4 + t] = v[k];
      }
      tc::tmem_ld16(lane_addr + kTmG3 + c0, v);
      for (int k = 0; k < 16; ++k) {
        const int c = c0 + k;
        if (t < 64 && c < 64) gp[kOffW3 + t * 64 + c] = v[k];
        if (t < 64 && c == 64) gp[kOffB3 + t] = v[k];
      }
      tc::tmem_ld16(lane_addr + kTmG2 + c0, v);
      for (int k = 0; k < 16; ++k) {
        const int c = c0 + k;
        if (t < 64 && c < 64) gp[kOffW2 + t * 64 + c] = v[k];
        if (t < 64 && c == 64) gp[kOffB2 + t] = v[k];
      }
    }
    tc::tmem_ld16(lane_addr + kTmG1, v);
    if (t < 64) {
      for (int k = 0; k < kGuideIn; ++k) gp[kOffW1 + t * kGuideIn + k] = v[k];
      gp[kOffB1 + t] = v[kGuideIn];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_wsum += __shfl_down_sync(0xffffffffu, my_wsum, o);
    if ((t & 31) == 0) wsum[warp] = my_wsum;
  } else {
    // A wait gave up: this CTA's row adds nothing.
    for (uint32_t e = t; e < (uint32_t)kGuideParams; e += 128) gp[e] = 0.0f;
    if ((t & 31) == 0) wsum[warp] = 0.0f;
  }
  if (!sy.ok && t == 0) atomicOr(g.err, kErrGuide);
  tc::fence_before_sync();
  __syncthreads();
  if (t == 0) g.wsum_part[blockIdx.x] = ((wsum[0] + wsum[1]) + wsum[2]) + wsum[3];
  if (warp == 0) tc::tmem_dealloc(tm, kTmCols);
}

// The BF16 weight tiles from the FP32 parameters.
__global__ void k_guide_prepare(GuideGPU g) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 64 * 64; e += gridDim.x * blockDim.x) {
    const int r = e / 64, k = e % 64;
    st_bf16(g.tiles + kTileW2, r, k, 64, g.params[kOffW2 + r * 64 + k]);
    st_bf16(g.tiles + kTileW3, r, k, 64, g.params[kOffW3 + r * 64 + k]);
    st_bf16(g.tiles + kTileW2T, r, k, 64, g.params[kOffW2 + k * 64 + r]);
    st_bf16(g.tiles + kTileW3T, r, k, 64, g.params[kOffW3 + k * 64 + r]);
    if (r < kGuideOutPad) st_bf16(g.tiles + kTileW4, r, k, 64, g.params[kOffW4 + r * 64 + k]);
    if (k < kGuideOutPad) st_bf16(g.tiles + kTileW4T, r, k, 48, g.params[kOffW4 + k * 64 + r]);
  }
}

// The step's gradient sum for parameter p: the training CTAs' rows added in
// CTA order (rows of CTAs that had no tile are not read).
__device__ __forceinline__ uint32_t guide_rows(const GuideGPU& g) {
  const uint32_t n_all = min(*g.batch_count, (uint32_t)g.batch_cap);
  return min((n_all + 127) / 128, (uint32_t)g.train_ctas);
}
__device__ __forceinline__ float guide_grad_sum(const GuideGPU& g, uint32_t rows, int p) {
  float sum = 0.0f;
  for (uint32_t r = 0; r < rows; ++r) sum += g.grad_part[(size_t)r * kGuideParams + p];
  return sum;
}
__device__ __forceinline__ float guide_weight_sum(const GuideGPU& g, uint32_t rows) {
  float ws = 0.0f;
  for (uint32_t r = 0; r < rows; ++r) ws += g.wsum_part[r];
  return ws;
}
__device__ __forceinline__ bool guide_pad(int p) {
  return (p >= kOffW4 + kGuideOut * 64 && p < kOffB4) || p >= kOffB4 + kGuideOut;
}

// One training step after the gradient pass, in one kernel: the gradient sum
// of each parameter (rows in CTA order), Adam on the mean gradient (sum / sum
// of importance; learning rate g.lr, beta 0.9 / 0.999), and the parameter's
// BF16 entries in the forward and transposed weight tiles (W2, W3, W4; W1 and
// the biases stay FP32).  The padding outputs 40-47 stay zero.  Block 0 also
// stores the importance sum for k_guide_step_done.
__global__ void k_guide_adam(GuideGPU g) {
  const uint32_t rows = guide_rows(g);
  const float ws = guide_weight_sum(g, rows);  // the same value in every thread
  if (blockIdx.x == 0 && threadIdx.x == 0) *g.weight_sum = ws;
  const uint32_t step = *g.adam_step + 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x) {
    if (guide_pad(p) || !(ws > 0.0f)) continue;
    const float gr = guide_grad_sum(g, rows, p) / ws;
    const float m = b1 * g.adam_m[p] + (1.0f - b1) * gr;
    const float v = b2 * g.adam_v[p] + (1.0f - b2) * gr * gr;
    g.adam_m[p] = m;
    g.adam_v[p] = v;
    const float w = g.params[p] - g.lr * (m / c1) / (sqrtf(v / c2) + eps);
    g.params[p] = w;
    if (p >= kOffW2 && p < kOffB2) {
      const int r = (p - kOffW2) / 64, k = (p - kOffW2) % 64;
      st_bf16(g.tiles + kTileW2, r, k, 64, w);
      st_bf16(g.tiles + kTileW2T, k, r, 64, w);
    } else if (p >= kOffW3 && p < kOffB3) {
      const int r = (p - kOffW3) / 64, k = (p - kOffW3) % 64;
      st_bf16(g.tiles + kTileW3, r, k, 64, w);
      st_bf16(g.tiles + kTileW3T, k, r, 64, w);
    } else if (p >= kOffW4 && p < kOffB4) {
      const int r = (p - kOffW4) / 64, k = (p - kOffW4) % 64;
      st_bf16(g.tiles + kTileW4, r, k, 64, w);
      st_bf16(g.tiles + kTileW4T, k, r, 48, w);
    }
  }
}

__global__ void k_guide_step_done(GuideGPU g, int last) {
  if (*g.weight_sum > 0.0f) *g.adam_step += 1;
  *g.weight_sum = 0.0f;
  if (last) *g.batch_count = 0;
}

// Paths whose photons reached a hitpoint, as training samples, in path
// order (so the batch, and with it the training, is the same run to run):
// per-block counts, one exclusive scan of them, then each block writes its
// paths at its offset.  The first batch_cap such paths are taken; a path's
// index says nothing about its photons, so they are an unbiased subset.
constexpr int kSelectBlock = 256;
constexpr int kSelectScanThreads = 1024;

__device__ __forceinline__ bool guide_takes(const GuideGPU& g, int i, int paths) {
  return i < paths && (g.importance[2 * (size_t)i] | g.importance[2 * (size_t)i + 1]) != 0ull;
}

// Number of paths a block takes, and each thread's rank among them.
__device__ __forceinline__ uint32_t select_block_rank(bool take, uint32_t* rank) {
  __shared__ uint32_t s_warp[kSelectBlock / 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t bal = __ballot_sync(0xffffffffu, take);
  if (lane == 0) s_warp[warp] = __popc(bal);
  __syncthreads();
  uint32_t before = 0, total = 0;
  for (uint32_t w = 0; w < kSelectBlock / 32; ++w) {
    if (w < warp) before += s_warp[w];
    total += s_warp[w];
  }
  *rank = before + __popc(bal & ((1u << lane) - 1u));
  return total;
}

__global__ void __launch_bounds__(kSelectBlock) k_guide_select_count(GuideGPU g, int paths) {
  uint32_t rank;
  const uint32_t n = select_block_rank(guide_takes(g, blockIdx.x * kSelectBlock + threadIdx.x, paths), &rank);
  if (threadIdx.x == 0) g.select_part[blockIdx.x] = n;
}

// One block: select_part[0..blocks) becomes exclusive offsets; batch_count
// the number of paths taken (before the cap).
__global__ void __launch_bounds__(kSelectScanThreads) k_guide_select_scan(GuideGPU g, int blocks) {
  __shared__ uint32_t s_sum[kSelectScanThreads];
  const uint32_t t = threadIdx.x;
  const uint32_t per = (blocks + kSelectScanThreads - 1) / kSelectScanThreads;
  const uint32_t b0 = t * per, b1 = min(b0 + per, (uint32_t)blocks);
  uint32_t mine = 0;
  for (uint32_t b = b0; b < b1; ++b) mine += g.select_part[b];
  s_sum[t] = mine;
  __syncthreads();
  for (uint32_t o = 1; o < kSelectScanThreads; o <<= 1) {  // inclusive Hillis-Steele scan
    const uint32_t v = t >= o ? s_sum[t - o] : 0u;
    __syncthreads();
    s_sum[t] += v;
    __syncthreads();
  }
  uint32_t run = s_sum[t] - mine;
  for (uint32_t b = b0; b < b1; ++b) {
    const uint32_t c = g.select_part[b];
    g.select_part[b] = run;
    run += c;
  }
  if (t == kSelectScanThreads - 1) *g.batch_count = s_sum[t];
}

__global__ void __launch_bounds__(kSelectBlock) k_guide_select_write(GuideGPU g, int paths) {
  const int i = blockIdx.x * kSelectBlock + threadIdx.x;
  const bool take = guide_takes(g, i, paths);
  uint32_t rank;
  select_block_rank(take, &rank);
  const uint32_t slot = g.select_part[blockIdx.x] + rank;
  if (take && slot < (uint32_t)g.batch_cap) {
    g.batch[slot] = (uint32_t)i;
    g.batch_w[slot] = importance_value(g.importance[2 * (size_t)i], g.importance[2 * (size_t)i + 1]);
    g.batch_feat[slot] = g.feat[i];
    g.batch_dir[slot] = g.dir[i];
  }
}

// The step's gradient and importance sums alone (fr_guide_gradient): the
// same sums k_guide_adam forms.
__global__ void k_guide_reduce(GuideGPU g) {
  const uint32_t rows = guide_rows(g);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x)
    g.grad[p] = guide_pad(p) ? 0.0f : guide_grad_sum(g, rows, p);
  if (blockIdx.x == 0 && threadIdx.x == 0) *g.weight_sum = guide_weight_sum(g, rows);
}

inline void launch_guide_select(const GuideGPU& g, int paths, cudaStream_t s) {
  const int blocks = (paths + kSelectBlock - 1) / kSelectBlock;
  k_guide_select_count<<<blocks, kSelectBlock, 0, s>>>(g, paths);
  k_guide_select_scan<<<1, kSelectScanThreads, 0, s>>>(g, blocks);
  k_guide_select_write<<<blocks, kSelectBlock, 0, s>>>(g, paths);
}

}  // namespace

int guide_train_smem() { return kTrainSmem; }

// The sample selection of an iteration: its paths with importance, their
// importance, inputs and directions copied into the batch.  Returns the
// kernels launched.
int launch_guide_select_batch(const GuideGPU& g, int paths, cudaStream_t s) {
  launch_guide_select(g, paths, s);
  return 3;
}

// g.steps Adam steps on the selected samples (each a gradient pass with the
// current weights).  Returns the kernels launched.
int launch_guide_steps(const GuideGPU& g, cudaStream_t s) {
  for (int k = 0; k < g.steps; ++k) {
    k_guide_train<<<g.train_ctas, 128, kTrainSmem, s>>>(g);
    k_guide_adam<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g);
    k_guide_step_done<<<1, 1, 0, s>>>(g, k == g.steps - 1);
  }
  return 3 * g.steps;
}

// The training's weights become the emission's (two device copies).
int launch_guide_publish(const GuideGPU& g, cudaStream_t s) {
  if (cudaMemcpyAsync(g.emit_params, g.params, sizeof(float) * kGuideParams, cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(g.emit_tiles, g.tiles, kTileBytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return -1;
  return 0;
}

void launch_guide_prepare(const GuideGPU& g, cudaStream_t s) { k_guide_prepare<<<16, 256, 0, s>>>(g); }

void launch_guide_gradients(const GuideGPU& g, int paths, cudaStream_t s) {
  launch_guide_select(g, paths, s);
  k_guide_train<<<g.train_ctas, 128, kTrainSmem, s>>>(g);
  k_guide_reduce<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g);
}

int guide_select_blocks(int paths) { return (paths + kSelectBlock - 1) / kSelectBlock; }

int guide_configure() {
  return cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem) == cudaSuccess
             ? 0
             : -1;
}

// Initial parameters: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero
// hidden biases; lobe means from the output biases spread over the sphere,
// broad concentrations (raw 0) and equal weights.
std::vector<float> guide_initial_params(uint32_t seed) {
  std::vector<float> p(kGuideParams, 0.0f);
  std::mt19937 gen(seed);
  auto fill = [&](int off, int n_out, int n_in) {
    std::uniform_real_distribution<float> u(-1.0f / std::sqrt((float)n_in), 1.0f / std::sqrt((float)n_in));
    for (int k = 0; k < n_out * n_in; ++k) p[off + k] = u(gen);
  };
  fill(kOffW1, kGuideHidden, kGuideIn);
  fill(kOffW2, kGuideHidden, kGuideHidden);
  fill(kOffW3, kGuideHidden, kGuideHidden);
  fill(kOffW4, kGuideOut, kGuideHidden);
  for (int k = 0; k < kGuideLobes; ++k) {  // Fibonacci sphere directions, scaled
    const float z = 1.0f - (2.0f * k + 1.0f) / kGuideLobes;
    const float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
    const float ph = 2.39996323f * k;
    p[kOffB4 + 5 * k] = 2.0f * r * std::cos(ph);
    p[kOffB4 + 5 * k + 1] = 2.0f * z;
    p[kOffB4 + 5 * k + 2] = 2.0f * r * std::sin(ph);
  }
  return p;
}

}  // namespace fr
