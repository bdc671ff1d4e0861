// Device check of the tcgen05 GEMM block (fr_tc.cuh) against a host GEMM on
// the same BF16-rounded inputs: D = A * B^T (128x64x64), D += A * B^T
// (accumulate), and D = A * B[0:48]^T (N = 48).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "fr_kernels.h"
#include "fr_tc.cuh"

namespace fr {
namespace {

constexpr int kM = 128, kN = 64, kK = 64;

__global__ void __launch_bounds__(128) k_tc_check(const float* A, const float* B, float* D, int* err) {
  // Operand tiles (with room to spare), TMEM address, mbarrier.
  __shared__ __align__(1024) uint8_t sa[kM * kK * 2 + 8192];
  __shared__ __align__(1024) uint8_t sb[kN * kK * 2 + 4096];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t bar;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int e = t; e < kM * kK; e += blockDim.x) {
    const int r = e / kK, k = e % kK;
    *reinterpret_cast<__nv_bfloat16*>(sa + tc::tile_offset(r, k, kK)) = __float2bfloat16_rn(A[e]);
  }
  for (int e = t; e < kN * kK; e += blockDim.x) {
    const int r = e / kK, k = e % kK;
    *reinterpret_cast<__nv_bfloat16*>(sb + tc::tile_offset(r, k, kK)) = __float2bfloat16_rn(B[e]);
  }
  if (warp == 0) tc::tmem_alloc(&tbase, 128);
  if (t == 0) tc::mbar_init(&bar, 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tbase;
  const uint32_t a = tc::smem_addr(sa), b = tc::smem_addr(sb);
  bool ok = true;
  for (int pass = 0; pass < 3; ++pass) {
    if (t == 0) {
      if (pass < 2) tc::gemm_issue(tm, a, b, kN, kK, pass == 1);
      else tc::gemm_issue(tm + 64, a, b, 48, kK, false);
      tc::mma_commit(&bar);
    }
    ok = __syncthreads_and(tc::mbar_wait(&bar, (uint32_t)(pass & 1)) && ok) != 0;
    tc::fence_after_sync();
    if (!ok) break;
    const int row = warp * 32 + lane;
    const int ncol = pass < 2 ? kN : 48;
    for (int c0 = 0; c0 < ncol; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)((pass == 2 ? 64 : 0) + c0), v);
      for (int k = 0; k < 16; ++k) D[pass * kM * kN + row * kN + c0 + k] = v[k];
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (!ok && t == 0) atomicOr(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, 128);
}

float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

}  // namespace

int check_tc_gemm(uint32_t seed, double* max_err, const char** msg) {
  std::mt19937 gen(seed);
  std::uniform_real_distribution<float> u(-1.0f, 1.0f);
  std::vector<float> A(kM * kK), B(kN * kK);
  for (auto& x : A) x = u(gen);
  for (auto& x : B) x = u(gen);
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dErr = nullptr;
  if (cudaMalloc(&dA, A.size() * 4) || cudaMalloc(&dB, B.size() * 4) || cudaMalloc(&dD, 3 * kM * kN * 4) ||
      cudaMalloc(&dErr, 4)) {
    *msg = "cudaMalloc failed";
    return -1;
  }
  cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
  cudaMemset(dD, 0, 3 * kM * kN * 4);
  cudaMemset(dErr, 0, 4);
  k_tc_check<<<1, 128>>>(dA, dB, dD, dErr);
  std::vector<float> D(3 * kM * kN);
  int err = 0;
  const cudaError_t e = cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&err, dErr, 4, cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dErr);
  if (e != cudaSuccess) {
    *msg = cudaGetErrorString(e);
    return -1;
  }
  if (err) {
    *msg = "mbarrier wait gave up";
    return -1;
  }
  for (int p = 0; p < 3; ++p) max_err[p] = 0.0;
  for (int r = 0; r < kM; ++r)
    for (int c = 0; c < kN; ++c) {
      double ref = 0.0;
      for (int k = 0; k < kK; ++k) ref += (double)bf16_round(A[r * kK + k]) * (double)bf16_round(B[c * kK + k]);
      max_err[0] = std::fmax(max_err[0], std::fabs(D[r * kN + c] - ref));
      max_err[1] = std::fmax(max_err[1], std::fabs(D[kM * kN + r * kN + c] - 2.0 * ref));
      if (c < 48) max_err[2] = std::fmax(max_err[2], std::fabs(D[2 * kM * kN + r * kN + c] - ref));
    }
  return 0;
}

}  // namespace fr
