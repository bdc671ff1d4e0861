// Blackwell (sm_103a) tensor-core building block for the photon guide's MLP:
// D[128 x N] (+)= A[128 x K] * B[N x K]^T with BF16 operands in shared memory
// and an FP32 accumulator in tensor memory (TMEM), issued with tcgen05.mma by
// one thread, completion signalled through an mbarrier (tcgen05.commit), and
// read back with tcgen05.ld.
//
// Operand layout in shared memory ("K-major, no swizzle"): a tile of R rows by
// K bf16 columns is stored as 8x8 core matrices of 128 contiguous bytes (8
// rows of 16 bytes); core matrix (r/8, k/8) starts at ((r/8)*(K/8) + k/8)*128.
// In the shared-memory matrix descriptor the leading byte offset (between
// core matrices adjacent along K) is then 128 B and the stride byte offset
// (between 8-row groups) K/8 * 128 B.
//
// Every wait on an mbarrier is bounded: after kTcSpinLimit polls the wait
// gives up and reports failure, and the caller sets its error word.
#pragma once
#include <cstdint>

namespace fr {
namespace tc {

constexpr uint32_t kTcSpinLimit = 1u << 26;

// Byte offset of element (r, k) of a K-major tile with K columns.
__device__ __forceinline__ uint32_t tile_offset(uint32_t r, uint32_t k, uint32_t K) {
  return (((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading and stride
// byte offsets (all >> 4), descriptor version 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4)               // D format F32
         | (1u << 7)             // A format BF16
         | (1u << 10)            // B format BF16
         | ((N >> 3) << 17)      // N / 8
         | ((M >> 4) << 24);     // M / 16
}

// TMEM allocation by one full warp; the address lands in *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t n = 0; n < kTcSpinLimit; ++n) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Generic-proxy writes to shared memory made visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// One MMA: D[tmem] (+)= A(desc) * B(desc)^T for one K step of 16.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrive on *bar once every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// D[128 x N] (+)= A[128 x K] * B[N x K]^T from K-major tiles at sa / sb,
// K a multiple of 16; issued by the calling thread.
__device__ __forceinline__ void gemm_issue(uint32_t d_tmem, uint32_t sa, uint32_t sb, uint32_t N, uint32_t K,
                                          bool accumulate) {
  const uint32_t idesc = idesc_bf16(128, N);
  const uint32_t sbo = (K >> 3) << 7;
  for (uint32_t k = 0; k < K; k += 16) {
    const uint32_t koff = (k >> 3) << 7;  // two core matrices per K step
    mma_bf16(d_tmem, smem_desc(sa + koff, 128, sbo), smem_desc(sb + koff, 128, sbo), idesc, accumulate || k > 0);
  }
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w of the CTA
// reads lanes 32w..32w+31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace tc
}  // namespace fr
