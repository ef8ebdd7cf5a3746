// fvx_tc.cuh -- 5th-generation tensor-core (tcgen05) building blocks, sm_103a.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzle: a tile of R rows x K columns of BF16 is stored as 8-row x 16-byte
// "core matrices" of 128 contiguous bytes; element (r, k) sits at byte
//   ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent along K are 128 B apart and 8-row groups are
// K/8 * 128 B apart (the two strides the matrix descriptor carries).  The
// accumulator (M = 128 rows x N FP32 columns) lives in tensor memory, row i
// in lane i; one elected thread issues tcgen05.mma, completion is committed to
// an mbarrier and every wait on it is bounded.
#pragma once

#include <cuda_bf16.h>

#include "fvx_common.cuh"

namespace fvx {
namespace tc {

// byte offset of element (r, k) in a K-major canonical tile with K columns
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
  return static_cast<uint32_t>(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices along K), stride-dimension byte offset
// (between 8-row groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;  // version
  return d;                             // base offset 0, swizzle none
}

// Instruction descriptor of kind::f16 with BF16 A/B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                                  // D = F32
         | (1u << 7)                                // A = BF16
         | (1u << 10)                               // B = BF16
         | (static_cast<uint32_t>(N >> 3) << 17)    // N / 8
         | (static_cast<uint32_t>(M >> 4) << 24);   // M / 16
}

// Instruction descriptor of kind::f16 with F16 A/B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4)                                  // D = F32; A = B = F16 (format 0)
         | (static_cast<uint32_t>(N >> 3) << 17)    // N / 8
         | (static_cast<uint32_t>(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
      " [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Split form of tmem_ld16, so that a load can be in flight while the previous
// chunk is processed: issue, then wait.  The wait names the registers as
// read-write operands, which keeps every use of them after it.  Neither
// clobbers memory (TMEM is not C++ memory; both stay ordered with the other
// volatile tcgen05 statements), so shared-memory loads and stores of the
// epilogue may be scheduled across them.
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
      " [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}

// Issues the K/16 MMAs of D[128 x N] (+)= A[128 x K] B[N x K]^T from one
// thread, then commits to `bar`.  lbo/sbo: descriptor strides of the tiles.
__device__ __forceinline__ void gemm_issue(uint32_t d_tmem, const void* A, const void* B, int K,
                                          uint32_t idesc, bool accumulate, uint64_t* bar,
                                          int stride_mode) {
  const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
  const uint32_t kgrp = static_cast<uint32_t>(K >> 3) * 128u;  // 8-row group stride
  const uint32_t lbo = stride_mode == 0 ? 128u : kgrp;
  const uint32_t sbo = stride_mode == 0 ? kgrp : 128u;
  for (int kk = 0; kk < K / 16; ++kk) {
    const uint32_t off = static_cast<uint32_t>(kk) * 256u;  // two core matrices along K
    mma_bf16(d_tmem, smem_desc(a0 + off, lbo, sbo), smem_desc(b0 + off, lbo, sbo), idesc,
             (accumulate || kk > 0) ? 1u : 0u);
  }
  mma_commit(bar);
}

}  // namespace tc
}  // namespace fvx
