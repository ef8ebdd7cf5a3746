// fvx_mlp.cu -- BF16 tensor-core MLP of the learned far-field operator.
//
// Network: 48 inputs (35 features, zero padded) -> 3 x 128 hidden (SiLU) ->
// 16 outputs (12 used), weights [out][in] in BF16 with FP32 master copies,
// FP32 biases.  Inference and training run on tcgen05 (fvx_tc.cuh): one CTA
// of 128 threads takes 128-row tiles (persistent over the tiles), keeps all
// weights in shared memory in the K-major canonical layout, and chains the
// four layers through tensor memory: MMA into TMEM -> tcgen05.ld -> bias +
// SiLU in registers -> BF16 back into the shared activation tile -> next MMA.
// The backward pass uses the same machinery for dX = dZ W (weights staged
// transposed) and dW = dZ^T X (operands staged transposed, one MMA chain per
// 128-row tile, partial dW accumulated across CTAs with FP32 atomics).
#include <cuda_bf16.h>

#include "fvx_common.cuh"
#include "fvx_tc.cuh"

namespace fvx {
namespace mlp {

constexpr int IN = 48, H = 128, OUT = 16;
constexpr int kThreads = 128;
// packed BF16 weight offsets (elements)
constexpr int W1o = 0, W2o = W1o + H * IN, W3o = W2o + H * H, W4o = W3o + H * H,
              WN = W4o + OUT * H;
// packed bias offsets
constexpr int B1o = 0, B2o = H, B3o = 2 * H, B4o = 3 * H, BN = 3 * H + OUT;

struct FwdSmem {
  __nv_bfloat16 w1[H * IN];
  __nv_bfloat16 w2[H * H];
  __nv_bfloat16 w3[H * H];
  __nv_bfloat16 w4[OUT * H];
  __nv_bfloat16 act[128 * H];
  float bias[BN];
  uint64_t bar;
  uint32_t tmem;
};

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }

// Copies a row-major [R][K] BF16 matrix into the K-major canonical layout.
__device__ void stage_kmajor(__nv_bfloat16* dst, const __nv_bfloat16* src, int R, int K) {
  const int chunks = R * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    const int r = c / (K / 8), k8 = c % (K / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(src + static_cast<int64_t>(r) * K + 8 * k8);
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(dst) + tc::kmajor_offset(r, 8 * k8, K)) = v;
  }
}

// this thread's row of a 128 x H accumulator -> bias + SiLU -> BF16 act tile;
// optionally keeps the pre-activation (FP32) and activation (BF16) rows
__device__ void epilogue_hidden(uint32_t tmem, const float* bias, __nv_bfloat16* act, int row,
                                float* z_out, __nv_bfloat16* h_out) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lane_base = static_cast<uint32_t>(32 * (warp & 3)) << 16;
  for (int c0 = 0; c0 < H; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tmem + lane_base + c0, v);
    __align__(16) __nv_bfloat16 b[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const float z = v[i] + bias[c0 + i];
      if (z_out) z_out[c0 + i] = z;
      b[i] = __float2bfloat16(silu(z));
    }
    char* base = reinterpret_cast<char*>(act);
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(threadIdx.x, c0, H)) =
        *reinterpret_cast<uint4*>(&b[0]);
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(threadIdx.x, c0 + 8, H)) =
        *reinterpret_cast<uint4*>(&b[8]);
    if (h_out) {
      *reinterpret_cast<uint4*>(h_out + c0) = *reinterpret_cast<uint4*>(&b[0]);
      *reinterpret_cast<uint4*>(h_out + c0 + 8) = *reinterpret_cast<uint4*>(&b[8]);
    }
  }
  (void)row;
}

// Waits for the MMA chain committed to `bar` (phase `ph`), bounded.
__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& ph) {
  const bool ok = mbar_wait(bar, ph);
  ph ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// Y[rows][16] = MLP(X[rows][48]); with z/h stores for training.
__global__ void __launch_bounds__(kThreads) mlp_fwd_kernel(
    const __nv_bfloat16* __restrict__ X, int rows, const __nv_bfloat16* __restrict__ W,
    const float* __restrict__ bias, float* __restrict__ Y, float* __restrict__ z_store,
    __nv_bfloat16* __restrict__ h_store, int stride_mode) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  FwdSmem& S = *reinterpret_cast<FwdSmem*>(smem_raw);
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, 128);
  if (threadIdx.x == 0) {
    mbar_init(&S.bar, 1);
    fence_mbar_init();
  }
  stage_kmajor(S.w1, W + W1o, H, IN);
  stage_kmajor(S.w2, W + W2o, H, H);
  stage_kmajor(S.w3, W + W3o, H, H);
  stage_kmajor(S.w4, W + W4o, OUT, H);
  for (int i = threadIdx.x; i < BN; i += blockDim.x) S.bias[i] = bias[i];
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  uint32_t ph = 0;
  bool ok = true;
  const int ntiles = (rows + 127) / 128;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int row = tile * 128 + threadIdx.x;
    const bool act_row = row < rows;
    // input tile (K = 48)
    {
      char* base = reinterpret_cast<char*>(S.act);
      for (int k8 = 0; k8 < IN / 8; ++k8) {
        uint4 v = make_uint4(0, 0, 0, 0);
        if (act_row)
          v = *reinterpret_cast<const uint4*>(X + static_cast<int64_t>(row) * IN + 8 * k8);
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(threadIdx.x, 8 * k8, IN)) = v;
      }
    }
    const __nv_bfloat16* wl[3] = {S.w1, S.w2, S.w3};
    for (int l = 0; l < 3 && ok; ++l) {
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (threadIdx.x == 0)
        tc::gemm_issue(tmem, S.act, wl[l], l == 0 ? IN : H, tc::idesc_bf16(128, H), false,
                       &S.bar, stride_mode);
      if (!__syncthreads_and(wait_mma(&S.bar, ph))) {
        ok = false;
        break;
      }
      epilogue_hidden(tmem, S.bias + l * H, S.act, row,
                      (z_store && act_row) ? z_store + (static_cast<int64_t>(l) * rows + row) * H
                                           : nullptr,
                      (h_store && act_row) ? h_store + (static_cast<int64_t>(l) * rows + row) * H
                                           : nullptr);
    }
    if (!ok) break;
    // output layer (N = 16)
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0)
      tc::gemm_issue(tmem, S.act, S.w4, H, tc::idesc_bf16(128, OUT), false, &S.bar, stride_mode);
    if (!__syncthreads_and(wait_mma(&S.bar, ph))) {
      ok = false;
      break;
    }
    float v[16];
    tc::tmem_ld16(tmem + (static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16), v);
    if (act_row) {
      float4* y = reinterpret_cast<float4*>(Y + static_cast<int64_t>(row) * OUT);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        y[q] = make_float4(v[4 * q] + S.bias[B4o + 4 * q], v[4 * q + 1] + S.bias[B4o + 4 * q + 1],
                           v[4 * q + 2] + S.bias[B4o + 4 * q + 2],
                           v[4 * q + 3] + S.bias[B4o + 4 * q + 3]);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (!ok && threadIdx.x == 0) flag_status(kStatusTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 128);
}

// ---- probe: C[128][N] = A[128][K] B[N][K]^T (validates layouts / descriptors) ----
__global__ void __launch_bounds__(128) gemm_probe_kernel(const __nv_bfloat16* __restrict__ A,
                                                         const __nv_bfloat16* __restrict__ B,
                                                         int N, int K, float* __restrict__ C,
                                                         int stride_mode) {
  __shared__ __align__(1024) __nv_bfloat16 sA[128 * 128];
  __shared__ __align__(1024) __nv_bfloat16 sB[128 * 128];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  if (threadIdx.x < 32) tc::tmem_alloc(&tslot, 128);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  stage_kmajor(sA, A, 128, K);
  stage_kmajor(sB, B, N, K);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) tc::gemm_issue(tmem, sA, sB, K, tc::idesc_bf16(128, N), false, &bar, stride_mode);
  uint32_t ph = 0;
  const bool ok = __syncthreads_and(wait_mma(&bar, ph));
  if (ok) {
    const uint32_t lb = static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lb + c0, v);
      for (int i = 0; i < 16; ++i) C[threadIdx.x * N + c0 + i] = v[i];
    }
  } else if (threadIdx.x == 0) {
    flag_status(kStatusTimeout);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 128);
}

}  // namespace mlp
}  // namespace fvx

extern "C" {

int fvx_tc_gemm_probe(const void* A, const void* B, int N, int K, float* C, int stride_mode,
                      void* stream) {
  FVX_ARG_CHECK(A && B && C, "null pointer");
  FVX_ARG_CHECK(N >= 16 && N <= 128 && N % 16 == 0 && K >= 16 && K <= 128 && K % 16 == 0,
                "probe needs 16 <= N, K <= 128, multiples of 16");
  FVX_ARG_CHECK(stride_mode == 0 || stride_mode == 1, "bad stride mode");
  fvx::mlp::gemm_probe_kernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), N, K, C,
      stride_mode);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_forward(const void* X, int rows, const void* W, const float* bias, float* Y,
                    float* z_store, void* h_store, int stride_mode, void* stream) {
  using namespace fvx::mlp;
  FVX_ARG_CHECK(rows >= 0 && X && W && bias && Y, "null argument");
  if (rows == 0) return FVX_OK;
  const size_t smem = sizeof(FwdSmem);
  static bool attr_set = false;
  if (!attr_set) {
    FVX_CUDA_TRY(cudaFuncSetAttribute(mlp_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
    attr_set = true;
  }
  const int ntiles = (rows + 127) / 128;
  const int grid = ntiles < fvx::device_sm_count() ? ntiles : fvx::device_sm_count();
  mlp_fwd_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(X), rows, static_cast<const __nv_bfloat16*>(W), bias, Y,
      z_store, static_cast<__nv_bfloat16*>(h_store), stride_mode);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

}  // extern "C"
