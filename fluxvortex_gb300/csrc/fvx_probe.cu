// fvx_probe.cu -- FP32 FMA-throughput probe used by bench.py to measure the
// CUDA-core FP32 peak of the device it runs on (the denominator of the
// particle sweeps' roofline, which no library GEMM measures).
#include "fvx_common.cuh"

namespace fvx {
namespace {

// 8 independent FMA chains per thread; `iters` rounds of 8 FMAs each.
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, float seed, float* sink) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.9999f, c = 1e-7f;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
    a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
  }
  float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678f) sink[0] = s;  // keeps the chains live
}

}  // namespace
}  // namespace fvx

extern "C" int fvx_probe_fp32_fma(int blocks_per_sm, int iters, float* sink, void* stream) {
  FVX_ARG_CHECK(blocks_per_sm > 0 && iters > 0 && sink, "bad probe arguments");
  const int grid = blocks_per_sm * fvx::device_sm_count();
  fvx::fma_probe_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(iters, 1.0f, sink);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}
