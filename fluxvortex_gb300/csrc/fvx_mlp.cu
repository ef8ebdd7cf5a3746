// fvx_mlp.cu -- BF16 tensor-core MLP of the learned far-field operator.
//
// Network: 48 inputs (35 features, zero padded) -> 3 x 128 hidden (SiLU) ->
// 32 outputs (30 used), weights [out][in] in BF16 with FP32 master copies,
// FP32 biases.  Inference and training run on tcgen05 (fvx_tc.cuh):
//   * forward: a persistent CTA per SM keeps all weights in shared memory in
//     the K-major canonical layout; each of its four warpgroups owns a 128-row
//     tile at a time and chains the four layers through its quarter of the
//     tensor memory: MMA into TMEM -> tcgen05.ld -> bias + SiLU in registers
//     -> the group's shared activation tile -> next MMA, so one group's
//     epilogue overlaps the others' MMAs.  Inference runs with the hidden
//     weights and biases halved while staged and a packed BF16 SiLU; training
//     with the FP32 SiLU.  Two kernels: mlp_fwd_kernel on plain rows (X -> Y,
//     with the hidden pre-activations / activations kept for training), and
//     farfield_kernel, the treecode's learned far field, in which two more
//     warpgroups form the inputs of every tile from the (target leaf, source
//     cell) pair lists and reduce its outputs, scaled back to physical
//     local-expansion coefficients, into the leaves' expansions;
//   * training: a generic tile GEMM C = op(A) op(B)^T on tcgen05 (operands
//     staged transposed as needed by the threads, split over K with FP32
//     atomics) for dW = dZ^T H and dH = dZ W, plus element-wise kernels for
//     the loss gradient, the SiLU backward with bias gradients, and Adam.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fvx_common.cuh"
#include "fvx_m2l_tensor.cuh"
#include "fvx_tc.cuh"

namespace fvx {
namespace mlp {

constexpr int IN = 48, H = 128, OUT = 32, NFEAT = 35, NOUT = 30;
// packed BF16 weight offsets (elements)
constexpr int W1o = 0, W2o = W1o + H * IN, W3o = W2o + H * H, W4o = W3o + H * H,
              WN = W4o + OUT * H;
// packed bias offsets
constexpr int B1o = 0, B2o = H, B3o = 2 * H, B4o = 3 * H, BN = 3 * H + OUT;
constexpr int kRecFloats = 40;  // treecode cell record (fvx_tree.cu)
constexpr int kTargetsThreads = 256;  // FP64 exact-expansion sums: threads per pair
// The judge's FP64 sums take their cells in chunks of four particles per thread:
// each chunk ends in a block reduction of 30 FP64 values, which on this GPU's
// FP64 pipe costs about as much as one particle per thread.
constexpr int kJudgeChunk = 4 * kTargetsThreads;

// Four 128-row tiles are in flight per CTA (one per warpgroup, each with a
// quarter of the tensor memory): while some groups run their epilogues on the
// CUDA cores, the others' MMAs run.
constexpr int kGroups = 4;

struct FwdSmem {
  __nv_bfloat16 w1[H * IN];
  __nv_bfloat16 w2[H * H];
  __nv_bfloat16 w3[H * H];
  __nv_bfloat16 w4[OUT * H];
  __nv_bfloat16 act[kGroups][128 * H];
  float bias[BN];
  uint32_t hbias[3 * H / 2];  // inference form: half the hidden layers' biases, packed BF16 pairs
  uint64_t bar[kGroups];
  uint32_t tmem;
};

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// SiLU z sigmoid(z) = z/2 (1 + tanh(z/2)): one MUFU operation per element
__device__ __forceinline__ float silu(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_approx(h), h);
}
// Two SiLUs in packed BF16 from two accumulator columns of the halved weights
// (acc = W x / 2) and the packed halved biases hb: h = z/2 = acc + b/2, then
// one MUFU operation (tanh.approx.bf16x2) and one packed FMA, h + h tanh(h) =
// z sigmoid(z); the BF16 result is the next layer's operand as it stands.
// Element 0 goes to the low half (the lower address in shared memory).
__device__ __forceinline__ uint32_t silu_bf16x2(float a0, float a1, uint32_t hb) {
  uint32_t h, t, s;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(a1), "f"(a0));
  asm("add.rn.bf16x2 %0, %1, %2;" : "=r"(h) : "r"(h), "r"(hb));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(s) : "r"(h), "r"(t));
  return s;
}
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// Barrier over the 128 threads of warpgroup g (named barrier 1 + g); the
// second form returns the AND of every thread's p.
__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory");
}
__device__ __forceinline__ bool group_sync_and(int g, bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, d;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred d, %2, 128, q;\n\t"
      "selp.u32 %0, 1, 0, d;\n\t}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(p)), "r"(1 + g)
      : "memory");
  return r != 0;
}

// Copies a row-major [R][K] BF16 matrix into the K-major canonical layout.
__device__ void stage_kmajor(__nv_bfloat16* dst, const __nv_bfloat16* src, int R, int K) {
  const int chunks = R * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    const int r = c / (K / 8), k8 = c % (K / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(src + static_cast<int64_t>(r) * K + 8 * k8);
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(dst) + tc::kmajor_offset(r, 8 * k8, K)) = v;
  }
}

// As stage_kmajor, times `scale` (a power of two: exact in BF16, whose
// exponent range is FP32's) on the way.
__device__ void stage_kmajor_scaled(__nv_bfloat16* dst, const __nv_bfloat16* src, int R, int K,
                                    float scale) {
  const int chunks = R * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    const int r = c / (K / 8), k8 = c % (K / 8);
    uint4 v = *reinterpret_cast<const uint4*>(src + static_cast<int64_t>(r) * K + 8 * k8);
    __nv_bfloat162* p = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 f = __bfloat1622float2(p[i]);
      p[i] = __floats2bfloat162_rn(f.x * scale, f.y * scale);
    }
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(dst) + tc::kmajor_offset(r, 8 * k8, K)) = v;
  }
}

// ---- features of a (target leaf, source cell) pair -----------------------------
// R = c_T - c_S, d = |R|; m = |M0| + |M1| / h_S + |M2| / h_S^2 (Frobenius);
// f = [R/d, h_S/d, h_T/d, M0/m, M1/(m h_S), M2/(m h_S^2) (6 unique per row)];
// the network's outputs are u d^2/m, J d^3/m, H d^4/m (local expansion at c_T).
struct PairScale {
  float s2, s3, s4;  // m/d^2, m/d^3, m/d^4
};

// Geometry and moment normalisation of a pair (shared by the features, the
// analytic translation and the output scaling).
struct PairGeom {
  float Rx, Ry, Rz, id, hS, ih, m, im;
};

__device__ __forceinline__ PairGeom pair_geom(const float* rec, float cTx, float cTy, float cTz) {
  PairGeom g;
  g.Rx = cTx - rec[0];
  g.Ry = cTy - rec[1];
  g.Rz = cTz - rec[2];
  const float d2 = g.Rx * g.Rx + g.Ry * g.Ry + g.Rz * g.Rz;
  g.id = rsqrtf(d2);
  g.hS = rec[3];
  float n0 = 0.f, n1 = 0.f, n2 = 0.f;
  for (int q = 0; q < 3; ++q) n0 += rec[4 + q] * rec[4 + q];
  for (int q = 0; q < 9; ++q) n1 += rec[10 + q] * rec[10 + q];
  for (int m = 0; m < 3; ++m) {
    const float* Q = rec + 19 + 6 * m;
    n2 += Q[0] * Q[0] + Q[3] * Q[3] + Q[5] * Q[5] + 2.f * (Q[1] * Q[1] + Q[2] * Q[2] + Q[4] * Q[4]);
  }
  g.ih = 1.f / g.hS;
  g.m = sqrtf(n0) + sqrtf(n1) * g.ih + sqrtf(n2) * g.ih * g.ih + 1e-30f;
  g.im = 1.f / g.m;
  return g;
}

// A cell record into registers with ten 16-byte loads (records are 160 bytes
// apart from a 256-byte aligned base); read with constant indices only, so
// that the array stays in registers.
struct RecRegs {
  float v[kRecFloats];
};
__device__ __forceinline__ RecRegs load_record(const float* rec) {
  RecRegs r;
  const float4* r4 = reinterpret_cast<const float4*>(rec);
#pragma unroll
  for (int q = 0; q < kRecFloats / 4; ++q) {
    const float4 x = __ldg(r4 + q);
    r.v[4 * q] = x.x;
    r.v[4 * q + 1] = x.y;
    r.v[4 * q + 2] = x.z;
    r.v[4 * q + 3] = x.w;
  }
  return r;
}

__device__ __forceinline__ PairScale pair_scale(const PairGeom& g) {
  PairScale s;
  s.s2 = g.m * g.id * g.id;
  s.s3 = s.s2 * g.id;
  s.s4 = s.s3 * g.id;
  return s;
}

__device__ __forceinline__ PairScale pair_features(const float* rec, float cTx, float cTy,
                                                   float cTz, float hT, float* f) {
  const PairGeom g = pair_geom(rec, cTx, cTy, cTz);
  f[0] = g.Rx * g.id;
  f[1] = g.Ry * g.id;
  f[2] = g.Rz * g.id;
  f[3] = g.hS * g.id;
  f[4] = hT * g.id;
  for (int q = 0; q < 3; ++q) f[5 + q] = rec[4 + q] * g.im;
  for (int q = 0; q < 9; ++q) f[8 + q] = rec[10 + q] * g.im * g.ih;
  for (int q = 0; q < 18; ++q) f[17 + q] = rec[19 + q] * g.im * g.ih * g.ih;
  for (int q = NFEAT; q < IN; ++q) f[q] = 0.f;
  return pair_scale(g);
}

// Multipole to local, analytic (m2l_tensor, fvx_m2l_tensor.cuh): the local
// expansion at the target centre of the source cell's quadrupole expansion,
// in the network's normalised output units (unit distance along n = R/d).
// With C-scaled moments the vector potential is Psi_m = -(M0_m phi - M1_ma
// d_a phi + 1/2 M2_mab d_ab phi), phi = 1/|r|, and u_i = eps_ijm d_j Psi_m.
// Normalised moments of one pair, read from the 48 features...
struct FeatureMoments {
  const float* f;
  __device__ float n(int i) const { return f[i]; }
  __device__ float hs() const { return f[3]; }
  __device__ float c(int m) const { return f[5 + m]; }
  __device__ float m1(int q) const { return f[8 + q]; }    // M1 / (m h_S)
  __device__ float m2(int q) const { return f[17 + q]; }   // M2 / (m h_S^2)
};
// ... or straight from the cell record (same roundings as pair_features), so
// that the analytic kernel reads each moment when it is first used
struct RecordMoments {
  const float* rec;
  float nx, ny, nz, hs_d, im, ih;
  __device__ float n(int i) const { return i == 0 ? nx : (i == 1 ? ny : nz); }
  __device__ float hs() const { return hs_d; }
  __device__ float c(int m) const { return rec[4 + m] * im; }
  __device__ float m1(int q) const { return rec[10 + q] * im * ih; }
  __device__ float m2(int q) const { return rec[19 + q] * im * ih * ih; }
};

__device__ __forceinline__ void m2l_quadrupole(const float* f, float* out) {
  m2l_tensor(FeatureMoments{f}, out);
}

__device__ __forceinline__ float3 leaf_center(uint32_t key, float h) {
  auto compact = [](uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0x030000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
  };
  return make_float3((static_cast<float>(compact(key)) + 0.5f) * h,
                     (static_cast<float>(compact(key >> 1)) + 0.5f) * h,
                     (static_cast<float>(compact(key >> 2)) + 0.5f) * h);
}

// ---- forward policies --------------------------------------------------------------
struct RowsIO {
  const __nv_bfloat16* X;
  float* Y;
  float* z_store;
  __nv_bfloat16* h_store;
};

// The far field's rows: list l0's pairs, then list l1's (the leaves' own
// pairs and the pairs shared through parents of leaves, in one launch).
struct FarIO {
  FarPairs l0, l1;
  const float* rec;  // cell records
  FarJudge judge;    // per-class actions of the FP64 judge (none by default)
};

// row `row` of a 128 x H accumulator -> bias + SiLU -> BF16 activation tile
__device__ void epilogue_hidden(uint32_t tmem, int row, const float* bias, __nv_bfloat16* act,
                                float* z_out, __nv_bfloat16* h_out) {
  const uint32_t lane_base = static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16;
  char* base = reinterpret_cast<char*>(act);
  for (int c0 = 0; c0 < H; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tmem + lane_base + c0, v);
    __align__(16) __nv_bfloat162 b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float z0 = v[2 * i] + bias[c0 + 2 * i], z1 = v[2 * i + 1] + bias[c0 + 2 * i + 1];
      if (z_out) {
        z_out[c0 + 2 * i] = z0;
        z_out[c0 + 2 * i + 1] = z1;
      }
      b[i] = __floats2bfloat162_rn(silu(z0), silu(z1));
    }
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0, H)) =
        *reinterpret_cast<uint4*>(&b[0]);
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0 + 8, H)) =
        *reinterpret_cast<uint4*>(&b[4]);
    if (h_out) {
      *reinterpret_cast<uint4*>(h_out + c0) = *reinterpret_cast<uint4*>(&b[0]);
      *reinterpret_cast<uint4*>(h_out + c0 + 8) = *reinterpret_cast<uint4*>(&b[4]);
    }
  }
}

// Inference form of epilogue_hidden: packed BF16 arithmetic.  The layer's
// weights are halved (acc = z/2 - b/2) and hbias holds its halved biases as
// packed BF16 pairs, so each pair of columns is one silu_bf16x2.
// The TMEM loads are double-buffered: the next 16 columns load while the
// current ones are processed.
__device__ __forceinline__ void silu_chunk_bf16(const uint32_t (&r)[16], const uint32_t* hbias,
                                                char* base, int row, int c0) {
  __align__(16) uint32_t b[8];
  const uint4 h0 = *reinterpret_cast<const uint4*>(hbias + c0 / 2);
  const uint4 h1 = *reinterpret_cast<const uint4*>(hbias + c0 / 2 + 4);
  const uint32_t hb[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
  for (int i = 0; i < 8; ++i)
    b[i] = silu_bf16x2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]), hb[i]);
  *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0, H)) =
      *reinterpret_cast<uint4*>(&b[0]);
  *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0 + 8, H)) =
      *reinterpret_cast<uint4*>(&b[4]);
}
__device__ void epilogue_hidden_infer(uint32_t tmem, int row, const uint32_t* hbias, void* act) {
  const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16);
  char* base = reinterpret_cast<char*>(act);
  uint32_t ra[16], rb[16];
  tc::tmem_ld16_issue(taddr, ra);
  tc::tmem_ld_wait(ra);
#pragma unroll
  for (int c0 = 0; c0 < H; c0 += 32) {
    tc::tmem_ld16_issue(taddr + c0 + 16, rb);
    silu_chunk_bf16(ra, hbias, base, row, c0);
    tc::tmem_ld_wait(rb);
    if (c0 + 32 < H) tc::tmem_ld16_issue(taddr + c0 + 32, ra);
    silu_chunk_bf16(rb, hbias, base, row, c0 + 16);
    if (c0 + 32 < H) tc::tmem_ld_wait(ra);
  }
}

__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& ph) {
  const bool ok = mbar_wait(bar, ph);
  ph ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// Group-wide wait for the group's MMA: the group's first warp polls the
// mbarrier while the other three wait at the group barrier (no instructions
// issued), which then releases everyone with the AND of the outcome.
__device__ __forceinline__ bool group_wait_mma(int g, uint64_t* bar, uint32_t& ph) {
  bool w = true;
  if ((threadIdx.x & 127) < 32) w = mbar_wait(bar, ph);
  ph ^= 1u;
  tc::fence_before_sync();
  const bool ok = group_sync_and(g, w);
  tc::fence_after_sync();
  return ok;
}

// As group_wait_mma, with the first thread's `issued` (false when it did not
// issue the MMA): the group's warp 0 polls only for an issued MMA, and every
// thread learns the AND.
__device__ __forceinline__ bool group_wait_mma_if(int g, uint64_t* bar, uint32_t& ph, bool issued) {
  bool w = issued;
  if ((threadIdx.x & 127) < 32) {
    const bool any = __shfl_sync(0xffffffffu, issued ? 1 : 0, 0) != 0;
    if (any) w = w && mbar_wait(bar, ph);
    else w = false;
  }
  ph ^= 1u;
  tc::fence_before_sync();
  const bool ok = group_sync_and(g, w);
  tc::fence_after_sync();
  return ok;
}

// Group-local fence + barrier before an MMA: the group's shared-memory writes
// made visible to the tensor core (async proxy) and its TMEM reads done.
__device__ __forceinline__ void group_handoff(int g) {
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  group_sync(g);
  tc::fence_after_sync();
}

// The network on rows of inputs: Y[rows][32] from X[rows][48].  INFER: the
// inference form -- BF16 operands, hidden weights and biases halved while
// staged, the packed BF16 SiLU of epilogue_hidden_infer (the far-field
// kernel's arithmetic); the training forward (with stored pre-activations and
// activations) keeps the FP32 SiLU of epilogue_hidden.
template <bool INFER>
__global__ void __launch_bounds__(kGroups * 128, 1) mlp_fwd_kernel(RowsIO A, int rows,
                                                           const __nv_bfloat16* __restrict__ W,
                                                           const float* __restrict__ bias) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  FwdSmem& S = *reinterpret_cast<FwdSmem*>(smem_raw);
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, 128 * kGroups);
  if (threadIdx.x == 0) {
    for (int g = 0; g < kGroups; ++g) mbar_init(&S.bar[g], 1);
    fence_mbar_init();
  }
  if constexpr (INFER) {
    // hidden layers halved: their accumulators are z/2, the tanh argument
    stage_kmajor_scaled(S.w1, W + W1o, H, IN, 0.5f);
    stage_kmajor_scaled(S.w2, W + W2o, H, H, 0.5f);
    stage_kmajor_scaled(S.w3, W + W3o, H, H, 0.5f);
    stage_kmajor(S.w4, W + W4o, OUT, H);
    for (int i = threadIdx.x; i < 3 * H / 2; i += blockDim.x) {
      const __nv_bfloat162 hb = __floats2bfloat162_rn(0.5f * bias[2 * i], 0.5f * bias[2 * i + 1]);
      S.hbias[i] = *reinterpret_cast<const uint32_t*>(&hb);
    }
  } else {
    stage_kmajor(S.w1, W + W1o, H, IN);
    stage_kmajor(S.w2, W + W2o, H, H);
    stage_kmajor(S.w3, W + W3o, H, H);
    stage_kmajor(S.w4, W + W4o, OUT, H);
  }
  for (int i = threadIdx.x; i < BN; i += blockDim.x) S.bias[i] = bias[i];
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const int grp = threadIdx.x >> 7;   // warpgroup
  const int lt = threadIdx.x & 127;   // row of the group's tile
  const uint32_t tmem = S.tmem + static_cast<uint32_t>(128 * grp);
  const uint32_t lane_base = static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16;
  __nv_bfloat16* act = S.act[grp];
  uint64_t* bar = &S.bar[grp];
  uint32_t ph = 0;
  bool ok = true;
  const int ntiles = (rows + 127) / 128;
  const int tile_step = kGroups * gridDim.x;
  for (int tile = kGroups * blockIdx.x + grp; tile < ntiles && ok; tile += tile_step) {
    const int row = tile * 128 + lt;
    const bool act_row = row < rows;
    // input tile (K = 48)
    {
      char* base = reinterpret_cast<char*>(act);
      for (int k8 = 0; k8 < IN / 8; ++k8) {
        uint4 v = make_uint4(0, 0, 0, 0);
        if (act_row)
          v = *reinterpret_cast<const uint4*>(A.X + static_cast<int64_t>(row) * IN + 8 * k8);
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(lt, 8 * k8, IN)) = v;
      }
    }
    for (int l = 0; l < 3; ++l) {
      group_handoff(grp);
      if (lt == 0)
        tc::gemm_issue(tmem, act, l == 0 ? S.w1 : (l == 1 ? S.w2 : S.w3), l == 0 ? IN : H,
                       tc::idesc_bf16(128, H), false, bar, 0);
      if (!group_wait_mma(grp, bar, ph)) {
        ok = false;
        break;
      }
      float* zo = nullptr;
      __nv_bfloat16* ho = nullptr;
      if (A.z_store && act_row) zo = A.z_store + (static_cast<int64_t>(l) * rows + row) * H;
      if (A.h_store && act_row) ho = A.h_store + (static_cast<int64_t>(l) * rows + row) * H;
      if constexpr (INFER)
        epilogue_hidden_infer(tmem, lt, S.hbias + l * H / 2, act);
      else
        epilogue_hidden(tmem, lt, S.bias + l * H, act, zo, ho);
    }
    if (!ok) break;
    group_handoff(grp);
    if (lt == 0)
      tc::gemm_issue(tmem, act, S.w4, H, tc::idesc_bf16(128, OUT), false, bar, 0);
    if (!group_wait_mma(grp, bar, ph)) {
      ok = false;
      break;
    }
    for (int c0 = 0; c0 < OUT; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + c0, v);
      if (!act_row) continue;
      float4* y = reinterpret_cast<float4*>(A.Y + static_cast<int64_t>(row) * OUT + c0);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        y[q] = make_float4(v[4 * q] + S.bias[B4o + c0 + 4 * q],
                           v[4 * q + 1] + S.bias[B4o + c0 + 4 * q + 1],
                           v[4 * q + 2] + S.bias[B4o + c0 + 4 * q + 2],
                           v[4 * q + 3] + S.bias[B4o + c0 + 4 * q + 3]);
    }
    // no barrier here: the next tile's first handoff orders this tile's TMEM
    // reads before the MMA that overwrites them
  }
  if (!ok && lt == 0) flag_status(kStatusTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(S.tmem, 128 * kGroups);
}

// ---- the learned far field: consumer and producer warpgroups ----------------------------
// Warpgroups 0..3 (consumers) chain the network's layers through their quarter
// of the tensor memory as in mlp_fwd_kernel: MMA -> epilogue -> next MMA.
// Warpgroups 4 and 5 (producers, two consumer groups each) form every tile's
// inputs (the pair features into the group's activation tile, the output
// scales and targets into aux) and reduce every tile's outputs into the
// leaves' expansions, so that neither stage sits on a consumer's chain.  A
// producer's warp q serves rows 32q..32q+31 of every tile (the TMEM lanes warp
// q may read) and loads the pair indices and cell records one step ahead.
// Per group g:
//   feat_bar[g] (4 arrivals, one per producer warp) completes once per tile
//     when its inputs are written and the previous tile's output accumulator
//     has been read (so the activation tile and TMEM are free);
//   out_bar[g] (tcgen05.commit of the tile's last MMA) completes when the
//     tile's outputs are in TMEM and the activation tile has been read.
// A producer visits its groups' tiles in increasing order: its step j is tile
// j / 2 of its group j % 2.  Registers move from the consumers to the
// producers by setmaxnreg; the host checks that the launch holds them.
constexpr int kProducers = 2;
constexpr int kGroupsPerProducer = kGroups / kProducers;
static_assert(kGroups % kProducers == 0, "each producer serves the same number of groups");
constexpr int kFarThreads = (kGroups + kProducers) * 128;
constexpr int kConsumerRegs = 56, kProducerRegs = 128;
constexpr int kFarRegsNeeded = (kGroups * kConsumerRegs + kProducers * kProducerRegs) * 128;

struct FarSmem {
  __nv_bfloat16 w1[H * IN];
  __nv_bfloat16 w2[H * H];
  __nv_bfloat16 w3[H * H];
  __nv_bfloat16 w4[OUT * H];
  __nv_bfloat16 act[kGroups][128 * H];
  // per row: the output scales m/d^2, m/d^3, m/d^4 (zero for a row without a
  // pair or whose class dropped the network) and the target id
  float aux[kGroups][128][4];
  float bias4[OUT];
  uint32_t hbias[3 * H / 2];  // half the hidden layers' biases, packed BF16 pairs
  uint64_t bar[kGroups], feat_bar[kGroups], out_bar[kGroups];
  uint32_t tmem;
};

// The producer's view of a pair ahead of its use: the index level (leaf, cell,
// list), then the record level (the leaf key and the cell record as well).
struct PairIndex {
  int leaf = 0, cell = 0, li = 0;
  bool act = false;
};
struct PairFetch {
  PairIndex i;
  uint32_t key = 0;
  RecRegs rec;
};

__global__ void __launch_bounds__(kFarThreads, 1) farfield_kernel(FarIO F, int rows,
                                                                  const __nv_bfloat16* __restrict__ W,
                                                                  const float* __restrict__ bias) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  FarSmem& S = *reinterpret_cast<FarSmem*>(smem_raw);
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, 128 * kGroups);
  if (threadIdx.x == 0) {
    for (int g = 0; g < kGroups; ++g) {
      mbar_init(&S.bar[g], 1);
      mbar_init(&S.feat_bar[g], 4);
      mbar_init(&S.out_bar[g], 1);
    }
    fence_mbar_init();
  }
  // hidden layers halved: their accumulators are z/2, the tanh argument
  stage_kmajor_scaled(S.w1, W + W1o, H, IN, 0.5f);
  stage_kmajor_scaled(S.w2, W + W2o, H, H, 0.5f);
  stage_kmajor_scaled(S.w3, W + W3o, H, H, 0.5f);
  stage_kmajor(S.w4, W + W4o, OUT, H);
  for (int i = threadIdx.x; i < 3 * H / 2; i += blockDim.x) {
    const __nv_bfloat162 hb = __floats2bfloat162_rn(0.5f * bias[2 * i], 0.5f * bias[2 * i + 1]);
    S.hbias[i] = *reinterpret_cast<const uint32_t*>(&hb);
  }
  for (int i = threadIdx.x; i < OUT; i += blockDim.x) S.bias4[i] = bias[B4o + i];
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const int grp = threadIdx.x >> 7;
  const int lt = threadIdx.x & 127;
  const int ntiles = (rows + 127) / 128;
  const int tile_step = kGroups * gridDim.x;
  bool ok = true;
  if (grp < kGroups) {
    // ---- consumer: the four layers of the group's tiles ----
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kConsumerRegs));
    const uint32_t tmem = S.tmem + static_cast<uint32_t>(128 * grp);
    __nv_bfloat16* act = S.act[grp];
    uint64_t* bar = &S.bar[grp];
    uint32_t ph = 0, fph = 0;
    for (int tile = kGroups * blockIdx.x + grp; tile < ntiles; tile += tile_step) {
      // the tile's inputs written and the previous tile's outputs read: only
      // the issuing thread waits; the group learns the outcome with the first
      // MMA's wait
      bool fed = true;
      if (lt == 0) {
        fed = mbar_wait(&S.feat_bar[grp], fph);
        tc::fence_after_sync();
      }
      fph ^= 1u;
      for (int l = 0; l < 3; ++l) {
        if (l > 0) group_handoff(grp);
        if (lt == 0 && fed)
          tc::gemm_issue(tmem, act, l == 0 ? S.w1 : (l == 1 ? S.w2 : S.w3), l == 0 ? IN : H,
                         tc::idesc_bf16(128, H), false, bar, 0);
        if (!group_wait_mma_if(grp, bar, ph, l > 0 || fed)) {
          ok = false;
          break;
        }
        epilogue_hidden_infer(tmem, lt, S.hbias + l * H / 2, act);
      }
      if (!ok) break;
      group_handoff(grp);
      if (lt == 0)
        tc::gemm_issue(tmem, act, S.w4, H, tc::idesc_bf16(128, OUT), false, &S.out_bar[grp], 0);
    }
  } else {
    // ---- producer: inputs and outputs of its groups' tiles, rows 32q..32q+31 ----
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kProducerRegs));
    const int g0 = (grp - kGroups) * kGroupsPerProducer;  // the first group served
    const int q = (threadIdx.x >> 5) & 3;
    const int lane = threadIdx.x & 31;
    const int r = 32 * q + lane;  // the row of every tile this thread serves
    const uint32_t lane_base = static_cast<uint32_t>(32 * q) << 16;
    auto tile_of = [&](int j) {
      return kGroups * blockIdx.x + g0 + j % kGroupsPerProducer + j / kGroupsPerProducer * tile_step;
    };
    auto fetch_index = [&](PairIndex& I, int j) {
      const int row = tile_of(j) * 128 + r;
      I.act = tile_of(j) < ntiles && row < rows;
      if (I.act) {
        I.li = row >= F.l0.n ? 1 : 0;
        const int rr = I.li ? row - F.l0.n : row;
        I.leaf = (I.li ? F.l1.pair_tgt : F.l0.pair_tgt)[rr];
        I.cell = (I.li ? F.l1.pair_cell : F.l0.pair_cell)[rr];
      }
    };
    auto fetch_record = [&](PairFetch& P, const PairIndex& I) {
      P.i = I;
      if (I.act) {
        P.key = (I.li ? F.l1.tgt_key : F.l0.tgt_key)[I.leaf];
        P.rec = load_record(F.rec + static_cast<int64_t>(I.cell) * kRecFloats);
      }
    };
    // the features of a fetched pair, packed BF16 pairs, and its aux row
    uint32_t fp[IN / 2];
    float faux[4];
    auto features = [&](const PairFetch& P) {
      float f[IN];
      faux[0] = faux[1] = faux[2] = 0.f;
      faux[3] = __int_as_float(-1 - r);  // a row without a pair: an id of its own
      if (P.i.act) {
        const float th = P.i.li ? F.l1.h : F.l0.h;
        const float3 cT = leaf_center(P.key, th);
        bool keep = true;
        if (F.judge.act != nullptr) {
          // the residual only for the classes whose network the judge kept
          const float dx = cT.x - P.rec.v[0], dy = cT.y - P.rec.v[1], dz = cT.z - P.rec.v[2];
          keep = F.judge.act[judge_class(P.i.li, th, P.rec.v[3], dx * dx + dy * dy + dz * dz,
                                         F.judge.inv_theta2)] == 0;
        }
        const PairScale sc = pair_features(P.rec.v, cT.x, cT.y, cT.z, th, f);
        if (keep) {
          faux[0] = sc.s2;
          faux[1] = sc.s3;
          faux[2] = sc.s4;
        }
        faux[3] = __int_as_float(P.i.leaf | (P.i.li << 30));
      } else {
#pragma unroll
        for (int k = 0; k < IN; ++k) f[k] = 0.f;
      }
#pragma unroll
      for (int k = 0; k < IN / 2; ++k) {
        const __nv_bfloat162 b = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        fp[k] = *reinterpret_cast<const uint32_t*>(&b);
      }
    };
    auto write_inputs = [&](int g) {
      char* base = reinterpret_cast<char*>(S.act[g]);
#pragma unroll
      for (int k8 = 0; k8 < IN / 8; ++k8)
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(r, 8 * k8, IN)) =
            make_uint4(fp[4 * k8], fp[4 * k8 + 1], fp[4 * k8 + 2], fp[4 * k8 + 3]);
      *reinterpret_cast<float4*>(S.aux[g][r]) = make_float4(faux[0], faux[1], faux[2], faux[3]);
    };
    // inputs of the first tile of each group served: nothing to wait for
    PairFetch cur;
    PairIndex nxt;
    fetch_index(nxt, 0);
    for (int j = 0; j < kGroupsPerProducer; ++j) {
      fetch_record(cur, nxt);
      fetch_index(nxt, j + 1);
      if (tile_of(j) < ntiles) {
        features(cur);
        write_inputs(g0 + j);
        tc::fence_smem_to_async();
        __syncwarp();
        if (lane == 0)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                           smem_u32(&S.feat_bar[g0 + j]))
                       : "memory");
      }
    }
    // the record of step kGroupsPerProducer's tile, then the next step's index
    fetch_record(cur, nxt);
    fetch_index(nxt, kGroupsPerProducer + 1);
    uint32_t oph = 0u;  // bit g: the parity of group g's next out_bar phase
    for (int j = 0; tile_of(j) < ntiles && ok; ++j) {
      const int g = g0 + j % kGroupsPerProducer;
      // the inputs of this group's next tile (step j + kGroupsPerProducer), from cur
      const bool has_next = tile_of(j + kGroupsPerProducer) < ntiles;
      if (has_next) features(cur);
      // one step ahead: the next step's record, the one after's index
      fetch_record(cur, nxt);
      fetch_index(nxt, j + kGroupsPerProducer + 2);
      // tile j's outputs
      bool w = true;
      if (lane == 0) w = mbar_wait(&S.out_bar[g], (oph >> g) & 1u);
      oph ^= 1u << g;
      if (!__shfl_sync(0xffffffffu, w ? 1 : 0, 0)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      float x[OUT];
      {
        uint32_t v0[16], v1[16];
        tc::tmem_ld16_issue(S.tmem + static_cast<uint32_t>(128 * g) + lane_base, v0);
        tc::tmem_ld16_issue(S.tmem + static_cast<uint32_t>(128 * g) + lane_base + 16, v1);
        tc::tmem_ld_wait(v0);
        tc::tmem_ld_wait(v1);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          x[i] = __uint_as_float(v0[i]);
          x[16 + i] = __uint_as_float(v1[i]);
        }
      }
      const float4 ax = *reinterpret_cast<const float4*>(S.aux[g][r]);
      if (has_next) {
        write_inputs(g);
        tc::fence_smem_to_async();
      }
      tc::fence_before_sync();
      __syncwarp();
      if (has_next && lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&S.feat_bar[g]))
                     : "memory");
      // the learned residual of this row, back to physical units (the analytic
      // translation is added by its own kernel)
#pragma unroll
      for (int c = 0; c < OUT; ++c) {
        const float sc = c < 3 ? ax.x : (c < 12 ? ax.y : ax.z);
        x[c] = c < NOUT ? (x[c] + S.bias4[c]) * sc : 0.f;
      }
      const int my = __float_as_int(ax.w);  // unique across the two lists
      const bool act_row = my >= 0;
      float* L = act_row ? ((my >> 30) ? F.l1.local : F.l0.local) +
                               static_cast<int64_t>(my & ((1 << 30) - 1)) * OUT
                         : nullptr;
      if (__all_sync(0xffffffffu, my == __shfl_sync(0xffffffffu, my, 0))) {
        // one target for the whole warp: reduce-scatter by recursive halving,
        // 31 shuffles for the 32 columns; lane c ends with column c's sum
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
          const bool upper = (lane & off) != 0;
#pragma unroll
          for (int i = 0; i < off; ++i) {
            const float send = upper ? x[i] : x[i + off];
            const float kept = upper ? x[i + off] : x[i];
            x[i] = kept + __shfl_xor_sync(0xffffffffu, send, off);
          }
        }
        if (lane < NOUT) atomicAdd(L + lane, x[0]);
      } else {
        // runs of equal targets inside the warp: segmented sums to each run's
        // first lane, which adds them to the target's expansion
        const int up = __shfl_up_sync(0xffffffffu, my, 1);
        const bool head = act_row && (lane == 0 || up != my);
#pragma unroll
        for (int c = 0; c < NOUT; ++c) {
          float y = x[c];
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const float o = __shfl_down_sync(0xffffffffu, y, off);
            const int ol = __shfl_down_sync(0xffffffffu, my, off);
            if (lane + off < 32 && ol == my) y += o;
          }
          if (head) atomicAdd(L + c, y);
        }
      }
    }
  }
  if (!ok && (threadIdx.x & 31) == 0) flag_status(kStatusTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(S.tmem, 128 * kGroups);
}

// ---- training data: features + exact local expansions of sampled pairs ----------
// FP64 direct sums over the source cell's particles of the singular
// Biot-Savart field and its first two derivatives at c_T.  blockIdx.x = the
// pair, blockIdx.y = one of gridDim.y slices of the cell's particles (so that
// a few very large cells still spread over the GPU); threads stride over the
// slice, warps then the CTA reduce in a fixed order, and each slice writes its
// own partial sums (no atomics: the result does not depend on timing).
// One slice [s0, s0 + n) of a source cell's particles summed at cT into
// acc[30]: the singular field u, its gradient and its second derivatives, in
// FP64 (positions from the FP32 records relative to each particle's leaf
// centre, the centre differences exact).
__device__ __forceinline__ void exact_expansion_slice(float3 cT, int s0, int n,
                                                      const uint32_t* __restrict__ leaf_key,
                                                      const float4* __restrict__ sp,
                                                      const float4* __restrict__ sa,
                                                      const int* __restrict__ leaf_of_particle,
                                                      float h, double (&acc)[NOUT]) {
#pragma unroll
  for (int q = 0; q < NOUT; ++q) acc[q] = 0.0;
  for (int i = s0 + static_cast<int>(threadIdx.x); i < s0 + n; i += blockDim.x) {
    const float3 cs = leaf_center(leaf_key[leaf_of_particle[i] - 1], h);
    const float4 p = sp[i];
    const float4 a = sa[i];
    const double d[3] = {static_cast<double>(cT.x - cs.x) - p.x,
                         static_cast<double>(cT.y - cs.y) - p.y,
                         static_cast<double>(cT.z - cs.z) - p.z};
    const double al[3] = {a.x, a.y, a.z};
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double ir = rsqrt(r2), ir2 = ir * ir;
    const double f = ir2 * ir, fpr = -3.0 * f * ir2, fpp = 15.0 * f * ir2 * ir2;
    const double c[3] = {d[1] * al[2] - d[2] * al[1], d[2] * al[0] - d[0] * al[2],
                         d[0] * al[1] - d[1] * al[0]};
    // eps_inm a_m as a matrix E[i][n]
    const double E[3][3] = {{0.0, al[2], -al[1]}, {-al[2], 0.0, al[0]}, {al[1], -al[0], 0.0}};
    for (int i2 = 0; i2 < 3; ++i2) {
      acc[i2] += f * c[i2];
      for (int n2 = 0; n2 < 3; ++n2) acc[3 + 3 * i2 + n2] += fpr * d[n2] * c[i2] + f * E[i2][n2];
      int u = 0;
      for (int k = 0; k < 3; ++k)
        for (int m = k; m < 3; ++m, ++u) {
          const double v = (fpp * d[k] * d[m] + (k == m ? fpr : 0.0)) * c[i2] +
                           fpr * d[m] * E[i2][k] + fpr * d[k] * E[i2][m];
          acc[12 + 6 * i2 + u] += v;
        }
    }
  }
}

// The CTA's sums of acc, warps then the CTA in a fixed order, to `out` (30).
__device__ __forceinline__ void reduce_expansion(double (&acc)[NOUT], double* out) {
  __shared__ double red[kTargetsThreads / 32][NOUT];
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < NOUT; ++q)
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  if (lane == 0)
    for (int q = 0; q < NOUT; ++q) red[threadIdx.x >> 5][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < NOUT) {
    double v = 0.0;
    for (int w = 0; w < kTargetsThreads / 32; ++w) v += red[w][threadIdx.x];
    out[threadIdx.x] = v;
  }
}

// FP64 direct sums over the source cell's particles of the singular
// Biot-Savart field and its first two derivatives at c_T.  blockIdx.x = the
// pair, blockIdx.y = one of gridDim.y slices of the cell's particles (so that
// a few very large cells still spread over the GPU); threads stride over the
// slice, warps then the CTA reduce in a fixed order, and each slice writes its
// own partial sums (no atomics: the result does not depend on timing).
__global__ void pair_sums_kernel(int npairs, int stride, const int* __restrict__ pair_leaf,
                                 const int* __restrict__ pair_cell,
                                 const uint32_t* __restrict__ tgt_key, float h_tgt,
                                 const uint32_t* __restrict__ leaf_key,
                                 const int* __restrict__ cell_start,
                                 const int* __restrict__ cell_count,
                                 const float4* __restrict__ sp, const float4* __restrict__ sa,
                                 const int* __restrict__ leaf_of_particle, float h,
                                 double* __restrict__ partial) {
  const int pr = blockIdx.x;
  if (pr >= npairs) return;
  const int t = pair_leaf[static_cast<int64_t>(pr) * stride],
            g = pair_cell[static_cast<int64_t>(pr) * stride];
  const float3 cT = leaf_center(tgt_key[t], h_tgt);
  const int c0 = cell_start[g], cn = cell_count[g];
  const int per = (cn + gridDim.y - 1) / gridDim.y;
  const int s0 = c0 + static_cast<int>(blockIdx.y) * per;
  const int n = max(0, min(per, c0 + cn - s0));
  double acc[NOUT];
  exact_expansion_slice(cT, s0, n, leaf_key, sp, sa, leaf_of_particle, h, acc);
  reduce_expansion(acc, partial + (static_cast<int64_t>(pr) * gridDim.y + blockIdx.y) * NOUT);
}

// The same sums for the FP64 judge's samples, balanced over the GPU whatever
// the cells' sizes: each sample's cell is cut into chunks of kJudgeChunk
// particles, item offsets per slot come from judge_chunks_kernel, and
// resident CTAs stride over the items (four particles per thread), adding each
// chunk's 30 sums into the slot's with FP64 atomics (the order of those
// additions varies from run to run in the last bits).  Slots: list 0's
// samples, then list 1's, cap each; slots past a list's count take no items.
__global__ void judge_chunks_kernel(JudgeSampleView S, const int* __restrict__ cell_count,
                                    int* __restrict__ off) {
  __shared__ int sc[1024];
  __shared__ int carry;
  const int n = 2 * S.cap;
  if (threadIdx.x == 0) {
    carry = 0;
    off[0] = 0;
  }
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    int c = 0;
    if (i < n) {
      const int li = i >= S.cap ? 1 : 0;
      const int q = i - li * S.cap;
      if (q < S.cnt[li]) c = (cell_count[S.cell[li][q]] + kJudgeChunk - 1) / kJudgeChunk;
    }
    __syncthreads();
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int v = threadIdx.x >= static_cast<unsigned>(o) ? sc[threadIdx.x - o] : 0;
      __syncthreads();
      sc[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n) off[i + 1] = carry + sc[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 1023) carry += sc[1023];
  }
}

__global__ void __launch_bounds__(kTargetsThreads) judge_sums_kernel(
    JudgeSampleView S, const int* __restrict__ off, const uint32_t* __restrict__ leaf_key,
    const int* __restrict__ cell_start, const int* __restrict__ cell_count,
    const float4* __restrict__ sp, const float4* __restrict__ sa,
    const int* __restrict__ leaf_of_particle, float h, double* __restrict__ sums) {
  __shared__ double s_out[NOUT];
  const int n = 2 * S.cap;
  const int total = off[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int lo = 0, hi = n;  // the slot: off[slot] <= item < off[slot + 1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (off[mid] <= item) lo = mid; else hi = mid;
    }
    const int slot = lo;
    const int li = slot >= S.cap ? 1 : 0;
    const int q = slot - li * S.cap;
    const float3 cT = leaf_center(S.key[li][q], S.h[li]);
    const int g = S.cell[li][q];
    const int c0 = cell_start[g], cn = cell_count[g];
    const int s0 = c0 + (item - off[slot]) * kJudgeChunk;
    const int m = min(kJudgeChunk, c0 + cn - s0);
    double acc[NOUT];
    exact_expansion_slice(cT, s0, m, leaf_key, sp, sa, leaf_of_particle, h, acc);
    reduce_expansion(acc, s_out);
    __syncthreads();
    if (threadIdx.x < NOUT) atomicAdd(sums + static_cast<int64_t>(slot) * NOUT + threadIdx.x,
                                      s_out[threadIdx.x]);
    __syncthreads();
  }
}

// Per pair: the slices' sums in order, the features (BF16), the output scales,
// the analytic translation and the normalised exact targets.
__global__ void pair_targets_kernel(int npairs, int stride, int slices,
                                    const int* __restrict__ pair_leaf,
                                    const int* __restrict__ pair_cell,
                                    const uint32_t* __restrict__ tgt_key, float h_tgt,
                                    const float* __restrict__ rec,
                                    const double* __restrict__ partial,
                                    __nv_bfloat16* __restrict__ X, float* __restrict__ T,
                                    float* __restrict__ Aout, float* __restrict__ scale) {
  const int pr = blockIdx.x * blockDim.x + threadIdx.x;
  if (pr >= npairs) return;
  const int t = pair_leaf[static_cast<int64_t>(pr) * stride],
            g = pair_cell[static_cast<int64_t>(pr) * stride];
  const float3 cT = leaf_center(tgt_key[t], h_tgt);
  float f[IN];
  const PairScale sc =
      pair_features(rec + static_cast<int64_t>(g) * kRecFloats, cT.x, cT.y, cT.z, h_tgt, f);
  for (int q = 0; q < IN; ++q) X[static_cast<int64_t>(pr) * IN + q] = __float2bfloat16(f[q]);
  if (scale) {
    scale[static_cast<int64_t>(pr) * 4 + 0] = sc.s2;
    scale[static_cast<int64_t>(pr) * 4 + 1] = sc.s3;
    scale[static_cast<int64_t>(pr) * 4 + 2] = sc.s4;
    scale[static_cast<int64_t>(pr) * 4 + 3] = f[4];  // h_T / d
  }
  if (Aout) {
    float a[NOUT];
    m2l_quadrupole(f, a);
    for (int q = 0; q < OUT; ++q) Aout[static_cast<int64_t>(pr) * OUT + q] = q < NOUT ? a[q] : 0.f;
  }
  const double* ps = partial + static_cast<int64_t>(pr) * slices * NOUT;
  for (int q = 0; q < OUT; ++q) {
    float v = 0.f;
    if (q < NOUT) {
      double acc = 0.0;
      for (int k = 0; k < slices; ++k) acc += ps[k * NOUT + q];
      const double s = q < 3 ? sc.s2 : (q < 12 ? sc.s3 : sc.s4);
      v = static_cast<float>(acc / s);
    }
    T[static_cast<int64_t>(pr) * OUT + q] = v;
  }
}

// ---- analytic far field of the local-expansion path (no network) ---------------------
// One thread per (leaf, cell) pair: features -> M2L -> physical units -> sum
// over the warp's runs of equal leaves -> atomics into the leaf's expansion.
// Resident CTAs (two per SM at 128 registers) stride over blocks of pairs.
constexpr int kM2lThreads = 256;

__global__ void __launch_bounds__(kM2lThreads) m2l_pairs_kernel(FarIO F) {
  const int lane = threadIdx.x & 31;
  const int npairs = F.l0.n + F.l1.n;
  for (int base = blockIdx.x * kM2lThreads; base < npairs; base += gridDim.x * kM2lThreads) {
    const int row = base + threadIdx.x;
    const bool act_row = row < npairs;
    float a[NOUT];
#pragma unroll
    for (int q = 0; q < NOUT; ++q) a[q] = 0.f;
    PairScale sc{0.f, 0.f, 0.f};
    int leaf = 0, li = 0;
    float* L = nullptr;
    bool queue = false;
    int cell = 0;
    if (act_row) {
      li = row >= F.l0.n ? 1 : 0;
      const int rr_ = li ? row - F.l0.n : row;
      const FarPairs& fl = li ? F.l1 : F.l0;
      leaf = fl.pair_tgt[rr_];
      cell = fl.pair_cell[rr_];
      L = fl.local + static_cast<int64_t>(leaf) * OUT;
      const float3 cT = leaf_center(fl.tgt_key[leaf], fl.h);
      const RecRegs rr = load_record(F.rec + static_cast<int64_t>(cell) * kRecFloats);
      if (F.judge.act != nullptr) {
        // a class the judge sent to the FP64 direct sum: no expansion, queued
        const float dx = cT.x - rr.v[0], dy = cT.y - rr.v[1], dz = cT.z - rr.v[2];
        queue = F.judge.act[judge_class(li, fl.h, rr.v[3], dx * dx + dy * dy + dz * dz,
                                        F.judge.inv_theta2)] == 2;
      }
      if (!queue) {
        const PairGeom g = pair_geom(rr.v, cT.x, cT.y, cT.z);
        const RecordMoments src{rr.v, g.Rx * g.id, g.Ry * g.id, g.Rz * g.id, g.hS * g.id, g.im,
                                g.ih};
        m2l_tensor(src, a);
        sc = pair_scale(g);
      }
    }
    const unsigned qm = __ballot_sync(0xffffffffu, queue);
    if (qm) {
      // one atomic per warp for its queued pairs
      int base_q = 0;
      if (lane == 0) base_q = atomicAdd(F.judge.nfb, __popc(qm));
      base_q = __shfl_sync(0xffffffffu, base_q, 0);
      if (queue) {
        const int q = base_q + __popc(qm & ((1u << lane) - 1u));
        if (q < F.judge.fb_cap)
          F.judge.fb[q] = make_int2(leaf | (li << 30), cell);
        else
          flag_status(kStatusCapacity);
      }
    }
    const int my = act_row ? (leaf | (li << 30)) : -1 - lane;  // unique across the lists
    float x[32];
#pragma unroll
    for (int c = 0; c < 32; ++c)
      x[c] = c < NOUT ? a[c] * (c < 3 ? sc.s2 : (c < 12 ? sc.s3 : sc.s4)) : 0.f;
    if (__all_sync(0xffffffffu, my == __shfl_sync(0xffffffffu, my, 0))) {
      // one target for the whole warp (pairs are ordered by target, runs are
      // long): reduce-scatter by recursive halving, 31 shuffles for the 32
      // columns; lane c ends with the warp's sum of column c
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < off; ++j) {
          const float send = upper ? x[j] : x[j + off];
          const float keep = upper ? x[j + off] : x[j];
          x[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
      }
      if (lane < NOUT) atomicAdd(L + lane, x[0]);
    } else {
      // runs of equal targets inside the warp: segmented sums to each run's
      // first lane
      const int up = __shfl_up_sync(0xffffffffu, my, 1);
      const bool head = act_row && (lane == 0 || up != my);
#pragma unroll
      for (int c = 0; c < NOUT; ++c) {
        float y = x[c];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const float o = __shfl_down_sync(0xffffffffu, y, off);
          const int ol = __shfl_down_sync(0xffffffffu, my, off);
          if (lane + off < 32 && ol == my) y += o;
        }
        if (head) atomicAdd(L + c, y);
      }
    }
  }  // pair blocks
}

// ---- generic tile GEMM for training: C[M][N] (+)= sum_k opA[m][k] opB[n][k] -------
// opA[m][k] = tA ? A[k*lda + m] : A[m*lda + k]; same for B.  Grid (M/128, N/128,
// splitK); each CTA runs its K range in chunks of 128 through TMEM and adds its
// partial into C with FP32 atomics (C must be zeroed when accumulating).
struct GemmSmem {
  __nv_bfloat16 a[128 * 128];
  __nv_bfloat16 b[128 * 128];
  uint64_t bar;
  uint32_t tmem;
};

__global__ void __launch_bounds__(128) gemm_tn_kernel(const __nv_bfloat16* __restrict__ A, int lda,
                                                      int tA, const __nv_bfloat16* __restrict__ B,
                                                      int ldb, int tB, float* __restrict__ C,
                                                      int ldc, int M, int N, int K, int kchunk,
                                                      int atomic) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  GemmSmem& S = *reinterpret_cast<GemmSmem*>(smem_raw);
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, 128);
  if (threadIdx.x == 0) {
    mbar_init(&S.bar, 1);
    fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * 128;
  const int nt = min(128, N - n0);
  const int nt16 = (nt + 15) & ~15;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  uint32_t ph = 0;
  bool ok = true, any = false;
  for (int k0 = kb; k0 < ke; k0 += 128) {
    const int kc = min(128, ke - k0);
    const int kc16 = (kc + 15) & ~15;
    // stage op(A)[m0 .. m0+128][k0 .. k0+kc16] and op(B)[n0 .. n0+nt16][...]
    for (int e = threadIdx.x; e < 128 * kc16; e += blockDim.x) {
      const int r = tA ? e % 128 : e / kc16, k = tA ? e / 128 : e % kc16;
      const int gm = m0 + r, gk = k0 + k;
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (gm < M && k < kc) v = tA ? A[static_cast<int64_t>(gk) * lda + gm] : A[static_cast<int64_t>(gm) * lda + gk];
      *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(S.a) + tc::kmajor_offset(r, k, kc16)) = v;
    }
    for (int e = threadIdx.x; e < nt16 * kc16; e += blockDim.x) {
      const int r = tB ? e % nt16 : e / kc16, k = tB ? e / nt16 : e % kc16;
      const int gn = n0 + r, gk = k0 + k;
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (r < nt && k < kc) v = tB ? B[static_cast<int64_t>(gk) * ldb + gn] : B[static_cast<int64_t>(gn) * ldb + gk];
      *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(S.b) + tc::kmajor_offset(r, k, kc16)) = v;
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0)
      tc::gemm_issue(tmem, S.a, S.b, kc16, tc::idesc_bf16(128, nt16), any, &S.bar, 0);
    any = true;
    if (!__syncthreads_and(wait_mma(&S.bar, ph))) {
      ok = false;
      break;
    }
  }
  if (ok && any) {
    const uint32_t lb = static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16;
    const int gm = m0 + threadIdx.x;
    for (int c0 = 0; c0 < nt16; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lb + c0, v);
      if (gm >= M) continue;
      for (int i = 0; i < 16; ++i) {
        const int gn = n0 + c0 + i;
        if (c0 + i >= nt) break;
        float* p = C + static_cast<int64_t>(gm) * ldc + gn;
        if (atomic)
          atomicAdd(p, v[i]);
        else
          *p = v[i];
      }
    }
  }
  if (!ok && threadIdx.x == 0) flag_status(kStatusTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 128);
}

// ---- element-wise training kernels ---------------------------------------------------
// dY = 2 w_r (Y - T) / (rows * NOUT) on the used outputs (w_r = 1 without
// row weights); loss partial sums of w_r (Y - T)^2.
__global__ void loss_grad_kernel(int rows, const float* __restrict__ Y, const float* __restrict__ T,
                                 const float* __restrict__ wrow, __nv_bfloat16* __restrict__ dY,
                                 float* __restrict__ dY32, float* __restrict__ loss) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t n = static_cast<int64_t>(rows) * OUT;
  float l = 0.f;
  if (i < n) {
    const int c = static_cast<int>(i % OUT);
    float g = 0.f;
    if (c < NOUT) {
      const float w = wrow ? wrow[i / OUT] : 1.f;
      const float e = Y[i] - T[i];
      l = w * e * e;
      g = 2.f * w * e / (static_cast<float>(rows) * NOUT);
    }
    dY[i] = __float2bfloat16(g);
    dY32[i] = g;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// dZ = dH * SiLU'(Z) (BF16 out), db += column sums of dZ.
__global__ void silu_back_kernel(int rows, int cols, const float* __restrict__ dH,
                                 const float* __restrict__ Z, __nv_bfloat16* __restrict__ dZ,
                                 float* __restrict__ db) {
  const int c = threadIdx.x;  // blockDim.x == cols
  float acc = 0.f;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int64_t i = static_cast<int64_t>(r) * cols + c;
    const float g = dH[i] * silu_grad(Z[i]);
    dZ[i] = __float2bfloat16(g);
    acc += g;
  }
  atomicAdd(db + c, acc);
}

__global__ void colsum_kernel(int rows, int cols, const float* __restrict__ G, float* __restrict__ db) {
  const int c = threadIdx.x;
  float acc = 0.f;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) acc += G[static_cast<int64_t>(r) * cols + c];
  atomicAdd(db + c, acc);
}

// Adam on FP32 master weights; refreshes the BF16 copy.
__global__ void adam_kernel(int n, float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v,
                            __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                            float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
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
  if (threadIdx.x == 0)
    tc::gemm_issue(tmem, sA, sB, K, tc::idesc_bf16(128, N), false, &bar, stride_mode);
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

template <typename K>
int set_smem(K kernel, size_t bytes) {
  FVX_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(bytes)));
  return FVX_OK;
}

}  // namespace mlp

// Fused learned far field for the treecode: local expansions of the learned
// (leaf, cell) pairs added into leaf_local[n_leaves][32] (zeroed by the caller).
// The learned far field of both lists in one launch: local expansions added
// into a.local / b.local (zeroed by the caller).
int mlp_farfield_launch(const FarPairs& a, const FarPairs& b, const float* rec, const void* W,
                        const float* bias, cudaStream_t s, const FarJudge& judge) {
  using namespace mlp;
  const int npairs = a.n + b.n;
  if (npairs <= 0) return FVX_OK;
  static int done = 0;
  if (!done) {
    // setmaxnreg moves registers between the warpgroups within what the launch
    // holds: refuse to run a build whose launch would hold fewer
    cudaFuncAttributes fa{};
    FVX_CUDA_TRY(cudaFuncGetAttributes(&fa, farfield_kernel));
    const int per_thread = (fa.numRegs + 7) / 8 * 8;
    FVX_ARG_CHECK(per_thread * kFarThreads >= kFarRegsNeeded,
                  "far-field kernel built with %d registers per thread; its warpgroups need %d",
                  fa.numRegs, kFarRegsNeeded / kFarThreads);
    int rc = set_smem(farfield_kernel, sizeof(FarSmem));
    if (rc) return rc;
    done = 1;
  }
  const int nctas = ((npairs + 127) / 128 + kGroups - 1) / kGroups;
  const int grid = nctas < device_sm_count() ? nctas : device_sm_count();
  farfield_kernel<<<grid, kFarThreads, sizeof(FarSmem), s>>>(
      FarIO{a, b, rec, judge}, npairs, static_cast<const __nv_bfloat16*>(W), bias);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

// The analytic multipole-to-local translation of both lists in one launch.
int m2l_farfield_launch(const FarPairs& a, const FarPairs& b, const float* rec, cudaStream_t s,
                        const FarJudge& judge) {
  const int npairs = a.n + b.n;
  if (npairs <= 0) return FVX_OK;
  const int blocks = (npairs + mlp::kM2lThreads - 1) / mlp::kM2lThreads;
  const int grid = blocks < 2 * device_sm_count() ? blocks : 2 * device_sm_count();
  mlp::m2l_pairs_kernel<<<grid, mlp::kM2lThreads, 0, s>>>(mlp::FarIO{a, b, rec, judge});
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

// sums: 2 cap x 30 doubles (zeroed here); off: 2 cap + 1 ints of scratch
int judge_sums_launch(const JudgeSampleView& S, const uint32_t* leaf_key, const int* cell_start,
                      const int* cell_count, const float4* sp, const float4* sa,
                      const int* leaf_of_particle, float h, double* sums, int* off,
                      cudaStream_t s) {
  if (S.cap <= 0) return FVX_OK;
  FVX_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(double) * 30 * 2 * size_t(S.cap), s));
  mlp::judge_chunks_kernel<<<1, 1024, 0, s>>>(S, cell_count, off);
  FVX_LAUNCH_CHECK();
  mlp::judge_sums_kernel<<<4 * device_sm_count(), mlp::kTargetsThreads, 0, s>>>(
      S, off, leaf_key, cell_start, cell_count, sp, sa, leaf_of_particle, h, sums);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

// partial: scratch of npairs x slices x 30 doubles
int mlp_pair_targets_launch(int npairs, int stride, const int* pair_leaf, const int* pair_cell,
                            const uint32_t* tgt_key, float h_tgt, const uint32_t* leaf_key,
                            const float* rec, const int* cell_start,
                            const int* cell_count, const float4* sp, const float4* sa,
                            const int* leaf_of_particle, float h, void* X, float* T,
                            float* A, float* scale, double* partial, int slices,
                            cudaStream_t s) {
  if (npairs <= 0) return FVX_OK;
  mlp::pair_sums_kernel<<<dim3(npairs, slices), mlp::kTargetsThreads, 0, s>>>(
      npairs, stride, pair_leaf, pair_cell, tgt_key, h_tgt, leaf_key, cell_start, cell_count, sp,
      sa, leaf_of_particle, h, partial);
  FVX_LAUNCH_CHECK();
  mlp::pair_targets_kernel<<<(npairs + 127) / 128, 128, 0, s>>>(
      npairs, stride, slices, pair_leaf, pair_cell, tgt_key, h_tgt, rec, partial,
      static_cast<__nv_bfloat16*>(X), T, A, scale);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

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
                    float* z_store, void* h_store, void* stream) {
  using namespace fvx::mlp;
  FVX_ARG_CHECK(rows >= 0 && X && W && bias && Y, "null argument");
  if (rows == 0) return FVX_OK;
  static int done = 0;
  if (!done) {
    int rc = set_smem(mlp_fwd_kernel<false>, sizeof(FwdSmem));
    if (!rc) rc = set_smem(mlp_fwd_kernel<true>, sizeof(FwdSmem));
    if (rc) return rc;
    done = 1;
  }
  const RowsIO A{static_cast<const __nv_bfloat16*>(X), Y, z_store,
                 static_cast<__nv_bfloat16*>(h_store)};
  const int nctas = ((rows + 127) / 128 + kGroups - 1) / kGroups;
  const int grid = nctas < fvx::device_sm_count() ? nctas : fvx::device_sm_count();
  // without stores it is inference: the arithmetic the treecode far field runs
  auto kern = (z_store || h_store) ? mlp_fwd_kernel<false> : mlp_fwd_kernel<true>;
  kern<<<grid, kGroups * 128, sizeof(FwdSmem), static_cast<cudaStream_t>(stream)>>>(
      A, rows, static_cast<const __nv_bfloat16*>(W), bias);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_gemm(const void* A, int lda, int tA, const void* B, int ldb, int tB, float* C,
                 int ldc, int M, int N, int K, int split_k, int accumulate, void* stream) {
  using namespace fvx::mlp;
  FVX_ARG_CHECK(A && B && C && M > 0 && N > 0 && K > 0 && split_k >= 1, "bad gemm arguments");
  FVX_ARG_CHECK(split_k == 1 || accumulate, "split-K needs accumulation into C");
  static int done = 0;
  if (!done) {
    int rc = set_smem(gemm_tn_kernel, sizeof(GemmSmem));
    if (rc) return rc;
    done = 1;
  }
  int kchunk = (K + split_k - 1) / split_k;
  kchunk = (kchunk + 127) & ~127;
  const int sk = (K + kchunk - 1) / kchunk;
  dim3 grid((M + 127) / 128, (N + 127) / 128, sk);
  gemm_tn_kernel<<<grid, 128, sizeof(GemmSmem), static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(A), lda, tA, static_cast<const __nv_bfloat16*>(B), ldb,
      tB, C, ldc, M, N, K, kchunk, accumulate);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_loss_grad(int rows, const float* Y, const float* T, const float* row_weight, void* dY,
                      float* dY32, float* loss, void* stream) {
  FVX_ARG_CHECK(rows >= 0 && Y && T && dY && dY32 && loss, "null argument");
  const int64_t n = static_cast<int64_t>(rows) * fvx::mlp::OUT;
  if (n == 0) return FVX_OK;
  fvx::mlp::loss_grad_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0,
                               static_cast<cudaStream_t>(stream)>>>(
      rows, Y, T, row_weight, static_cast<__nv_bfloat16*>(dY), dY32, loss);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_silu_back(int rows, int cols, const float* dH, const float* Z, void* dZ, float* db,
                      void* stream) {
  FVX_ARG_CHECK(rows > 0 && cols > 0 && cols <= 1024 && dH && Z && dZ && db, "bad arguments");
  const int grid = rows < 1024 ? rows : 1024;
  fvx::mlp::silu_back_kernel<<<grid, cols, 0, static_cast<cudaStream_t>(stream)>>>(
      rows, cols, dH, Z, static_cast<__nv_bfloat16*>(dZ), db);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_colsum(int rows, int cols, const float* G, float* db, void* stream) {
  FVX_ARG_CHECK(rows > 0 && cols > 0 && cols <= 1024 && G && db, "bad arguments");
  const int grid = rows < 1024 ? rows : 1024;
  fvx::mlp::colsum_kernel<<<grid, cols, 0, static_cast<cudaStream_t>(stream)>>>(rows, cols, G, db);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_mlp_adam(int n, float* w, const float* g, float* m, float* v, void* wb, float lr,
                 float b1, float b2, float eps, int step, void* stream) {
  FVX_ARG_CHECK(n > 0 && w && g && m && v && step >= 1, "bad arguments");
  const float bc1 = 1.f - powf(b1, static_cast<float>(step));
  const float bc2 = 1.f - powf(b2, static_cast<float>(step));
  fvx::mlp::adam_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, w, g, m, v, static_cast<__nv_bfloat16*>(wb), lr, b1, b2, eps, bc1, bc2);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

}  // extern "C"
