// fvx_mlp.cu -- BF16 tensor-core MLP of the learned far-field operator.
//
// Network: 48 inputs (35 features, zero padded) -> 3 x 128 hidden (SiLU) ->
// 32 outputs (30 used), weights [out][in] in BF16 with FP32 master copies,
// FP32 biases.  Inference and training run on tcgen05 (fvx_tc.cuh):
//   * forward: a persistent CTA per SM keeps all weights in shared memory in
//     the K-major canonical layout; each of its two warpgroups owns a 128-row
//     tile at a time and chains the four layers through its half of the
//     tensor memory: MMA into TMEM -> tcgen05.ld -> bias + SiLU in registers
//     -> BF16 back into the group's shared activation tile -> next MMA, so
//     one group's epilogue overlaps the other's MMAs.  Two input/output policies: plain rows
//     (X -> Y, with the hidden pre-activations / activations kept for
//     training), and the treecode's learned far field (features computed
//     in-kernel from the (target leaf, source cell) pair list, outputs scaled
//     back to physical local-expansion coefficients and added to the leaf's
//     local expansion);
//   * training: a generic tile GEMM C = op(A) op(B)^T on tcgen05 (operands
//     staged transposed as needed by the threads, split over K with FP32
//     atomics) for dW = dZ^T H and dH = dZ W, plus element-wise kernels for
//     the loss gradient, the SiLU backward with bias gradients, and Adam.
#include <cuda_bf16.h>

#include "fvx_common.cuh"
#include "fvx_tc.cuh"

namespace fvx {
namespace mlp {

constexpr int IN = 48, H = 128, OUT = 32, NFEAT = 35, NOUT = 30;
constexpr int kThreads = 512;  // forward: four warpgroups
// packed BF16 weight offsets (elements)
constexpr int W1o = 0, W2o = W1o + H * IN, W3o = W2o + H * H, W4o = W3o + H * H,
              WN = W4o + OUT * H;
// packed bias offsets
constexpr int B1o = 0, B2o = H, B3o = 2 * H, B4o = 3 * H, BN = 3 * H + OUT;
constexpr int kRecFloats = 40;  // treecode cell record (fvx_tree.cu)
constexpr int kTargetsThreads = 256;  // FP64 exact-expansion sums: threads per pair

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
  float aux[kGroups][128][4];  // far field: the output scales m/d^2, m/d^3, m/d^4 of each row
  float bias[BN];
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
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// Barrier over the 128 threads of warpgroup g (named barrier 1 + g).
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

// Multipole to local, analytic: the local expansion at the target centre of
// the source cell's quadrupole expansion, in the network's normalised output
// units (unit distance along n = R/d; f = the pair's FP32 features).  With
// C-scaled moments the vector potential is Psi_m = -(M0_m phi - M1_ma d_a phi
// + 1/2 M2_mab d_ab phi), phi = 1/|r|, and u_i = eps_ijm d_j Psi_m; the
// derivatives of phi at |r| = 1 are contracted with the moments in closed
// form (d^p phi = sum over index pairings of (-1)^(p-k) (2p-2k-1)!! n..n d..d).
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
// that the analytic kernel keeps only one component's moments live
struct RecordMoments {
  const float* rec;
  float nx, ny, nz, hs_d, im, ih;
  __device__ float n(int i) const { return i == 0 ? nx : (i == 1 ? ny : nz); }
  __device__ float hs() const { return hs_d; }
  __device__ float c(int m) const { return rec[4 + m] * im; }
  __device__ float m1(int q) const { return rec[10 + q] * im * ih; }
  __device__ float m2(int q) const { return rec[19 + q] * im * ih * ih; }
};

// Multipole to local, analytic: the local expansion at the target centre of
// the source cell's quadrupole expansion, in the network's normalised output
// units (unit distance along n = R/d).  With C-scaled moments the vector
// potential is Psi_m = -(M0_m phi - M1_ma d_a phi + 1/2 M2_mab d_ab phi),
// phi = 1/|r|, and u_i = eps_ijm d_j Psi_m; the derivatives of phi at |r| = 1
// are contracted with the moments in closed form (d^p phi = sum over index
// pairings of (-1)^(p-k) (2p-2k-1)!! n..n d..d).
// Output accumulators of m2l_core: a register array, or a thread's column of
// a shared-memory block (stride = the block size), whose dynamic indexing
// (the output row depends on the loop's component) stays out of local memory.
struct SharedColumn {
  float* base;
  int stride;
  __device__ float& operator[](int q) const { return base[q * stride]; }
};

// x[i] of a 3-vector held in registers, for a run-time i (selects, not a
// local-memory array)
__device__ __forceinline__ float sel3(float x0, float x1, float x2, int i) {
  return i == 0 ? x0 : (i == 1 ? x1 : x2);
}

template <class Src, class Out>
__device__ __forceinline__ void m2l_core(const Src& src, Out&& out) {
  const float nv[3] = {src.n(0), src.n(1), src.n(2)};
  const float hs = src.hs();
#pragma unroll
  for (int q = 0; q < NOUT; ++q) out[q] = 0.f;
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    const float c = src.c(m);
    const float v[3] = {src.m1(3 * m) * hs, src.m1(3 * m + 1) * hs, src.m1(3 * m + 2) * hs};
    const float h2 = hs * hs;
    float q6[6];
#pragma unroll
    for (int u = 0; u < 6; ++u) q6[u] = src.m2(6 * m + u);
    const float Q[3][3] = {{q6[0] * h2, q6[1] * h2, q6[2] * h2},
                           {q6[1] * h2, q6[3] * h2, q6[4] * h2},
                           {q6[2] * h2, q6[4] * h2, q6[5] * h2}};
    const float vn = v[0] * nv[0] + v[1] * nv[1] + v[2] * nv[2];
    float qn[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) qn[j] = Q[j][0] * nv[0] + Q[j][1] * nv[1] + Q[j][2] * nv[2];
    const float nqn = qn[0] * nv[0] + qn[1] * nv[1] + qn[2] * nv[2];
    const float tr = Q[0][0] + Q[1][1] + Q[2][2];
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
      const int j = (m + 1 + jj) % 3;      // the two j != m
      const int i = 3 - m - j;
      const float sg = ((j - i + 3) % 3 == 1) ? 1.f : -1.f;  // eps_ijm
      const float nj = sel3(nv[0], nv[1], nv[2], j);
      const float vj = sel3(v[0], v[1], v[2], j);
      const float qnj = sel3(qn[0], qn[1], qn[2], j);
      // u: c phi_j - v_a phi_aj + 1/2 Q_ab phi_abj
      const float p1 = -nj * c - (3.f * vn * nj - vj) + 0.5f * (-15.f * nqn * nj + 3.f * tr * nj + 6.f * qnj);
      out[i] -= sg * p1;
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        const float dl = j == n ? 1.f : 0.f;
        const float nn = nv[n];
        const float phi2 = 3.f * nj * nn - dl;
        const float vphi3 = -15.f * vn * nj * nn + 3.f * (vj * nn + v[n] * nj + vn * dl);
        const float qjn = sel3(Q[0][n], Q[1][n], Q[2][n], j);
        const float qphi4 = 105.f * nqn * nj * nn -
                            15.f * (tr * nj * nn + 2.f * qnj * nn + 2.f * qn[n] * nj + nqn * dl) +
                            3.f * tr * dl + 6.f * qjn;
        out[3 + 3 * i + n] -= sg * (c * phi2 - vphi3 + 0.5f * qphi4);
      }
#pragma unroll
      for (int u = 0; u < 6; ++u) {
        const int k = u < 3 ? 0 : (u < 5 ? 1 : 2);
        const int n = u < 3 ? u : (u < 5 ? u - 2 : 2);
        const float nk = nv[k], nn = nv[n];
        const float djk = j == k ? 1.f : 0.f, djn = j == n ? 1.f : 0.f, dkn = k == n ? 1.f : 0.f;
        const float nnn = nj * nk * nn;
        const float dsum = djk * nn + djn * nk + dkn * nj;
        const float phi3 = -15.f * nnn + 3.f * dsum;
        const float vphi4 = 105.f * vn * nnn -
                            15.f * (vj * nk * nn + v[k] * nj * nn + v[n] * nj * nk + vn * dsum) +
                            3.f * (vj * dkn + v[k] * djn + v[n] * djk);
        const float qjn = sel3(Q[0][n], Q[1][n], Q[2][n], j);
        const float qjk = sel3(Q[0][k], Q[1][k], Q[2][k], j);
        const float qphi5 =
            -945.f * nqn * nnn +
            105.f * (tr * nnn + 2.f * (qnj * nk * nn + qn[k] * nj * nn + qn[n] * nj * nk) + nqn * dsum) -
            15.f * (2.f * (qnj * dkn + qn[k] * djn + qn[n] * djk) + nj * (tr * dkn + 2.f * Q[k][n]) +
                    nk * (tr * djn + 2.f * qjn) + nn * (tr * djk + 2.f * qjk));
        out[12 + 6 * i + u] -= sg * (c * phi3 - vphi4 + 0.5f * qphi5);
      }
    }
  }
}

__device__ __forceinline__ void m2l_quadrupole(const float* f, float* out) {
  m2l_core(FeatureMoments{f}, out);
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

struct FarIO {
  const int* pair_leaf;    // leaf id of each learned pair
  const int* pair_cell;    // global cell id of each learned pair
  const uint32_t* leaf_key;
  const float* rec;        // cell records
  float h;                 // leaf size
  float* leaf_local;       // [n_leaves][32] local expansions (accumulated)
};

template <bool FAR>
struct FwdArgs {
  RowsIO r;
  FarIO f;
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

__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& ph) {
  const bool ok = mbar_wait(bar, ph);
  ph ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// group-local fence + barrier: smem writes -> async proxy, TMEM reads done
__device__ __forceinline__ void group_handoff(int g) {
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  group_sync(g);
  tc::fence_after_sync();
}

template <bool FAR>
__global__ void __launch_bounds__(kThreads) mlp_fwd_kernel(FwdArgs<FAR> A, int rows,
                                                           const __nv_bfloat16* __restrict__ W,
                                                           const float* __restrict__ bias) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  FwdSmem& S = *reinterpret_cast<FwdSmem*>(smem_raw);
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, 128 * kGroups);
  if (threadIdx.x == 0) {
    for (int g = 0; g < kGroups; ++g) mbar_init(&S.bar[g], 1);
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
  const int grp = threadIdx.x >> 7;   // warpgroup
  const int lt = threadIdx.x & 127;   // row of the group's tile
  const uint32_t tmem = S.tmem + static_cast<uint32_t>(128 * grp);
  const uint32_t lane_base = static_cast<uint32_t>(32 * ((threadIdx.x >> 5) & 3)) << 16;
  __nv_bfloat16* act = S.act[grp];
  uint64_t* bar = &S.bar[grp];
  uint32_t ph = 0;
  bool ok = true;
  const int ntiles = (rows + 127) / 128;
  for (int tile = kGroups * blockIdx.x + grp; tile < ntiles && ok; tile += kGroups * gridDim.x) {
    const int row = tile * 128 + lt;
    const bool act_row = row < rows;
    int leaf = 0;
    // input tile (K = 48)
    {
      char* base = reinterpret_cast<char*>(act);
      if constexpr (FAR) {
        float f[IN];
        float* ax = S.aux[grp][lt];
        if (act_row) {
          leaf = A.f.pair_leaf[row];
          const float3 cT = leaf_center(A.f.leaf_key[leaf], A.f.h);
          const PairScale sc = pair_features(
              A.f.rec + static_cast<int64_t>(A.f.pair_cell[row]) * kRecFloats, cT.x, cT.y, cT.z,
              A.f.h, f);
          ax[0] = sc.s2;
          ax[1] = sc.s3;
          ax[2] = sc.s4;
        } else {
          for (int q = 0; q < IN; ++q) f[q] = 0.f;
        }
        for (int k8 = 0; k8 < IN / 8; ++k8) {
          __align__(16) __nv_bfloat162 b[4];
          for (int q = 0; q < 4; ++q) b[q] = __floats2bfloat162_rn(f[8 * k8 + 2 * q], f[8 * k8 + 2 * q + 1]);
          *reinterpret_cast<uint4*>(base + tc::kmajor_offset(lt, 8 * k8, IN)) =
              *reinterpret_cast<uint4*>(b);
        }
      } else {
        for (int k8 = 0; k8 < IN / 8; ++k8) {
          uint4 v = make_uint4(0, 0, 0, 0);
          if (act_row)
            v = *reinterpret_cast<const uint4*>(A.r.X + static_cast<int64_t>(row) * IN + 8 * k8);
          *reinterpret_cast<uint4*>(base + tc::kmajor_offset(lt, 8 * k8, IN)) = v;
        }
      }
    }
    const __nv_bfloat16* wl[3] = {S.w1, S.w2, S.w3};
    for (int l = 0; l < 3 && ok; ++l) {
      group_handoff(grp);
      if (lt == 0)
        tc::gemm_issue(tmem, act, wl[l], l == 0 ? IN : H, tc::idesc_bf16(128, H), false, bar, 0);
      if (!group_sync_and(grp, wait_mma(bar, ph))) {
        ok = false;
        break;
      }
      float* zo = nullptr;
      __nv_bfloat16* ho = nullptr;
      if constexpr (!FAR) {
        if (A.r.z_store && act_row) zo = A.r.z_store + (static_cast<int64_t>(l) * rows + row) * H;
        if (A.r.h_store && act_row) ho = A.r.h_store + (static_cast<int64_t>(l) * rows + row) * H;
      }
      epilogue_hidden(tmem, lt, S.bias + l * H, act, zo, ho);
    }
    if (!ok) break;
    group_handoff(grp);
    if (lt == 0) tc::gemm_issue(tmem, act, S.w4, H, tc::idesc_bf16(128, OUT), false, bar, 0);
    if (!group_sync_and(grp, wait_mma(bar, ph))) {
      ok = false;
      break;
    }
    if constexpr (FAR) {
      // the learned residual of this row, back to physical units (the analytic
      // translation is added by its own kernel)
      float x[OUT];
      for (int c0 = 0; c0 < OUT; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + lane_base + c0, v);
        const float* ax = S.aux[grp][lt];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int c = c0 + i;
          const float sc = c < 3 ? ax[0] : (c < 12 ? ax[1] : ax[2]);
          x[c] = (act_row && c < NOUT) ? (v[i] + S.bias[B4o + c]) * sc : 0.f;
        }
      }
      const int lane = threadIdx.x & 31;
      const int my = act_row ? leaf : -1 - lane;
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
        if (lane < NOUT) atomicAdd(A.f.leaf_local + static_cast<int64_t>(leaf) * OUT + lane, x[0]);
      } else {
        // runs of equal targets inside the warp: segmented sums to each run's
        // first lane, which adds them to the target's expansion
        const int up = __shfl_up_sync(0xffffffffu, my, 1);
        const bool head = act_row && (lane == 0 || up != my);
        float* L = act_row ? A.f.leaf_local + static_cast<int64_t>(leaf) * OUT : nullptr;
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
    for (int c0 = 0; c0 < OUT && !FAR; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + c0, v);
      if constexpr (FAR) continue;
      if (!act_row) continue;
      {
        float4* y = reinterpret_cast<float4*>(A.r.Y + static_cast<int64_t>(row) * OUT + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          y[q] = make_float4(v[4 * q] + S.bias[B4o + c0 + 4 * q],
                             v[4 * q + 1] + S.bias[B4o + c0 + 4 * q + 1],
                             v[4 * q + 2] + S.bias[B4o + c0 + 4 * q + 2],
                             v[4 * q + 3] + S.bias[B4o + c0 + 4 * q + 3]);
      }
    }
    tc::fence_before_sync();
    group_sync(grp);
    tc::fence_after_sync();
  }
  if (!ok && lt == 0) flag_status(kStatusTimeout);
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
  const int lane = threadIdx.x & 31;
  __shared__ double red[kTargetsThreads / 32][NOUT];
  if (pr >= npairs) return;
  const int t = pair_leaf[static_cast<int64_t>(pr) * stride],
            g = pair_cell[static_cast<int64_t>(pr) * stride];
  const float3 cT = leaf_center(tgt_key[t], h_tgt);
  double acc[NOUT];
#pragma unroll
  for (int q = 0; q < NOUT; ++q) acc[q] = 0.0;
  const int c0 = cell_start[g], cn = cell_count[g];
  const int per = (cn + gridDim.y - 1) / gridDim.y;
  const int s0 = c0 + static_cast<int>(blockIdx.y) * per;
  const int n = max(0, min(per, c0 + cn - s0));
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
#pragma unroll
  for (int q = 0; q < NOUT; ++q)
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  if (lane == 0)
    for (int q = 0; q < NOUT; ++q) red[threadIdx.x >> 5][q] = acc[q];
  __syncthreads();
  if (threadIdx.x < NOUT) {
    double v = 0.0;
    for (int w = 0; w < kTargetsThreads / 32; ++w) v += red[w][threadIdx.x];
    partial[(static_cast<int64_t>(pr) * gridDim.y + blockIdx.y) * NOUT + threadIdx.x] = v;
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
constexpr int kM2lThreads = 256;

__global__ void __launch_bounds__(kM2lThreads) m2l_pairs_kernel(int npairs, const int* __restrict__ pair_leaf,
                                                        const int* __restrict__ pair_cell,
                                                        const uint32_t* __restrict__ leaf_key,
                                                        const float* __restrict__ rec, float h,
                                                        float* __restrict__ leaf_local) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool act_row = row < npairs;
  __shared__ float s_acc[NOUT * kM2lThreads];
  const SharedColumn acc{s_acc + threadIdx.x, kM2lThreads};
  PairScale sc{0.f, 0.f, 0.f};
  int leaf = 0;
  if (act_row) {
    leaf = pair_leaf[row];
    const float3 cT = leaf_center(leaf_key[leaf], h);
    const float* r = rec + static_cast<int64_t>(pair_cell[row]) * kRecFloats;
    const PairGeom g = pair_geom(r, cT.x, cT.y, cT.z);
    const RecordMoments src{r, g.Rx * g.id, g.Ry * g.id, g.Rz * g.id, g.hS * g.id, g.im, g.ih};
    m2l_core(src, acc);
    sc = pair_scale(g);
  }
  float a[NOUT];
#pragma unroll
  for (int q = 0; q < NOUT; ++q) a[q] = act_row ? acc[q] : 0.f;
  const int my = act_row ? leaf : -1 - lane;
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
    if (lane < NOUT) atomicAdd(leaf_local + static_cast<int64_t>(leaf) * OUT + lane, x[0]);
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
      if (head) atomicAdd(leaf_local + static_cast<int64_t>(leaf) * OUT + c, y);
    }
  }
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
int mlp_farfield_launch(int npairs, const int* pair_leaf, const int* pair_cell,
                        const uint32_t* leaf_key, const float* rec, float h, const void* W,
                        const float* bias, float* leaf_local, cudaStream_t s) {
  using namespace mlp;
  if (npairs <= 0) return FVX_OK;
  static int done = 0;
  if (!done) {
    int rc = set_smem(mlp_fwd_kernel<true>, sizeof(FwdSmem));
    if (rc) return rc;
    done = 1;
  }
  FwdArgs<true> A;
  A.r = RowsIO{nullptr, nullptr, nullptr, nullptr};
  A.f = FarIO{pair_leaf, pair_cell, leaf_key, rec, h, leaf_local};
  const int nctas = ((npairs + 127) / 128 + kGroups - 1) / kGroups;
  const int grid = nctas < device_sm_count() ? nctas : device_sm_count();
  mlp_fwd_kernel<true><<<grid, kThreads, sizeof(FwdSmem), s>>>(
      A, npairs, static_cast<const __nv_bfloat16*>(W), bias);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int m2l_farfield_launch(int npairs, const int* pair_leaf, const int* pair_cell,
                        const uint32_t* leaf_key, const float* rec, float h, float* leaf_local,
                        cudaStream_t s) {
  if (npairs <= 0) return FVX_OK;
  mlp::m2l_pairs_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(npairs, pair_leaf, pair_cell,
                                                             leaf_key, rec, h, leaf_local);
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
    if (rc) return rc;
    done = 1;
  }
  FwdArgs<false> A;
  A.r = RowsIO{static_cast<const __nv_bfloat16*>(X), Y, z_store,
               static_cast<__nv_bfloat16*>(h_store)};
  A.f = FarIO{nullptr, nullptr, nullptr, nullptr, 0.f, nullptr};
  const int nctas = ((rows + 127) / 128 + kGroups - 1) / kGroups;
  const int grid = nctas < fvx::device_sm_count() ? nctas : fvx::device_sm_count();
  mlp_fwd_kernel<false><<<grid, kThreads, sizeof(FwdSmem), static_cast<cudaStream_t>(stream)>>>(
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
