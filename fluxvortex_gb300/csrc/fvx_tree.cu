// fvx_tree.cu -- cell-binned treecode for the particle self-induction sweeps.
//
// The reference sums every particle pair directly (src/fluxvortex/kernel.py:
// 69-190, O(N^2) per sweep).  This treecode replaces a self-sweep over N
// particles by
//   near field: direct FP32 pair sums (same core arithmetic as fvx_particles)
//               between each target leaf and the leaves its interaction list
//               keeps near, with compensated accumulation;
//   far field:  a quadrupole expansion of the vector potential
//               Psi_m = (1/4pi) sum a_m/|x - x_s| about each accepted cell's
//               centre (u = curl Psi, J_in = eps_ijm d_n d_j Psi_m), FP32.
//
// Build (every sweep state, all on the device):
//   bbox -> host picks the grid (tree_params.grid_params: root cube of 2^L
//   leaves of size c 2^k, c in {1, 5/4, 3/2, 7/4}, aligned to the leaf size) -> 30-bit Morton keys -> stable LSD radix
//   sort (4 x 8-bit digits, per-block histograms, warp-match ranking) ->
//   leaf cells = runs of equal keys, coarser levels = runs of equal key >> 3
//   among the finer level's cells -> sorted FP32 particle records relative to
//   their leaf centre -> leaf moments (one warp per leaf) -> M2M shifts up the
//   levels -> interaction lists per target leaf (depth-first traversal, exact
//   acceptance test |dc|^2 > 3/4 (h_T + h_S)^2 / theta^2 in FP64) -> eval.
// Because cell centres are exact binary fractions, centre differences are
// exact in FP32 and pair offsets are (c_T - c_S) + (o_t - o_s) with small
// in-cell offsets o.
#include <cstring>
#include <type_traits>

#include <algorithm>
#include <cstddef>
#include <cstring>

#include "fvx_common.cuh"
#include "fvx_pair_math.cuh"

namespace fvx {
namespace tree {

constexpr int kScanBlock = 2048;   // elements per scan block (1024 threads x 2)
constexpr int kSortItems = 1024;   // keys per radix-sort block (256 threads x 4)
constexpr int kEvalThreads = 32;   // eval CTA (one warp); 1, 2 or 4 targets per thread
constexpr int kFarTile = 32;       // far cells staged per tile
constexpr int kNearTile = 128;     // source particles staged per tile
constexpr int kRecFloats = 40;     // far-cell record
constexpr double kC = -0.07957747154594767;  // -1/(4 pi)

// ---- scan: exclusive / inclusive prefix sums of int32 ------------------------
__global__ void scan_block_kernel(const int* __restrict__ in, int n, int* __restrict__ out,
                                  int* __restrict__ block_sums, int inclusive) {
  __shared__ int s[kScanBlock];
  const int base = blockIdx.x * kScanBlock;
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x) {
    const int i = base + k;
    s[k] = i < n ? in[i] : 0;
  }
  __syncthreads();
  // Hillis-Steele on kScanBlock elements with kScanBlock / 2 threads
  for (int off = 1; off < kScanBlock; off <<= 1) {
    int v0 = 0, v1 = 0;
    const int k0 = threadIdx.x, k1 = threadIdx.x + blockDim.x;
    if (k0 >= off) v0 = s[k0 - off];
    if (k1 >= off) v1 = s[k1 - off];
    __syncthreads();
    s[k0] += v0;
    s[k1] += v1;
    __syncthreads();
  }
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x) {
    const int i = base + k;
    if (i < n) out[i] = inclusive ? s[k] : s[k] - (i < n ? in[i] : 0);
  }
  if (threadIdx.x == 0 && block_sums) block_sums[blockIdx.x] = s[kScanBlock - 1];
}

__global__ void scan_add_kernel(int* __restrict__ out, int n, const int* __restrict__ offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanBlock];
}

// total of an inclusive scan -> *total
__global__ void scan_total_kernel(const int* __restrict__ incl, int n, int* __restrict__ total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *total = n > 0 ? incl[n - 1] : 0;
}

}  // namespace tree

// Device-wide scan of n <= 2048*2048 ints (in -> out); tmp holds >= 2*2048 ints.
int scan_ints(const int* in, int n, int* out, int inclusive, int* tmp, cudaStream_t s) {
  using namespace tree;
  if (n <= 0) return FVX_OK;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  FVX_ARG_CHECK(nb <= kScanBlock, "scan of %d elements exceeds 2^22", n);
  int* bsum = tmp;
  int* bsum_ex = tmp + kScanBlock;
  scan_block_kernel<<<nb, kScanBlock / 2, 0, s>>>(in, n, out, bsum, inclusive);
  FVX_LAUNCH_CHECK();
  if (nb > 1) {
    scan_block_kernel<<<1, kScanBlock / 2, 0, s>>>(bsum, nb, bsum_ex, nullptr, 0);
    FVX_LAUNCH_CHECK();
    scan_add_kernel<<<(n + 255) / 256, 256, 0, s>>>(out, n, bsum_ex);
    FVX_LAUNCH_CHECK();
  }
  return FVX_OK;
}

namespace tree {

// ---- bounding box -------------------------------------------------------------
// Bounding box of the finite positions; particles with a non-finite
// coordinate are counted into *nonfinite (the sweep refuses them).
// Bounding box of the positions and the smallest core (7 values per block:
// lo xyz, hi xyz, min sigma), and the count of non-finite positions.
__global__ void bbox_partial_kernel(int64_t n, const double* __restrict__ pos,
                                    const double* __restrict__ sigma,
                                    double* __restrict__ partial,
                                    unsigned* __restrict__ nonfinite) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, smin = 1e300;
  unsigned bad = 0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    bool fin = true;
    for (int c = 0; c < 3; ++c) {
      const double v = pos[3 * i + c];
      fin = fin && isfinite(v);
      lo[c] = fmin(lo[c], v);
      hi[c] = fmax(hi[c], v);
    }
    smin = fmin(smin, sigma[i]);
    bad += fin ? 0u : 1u;
  }
  if (bad) atomicAdd(nonfinite, bad);
  __shared__ double s[7][256];
  for (int c = 0; c < 3; ++c) {
    s[c][threadIdx.x] = lo[c];
    s[3 + c][threadIdx.x] = hi[c];
  }
  s[6][threadIdx.x] = smin;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      for (int c = 0; c < 3; ++c) {
        s[c][threadIdx.x] = fmin(s[c][threadIdx.x], s[c][threadIdx.x + st]);
        s[3 + c][threadIdx.x] = fmax(s[3 + c][threadIdx.x], s[3 + c][threadIdx.x + st]);
      }
      s[6][threadIdx.x] = fmin(s[6][threadIdx.x], s[6][threadIdx.x + st]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 7) partial[blockIdx.x * 7 + threadIdx.x] = s[threadIdx.x][0];
}

// One CTA of kBboxFinalThreads: each thread folds a strided share of the
// partial boxes (independent loads), then warps and the CTA reduce.
constexpr int kBboxFinalThreads = 256;
__global__ void __launch_bounds__(kBboxFinalThreads) bbox_final_kernel(
    int nb, const double* __restrict__ partial, double* __restrict__ out) {
  double r[7] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300, 1e300};
  for (int b = threadIdx.x; b < nb; b += kBboxFinalThreads) {
    for (int c = 0; c < 3; ++c) {
      r[c] = fmin(r[c], partial[b * 7 + c]);
      r[3 + c] = fmax(r[3 + c], partial[b * 7 + 3 + c]);
    }
    r[6] = fmin(r[6], partial[b * 7 + 6]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    for (int c = 0; c < 3; ++c) {
      r[c] = fmin(r[c], __shfl_xor_sync(0xffffffffu, r[c], o));
      r[3 + c] = fmax(r[3 + c], __shfl_xor_sync(0xffffffffu, r[3 + c], o));
    }
    r[6] = fmin(r[6], __shfl_xor_sync(0xffffffffu, r[6], o));
  }
  __shared__ double s[kBboxFinalThreads / 32][7];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int c = 0; c < 7; ++c) s[w][c] = r[c];
  __syncthreads();
  if (threadIdx.x < 7) {
    const int c = threadIdx.x;
    double v = s[0][c];
    for (int k = 1; k < kBboxFinalThreads / 32; ++k)
      v = (c < 3 || c == 6) ? fmin(v, s[k][c]) : fmax(v, s[k][c]);
    out[c] = v;
  }
}

// ---- Morton keys ----------------------------------------------------------------
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__device__ __forceinline__ uint32_t compact10(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030C30C3u;
  v = (v | (v >> 4)) & 0x0300F00Fu;
  v = (v | (v >> 8)) & 0x030000FFu;
  v = (v | (v >> 16)) & 0x000003FFu;
  return v;
}

__global__ void keys_kernel(int64_t n, const double* __restrict__ pos, double ox, double oy,
                            double oz, double inv_h, int L, uint32_t* __restrict__ keys,
                            int* __restrict__ idx) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int top = (1 << L) - 1;
  const double o[3] = {ox, oy, oz};
  uint32_t q[3];
  for (int c = 0; c < 3; ++c) {
    double f = floor((pos[3 * i + c] - o[c]) * inv_h);
    int v = f < 0.0 ? 0 : (f > top ? top : static_cast<int>(f));
    q[c] = static_cast<uint32_t>(v);
  }
  keys[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
  idx[i] = static_cast<int>(i);
}

// ---- stable LSD radix sort, 8-bit digits ------------------------------------------
__global__ void __launch_bounds__(256) radix_hist_kernel(const uint32_t* __restrict__ keys, int n,
                                                         int shift, int nblk,
                                                         int* __restrict__ table) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortItems;
  for (int k = threadIdx.x; k < kSortItems; k += 256) {
    const int i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  table[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) radix_scatter_kernel(
    const uint32_t* __restrict__ keys, const int* __restrict__ idx, int n, int shift, int nblk,
    const int* __restrict__ offs, uint32_t* __restrict__ keys_out, int* __restrict__ idx_out) {
  __shared__ int run[256];
  __shared__ int whist[8][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  run[threadIdx.x] = offs[threadIdx.x * nblk + blockIdx.x];
  const unsigned lt = (1u << lane) - 1u;
  const int base = blockIdx.x * kSortItems;
  for (int it = 0; it < kSortItems / 256; ++it) {
    for (int w = 0; w < 8; ++w) whist[w][threadIdx.x] = 0;
    __syncthreads();
    const int i = base + it * 256 + warp * 32 + lane;
    const bool valid = i < n;
    const uint32_t key = valid ? keys[i] : 0u;
    const int val = valid ? idx[i] : 0;
    const unsigned digit = valid ? ((key >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const int rank = __popc(peers & lt);
    const int leader = 31 - __clz(peers);
    if (valid && lane == leader) whist[warp][digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      int off = run[digit] + rank;
      for (int w = 0; w < warp; ++w) off += whist[w][digit];
      keys_out[off] = key;
      idx_out[off] = val;
    }
    __syncthreads();
    int tot = 0;
    for (int w = 0; w < 8; ++w) tot += whist[w][threadIdx.x];
    run[threadIdx.x] += tot;
    __syncthreads();
  }
}

}  // namespace tree

// Stable LSD radix sort of (key, index) pairs by 32-bit keys, four 8-bit
// passes: the pairs are read from (keys, idx) and returned there, (keys_tmp,
// idx_tmp) hold n each, table sort_table_ints(n) ints, scan_tmp 2 x 2048 ints.
int sort_table_ints(int n) { return 256 * ((n + tree::kSortItems - 1) / tree::kSortItems) * 2; }

// passes: 8-bit digits sorted (an even number: the result is back in (keys, idx))
int sort_pairs_u32(uint32_t* keys, int* idx, uint32_t* keys_tmp, int* idx_tmp, int n, int* table,
                   int* scan_tmp, cudaStream_t s, int passes = 4);
int sort_pairs_u32(uint32_t* keys, int* idx, uint32_t* keys_tmp, int* idx_tmp, int n, int* table,
                   int* scan_tmp, cudaStream_t s, int passes) {
  using namespace tree;
  if (n <= 0) return FVX_OK;
  const int nblk = (n + kSortItems - 1) / kSortItems;
  int* table_ex = table + 256 * nblk;
  uint32_t *ka = keys, *kb = keys_tmp;
  int *ia = idx, *ib = idx_tmp;
  for (int pass = 0; pass < passes; ++pass) {
    radix_hist_kernel<<<nblk, 256, 0, s>>>(ka, n, 8 * pass, nblk, table);
    FVX_LAUNCH_CHECK();
    int rc = scan_ints(table, 256 * nblk, table_ex, 0, scan_tmp, s);
    if (rc) return rc;
    radix_scatter_kernel<<<nblk, 256, 0, s>>>(ka, ia, n, 8 * pass, nblk, table_ex, kb, ib);
    FVX_LAUNCH_CHECK();
    uint32_t* tk = ka;
    ka = kb;
    kb = tk;
    int* ti = ia;
    ia = ib;
    ib = ti;
  }
  return FVX_OK;  // an even number of passes: the result is back in (keys, idx)
}

namespace tree {

// ---- cells ----------------------------------------------------------------------
// flag[i] = 1 where the level key (key >> shift) changes
__global__ void flags_kernel(const uint32_t* __restrict__ keys, const int* __restrict__ n_ptr,
                             int n_cap, int shift, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = n_ptr ? *n_ptr : n_cap;
  if (i >= n_cap) return;
  if (i >= n) {
    flag[i] = 0;
    return;
  }
  flag[i] = (i == 0 || (keys[i] >> shift) != (keys[i - 1] >> shift)) ? 1 : 0;
}

struct Level {
  int* start;     // first sorted particle of each cell
  int* count;     // particles in each cell
  uint32_t* key;  // level key (Morton prefix)
  int* child_lo;  // first child cell (level l+1 local id)
  int* child_hi;  // one past the last child
};

// leaf cells from the particle flags (cid = inclusive scan of flags)
__global__ void leaf_cells_kernel(const uint32_t* __restrict__ keys, int n,
                                  const int* __restrict__ flag, const int* __restrict__ cid,
                                  Level lv, int* __restrict__ n_cells) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cid[i] - 1;
  if (flag[i]) {
    lv.start[c] = i;
    lv.key[c] = keys[i];
  }
  if (i == n - 1) *n_cells = c + 1;
}

__global__ void cell_counts_kernel(Level lv, const int* __restrict__ n_cells, int n_total) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = *n_cells;
  if (c >= nc) return;
  const int end = c + 1 < nc ? lv.start[c + 1] : n_total;
  lv.count[c] = end - lv.start[c];
}

// parent flags over the children cells of level l+1 (keys >> 3)
__global__ void parent_flags_kernel(Level child, const int* __restrict__ n_child, int cap,
                                    int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap) return;
  const int n = *n_child;
  if (i >= n) {
    flag[i] = 0;
    return;
  }
  flag[i] = (i == 0 || (child.key[i] >> 3) != (child.key[i - 1] >> 3)) ? 1 : 0;
}

__global__ void parent_cells_kernel(Level child, const int* __restrict__ n_child,
                                    const int* __restrict__ flag, const int* __restrict__ pid,
                                    Level par, int* __restrict__ n_par) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = *n_child;
  if (i >= n) return;
  const int p = pid[i] - 1;
  if (flag[i]) {
    par.start[p] = child.start[i];
    par.key[p] = child.key[i] >> 3;
    par.child_lo[p] = i;
  }
  if (i == n - 1 || flag[i + 1]) par.child_hi[p] = i + 1;
  if (i == n - 1) *n_par = p + 1;
}

// parent particle count = (last child's end) - (first child's start)
__global__ void parent_counts_kernel(Level child, Level par, const int* __restrict__ n_par) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *n_par) return;
  const int lc = par.child_hi[p] - 1;
  par.count[p] = child.start[lc] + child.count[lc] - par.start[p];
}

// ---- sorted particle records -----------------------------------------------------
struct Grid {
  double ox, oy, oz, h;
  int L;
};

__device__ __forceinline__ void cell_center(uint32_t key, double hl, const Grid& g, double c[3]) {
  c[0] = g.ox + (static_cast<double>(compact10(key)) + 0.5) * hl;
  c[1] = g.oy + (static_cast<double>(compact10(key >> 1)) + 0.5) * hl;
  c[2] = g.oz + (static_cast<double>(compact10(key >> 2)) + 0.5) * hl;
}
// centre relative to the grid origin (exact in FP32)
__device__ __forceinline__ float3 cell_center_rel(uint32_t key, float hl) {
  return make_float3((static_cast<float>(compact10(key)) + 0.5f) * hl,
                     (static_cast<float>(compact10(key >> 1)) + 0.5f) * hl,
                     (static_cast<float>(compact10(key >> 2)) + 0.5f) * hl);
}

template <int KERNEL>
__global__ void gather_kernel(int n, const int* __restrict__ perm, const int* __restrict__ leaf_of,
                              const uint32_t* __restrict__ leaf_key, Grid g,
                              const double* __restrict__ pos, const double* __restrict__ alpha,
                              const double* __restrict__ sigma, const double* __restrict__ tgam,
                              float4* __restrict__ sp, float4* __restrict__ sa,
                              float4* __restrict__ sg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = perm[i];
  const int leaf = leaf_of[i] - 1;
  double c[3];
  cell_center(leaf_key[leaf], g.h, g, c);
  const double s = sigma[j];
  sp[i] = make_float4(static_cast<float>(pos[3 * j] - c[0]), static_cast<float>(pos[3 * j + 1] - c[1]),
                      static_cast<float>(pos[3 * j + 2] - c[2]), static_cast<float>(s * s));
  sa[i] = make_float4(static_cast<float>(kC * alpha[3 * j]), static_cast<float>(kC * alpha[3 * j + 1]),
                      static_cast<float>(kC * alpha[3 * j + 2]),
                      static_cast<float>(KERNEL == FVX_KERNEL_WINCKELMANS ? 2.5 * s * s : 1.0 / s));
  if (tgam)
    sg[i] = make_float4(static_cast<float>(tgam[3 * j]), static_cast<float>(tgam[3 * j + 1]),
                        static_cast<float>(tgam[3 * j + 2]), 0.f);
}

// ---- moments ----------------------------------------------------------------------
// record: [cx cy cz h | M0(3) t(3) | M1(9) | M2 (3 x 6 unique: xx xy xz yy yz zz) | pad 2]
__device__ __forceinline__ int m2i(int j, int k) {
  // unique index of the symmetric pair (j, k)
  const int a = j < k ? j : k, b = j < k ? k : j;
  return a == 0 ? b : (a == 1 ? 2 + b : 5);
}

// one warp per leaf, moments of the C-scaled strengths about the leaf centre
__global__ void leaf_moments_kernel(Level lv, const int* __restrict__ n_leaves, float hl,
                                    const float4* __restrict__ sp, const float4* __restrict__ sa,
                                    float* __restrict__ rec) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= *n_leaves) return;
  float m[30];
#pragma unroll
  for (int q = 0; q < 30; ++q) m[q] = 0.f;
  const int s = lv.start[warp], e = s + lv.count[warp];
  for (int i = s + lane; i < e; i += 32) {
    const float4 p = sp[i];
    const float4 a = sa[i];
    const float d[3] = {p.x, p.y, p.z}, al[3] = {a.x, a.y, a.z};
#pragma unroll
    for (int mm = 0; mm < 3; ++mm) {
      m[mm] += al[mm];
#pragma unroll
      for (int j = 0; j < 3; ++j) m[3 + 3 * mm + j] += al[mm] * d[j];
      m[12 + 6 * mm + 0] += al[mm] * d[0] * d[0];
      m[12 + 6 * mm + 1] += al[mm] * d[0] * d[1];
      m[12 + 6 * mm + 2] += al[mm] * d[0] * d[2];
      m[12 + 6 * mm + 3] += al[mm] * d[1] * d[1];
      m[12 + 6 * mm + 4] += al[mm] * d[1] * d[2];
      m[12 + 6 * mm + 5] += al[mm] * d[2] * d[2];
    }
  }
#pragma unroll
  for (int q = 0; q < 30; ++q)
    for (int o = 16; o > 0; o >>= 1) m[q] += __shfl_xor_sync(0xffffffffu, m[q], o);
  if (lane == 0) {
    float* r = rec + static_cast<int64_t>(warp) * kRecFloats;
    const float3 c = cell_center_rel(lv.key[warp], hl);
    r[0] = c.x;
    r[1] = c.y;
    r[2] = c.z;
    r[3] = hl;
    for (int mm = 0; mm < 3; ++mm) {
      r[4 + mm] = m[mm];
      r[7 + mm] = m[12 + 6 * mm + 0] + m[12 + 6 * mm + 3] + m[12 + 6 * mm + 5];  // trace
    }
    for (int q = 0; q < 9; ++q) r[10 + q] = m[3 + q];
    for (int q = 0; q < 18; ++q) r[19 + q] = m[12 + q];
    r[37] = r[38] = r[39] = 0.f;
  }
}

// parent moments from children (shift by s = c_child - c_parent, exact)
__global__ void m2m_kernel(Level par, const int* __restrict__ n_par, float hl,
                           const float* __restrict__ child_rec, float* __restrict__ par_rec) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= *n_par) return;
  const float3 cp = cell_center_rel(par.key[p], hl);
  float M0[3] = {0, 0, 0}, M1[9], M2[18];
  for (int q = 0; q < 9; ++q) M1[q] = 0.f;
  for (int q = 0; q < 18; ++q) M2[q] = 0.f;
  for (int c = par.child_lo[p]; c < par.child_hi[p]; ++c) {
    const float* r = child_rec + static_cast<int64_t>(c) * kRecFloats;
    const float s[3] = {r[0] - cp.x, r[1] - cp.y, r[2] - cp.z};
    for (int m = 0; m < 3; ++m) {
      const float m0 = r[4 + m];
      M0[m] += m0;
      for (int j = 0; j < 3; ++j) M1[3 * m + j] += r[10 + 3 * m + j] + m0 * s[j];
      for (int j = 0; j < 3; ++j)
        for (int k = j; k < 3; ++k) {
          const int u = m2i(j, k);
          M2[6 * m + u] += r[19 + 6 * m + u] + r[10 + 3 * m + j] * s[k] +
                           r[10 + 3 * m + k] * s[j] + m0 * s[j] * s[k];
        }
    }
  }
  float* r = par_rec + static_cast<int64_t>(p) * kRecFloats;
  r[0] = cp.x;
  r[1] = cp.y;
  r[2] = cp.z;
  r[3] = hl;
  for (int m = 0; m < 3; ++m) {
    r[4 + m] = M0[m];
    r[7 + m] = M2[6 * m + 0] + M2[6 * m + 3] + M2[6 * m + 5];
  }
  for (int q = 0; q < 9; ++q) r[10 + q] = M1[q];
  for (int q = 0; q < 18; ++q) r[19 + q] = M2[q];
  r[37] = r[38] = r[39] = 0.f;
}

// ---- interaction lists --------------------------------------------------------------
struct TreeView {
  int L;
  double h;          // leaf size
  double mac_k;      // 3/4 / theta^2
  int base[11];      // global id of the first cell of each level
  int ncell[11];     // cells per level (device copy below)
  const int* start;  // global cell arrays (concatenated levels)
  const int* count;
  const uint32_t* key;
  const int* child_lo;  // level-local ids of the children (level l+1)
  const int* child_hi;
  const int4* cen;      // cell centres in units of h/2 (dual traversal)
  double mac_kl;        // learned far field: 3/4 / theta_L^2 (0: off)
  int learned_only;     // learned pairs leave the analytic list (weights loaded)
  // the acceptance tests in exact integers: with centre offsets in units of
  // h/2, a level-l cell is accepted when d2 > thr_far[l] (= floor of
  // mac_k (h_T + h_S)^2 in those units) and listed for the local-expansion
  // path when d2 > thr_lrn[l]
  int thr_far[11];
  int thr_lrn[11];
  int thr_par[11];  // the same test for a parent of leaves (size 2h) as the target
};

// (target leaf, source cell) pairs handed to the learned far-field operator
struct LearnedLists {
  int* cnt;
  const int* off;
  int* leaf;
  int* cell;
  int cap;
};

template <bool FILL>
__global__ void traverse_kernel(TreeView T, const int* __restrict__ near_off,
                                const int* __restrict__ far_off, int* __restrict__ near_cnt,
                                int* __restrict__ far_cnt, int* __restrict__ near_idx,
                                int* __restrict__ far_idx, int near_cap, int far_cap,
                                unsigned* __restrict__ overflow, LearnedLists LL) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nleaf = T.ncell[T.L];
  if (t >= nleaf) return;
  const int gT = T.base[T.L] + t;
  const uint32_t kT = T.key[gT];
  // centre of T in units of h/2 (exact integers below 2^11)
  const int tx = 2 * static_cast<int>(compact10(kT)) + 1,
            ty = 2 * static_cast<int>(compact10(kT >> 1)) + 1,
            tz = 2 * static_cast<int>(compact10(kT >> 2)) + 1;
  // stack entries: global cell id | level << 27
  int stack[96];
  int sp = 0;
  for (int c = T.ncell[0] - 1; c >= 0; --c) stack[sp++] = T.base[0] + c;
  int nn = 0, nf = 0, nl = 0;
  const int lo0 = (FILL && LL.off) ? LL.off[t] : 0;
  long long near_pairs = 0;
  const int cT_count = T.count[gT];
  int no = FILL ? near_off[t] : 0, fo = FILL ? far_off[t] : 0;
  while (sp > 0) {
    const int e = stack[--sp];
    const int g = e & ((1 << 27) - 1), l = e >> 27;
    const uint32_t k = T.key[g];
    const int sc = 1 << (T.L - l);  // cell size in units of h
    const int dx = tx - (2 * static_cast<int>(compact10(k)) + 1) * sc;
    const int dy = ty - (2 * static_cast<int>(compact10(k >> 1)) + 1) * sc;
    const int dz = tz - (2 * static_cast<int>(compact10(k >> 2)) + 1) * sc;
    const int d2 = dx * dx + dy * dy + dz * dz;
    if (d2 > T.thr_far[l]) {
      const bool lrn = d2 > T.thr_lrn[l];
      if (lrn) {
        if (FILL && LL.leaf && lo0 + nl < LL.cap) {
          LL.leaf[lo0 + nl] = t;
          LL.cell[lo0 + nl] = g;
        }
        ++nl;
      }
      if (!lrn || !T.learned_only) {
        if (FILL && fo + nf < far_cap) far_idx[fo + nf] = g;
        ++nf;
      }
    } else if (l == T.L) {
      if (FILL && no + nn < near_cap) near_idx[no + nn] = g - T.base[T.L];
      near_pairs += static_cast<long long>(cT_count) * T.count[g];
      ++nn;
    } else {
      const int lo = T.child_lo[g], hi = T.child_hi[g];
      for (int c = hi - 1; c >= lo; --c) {
        if (sp < 96) {
          stack[sp++] = (T.base[l + 1] + c) | ((l + 1) << 27);
        } else {
          atomicOr(overflow, 1u);
        }
      }
    }
  }
  if (!FILL) {
    near_cnt[t] = nn;
    far_cnt[t] = nf;
    if (LL.cnt) LL.cnt[t] = nl;
  } else {
    if (no + nn > near_cap || fo + nf > far_cap) atomicOr(overflow, 2u);
    // work counters: near particle pairs, far (target particle, cell) pairs
    unsigned long long* work = reinterpret_cast<unsigned long long*>(overflow + 2);
    atomicAdd(work, static_cast<unsigned long long>(near_pairs));
    atomicAdd(work + 1, static_cast<unsigned long long>(cT_count) * nf);
  }
}

// ---- two-level (dual) traversal for the local-expansion far field -------------------
// The source cells A are tested against the parent P of each leaf T (level
// L-1) first: A is accepted for the whole parent when the test passes for P
// (one local expansion about c_P, shared by P's leaves); a failing A larger
// than P is accepted by T itself when it passes for every possible child of P
// (the nearest octant), and opened otherwise; a failing A of P's size or a
// leaf is then tested against T, which accepts A (local pair), or -- A being a
// leaf -- keeps it as a near leaf, or accepts / keeps near each of A's children.  This is the dual-tree
// rule "split the larger cell" on (P, A) then (T, A): every source particle
// reaches every leaf exactly once, through P's expansion, T's own expansions
// or T's near list.  One thread per leaf (the parent-level decisions depend on
// P only, so siblings take them identically); the first child of each parent
// writes the parent's pairs.
struct DualLists {
  int* near_cnt;     // per leaf
  int* lrn_cnt;      // per leaf: (leaf, cell) local pairs
  int* par_cnt;      // per parent: (parent, cell) local pairs
  const int* near_off;
  const int* lrn_off;
  const int* par_off;
  int* near_idx;
  int* lrn_leaf;
  int* lrn_cell;
  int* par_par;
  int* par_cell;
  const int* leaf_parent;  // per leaf: its parent's level-local index
  int near_cap, lrn_cap, par_cap;
  // slot mode (fill pass with these > 0): leaf t's near leaves at
  // near_idx[t slot_near ..], its local cells at lrn_cell[t slot_lrn ..],
  // parent p's cells at par_cell[p slot_par ..]; the counts are written and
  // an overflow of a slot sets overflow bit 4 (lrn_leaf, par_par unused)
  int slot_near, slot_lrn, slot_par;
};

// Cell centres (2 c + 1) 2^(L - l) in units of h/2, c the level-l cell's
// integer coordinates, and the children's level-local range packed as
// (first << 4) | count (0 for leaves): what the dual traversal reads per
// visited cell, in one 16-byte load instead of a key to decode and the
// child bounds.
__global__ void cell_centres_kernel(TreeView T, int total_cells, int4* __restrict__ cen) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_cells) return;
  int l = 0;
  while (l < T.L && g >= T.base[l + 1]) ++l;
  if (g - T.base[l] >= T.ncell[l]) return;  // a level's unused capacity
  const uint32_t k = T.key[g];
  const int sc = 1 << (T.L - l);
  const int kids = l < T.L ? (T.child_lo[g] << 4) | (T.child_hi[g] - T.child_lo[g]) : 0;
  cen[g] = make_int4((2 * static_cast<int>(compact10(k)) + 1) * sc,
                     (2 * static_cast<int>(compact10(k >> 1)) + 1) * sc,
                     (2 * static_cast<int>(compact10(k >> 2)) + 1) * sc, kids);
}

// Sort keys of the evaluation order: leaves by decreasing near-field work
// (near leaves x own particles, 16 bits), ties in leaf order.
__global__ void order_keys_kernel(int nleaf, const int* __restrict__ near_cnt,
                                  const int* __restrict__ leaf_count, uint32_t* __restrict__ keys,
                                  int* __restrict__ idx) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nleaf) return;
  const long long w = static_cast<long long>(near_cnt[t]) * leaf_count[t];
  keys[t] = 0xFFFFu - static_cast<uint32_t>(w < 0xFFFF ? w : 0xFFFF);
  idx[t] = t;
}

// leaf -> its parent's level-local index, from the parents' child ranges
__global__ void leaf_parents_kernel(TreeView T, int* __restrict__ leaf_parent) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T.ncell[T.L - 1]) return;
  const int gP = T.base[T.L - 1] + p;
  for (int c = T.child_lo[gP]; c < T.child_hi[gP]; ++c) leaf_parent[c] = p;
}

template <bool FILL>
__global__ void traverse_dual_kernel(TreeView T, DualLists D, unsigned* __restrict__ overflow) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = T.L;
  const int nleaf = T.ncell[L];
  if (t >= nleaf) return;
  const int gT = T.base[L] + t;
  const int p = D.leaf_parent[t];
  const int gP = T.base[L - 1] + p;
  const bool first = T.child_lo[gP] == t;
  // centres in units of h/2: a parent (size 2h) at (2 k + 1) 2, a leaf at 2 k + 1
  const int4 cP = T.cen[gP], cT = T.cen[gT];
  const int px = cP.x, py = cP.y, pz = cP.z;
  const int tx = cT.x, ty = cT.y, tz = cT.z;
  const int tcount = T.count[gT];
  int nn = 0, nl = 0, np = 0;
  const bool slot = FILL && D.slot_near > 0;
  const int no = FILL ? (slot ? t * D.slot_near : D.near_off[t]) : 0;
  const int lo_ = FILL ? (slot ? t * D.slot_lrn : D.lrn_off[t]) : 0;
  const int po = (FILL && first) ? (slot ? p * D.slot_par : D.par_off[p]) : 0;
  const int near_end = slot ? no + D.slot_near : D.near_cap;
  const int lrn_end = slot ? lo_ + D.slot_lrn : D.lrn_cap;
  const int par_end = slot ? po + D.slot_par : D.par_cap;
  long long near_pairs = 0;
  // T against source cell g at level l; false: an inner cell that fails
  auto leaf_visit = [&](int g, int l) {
    const int4 c = T.cen[g];
    const int dx = tx - c.x, dy = ty - c.y, dz = tz - c.z;
    const int d2 = dx * dx + dy * dy + dz * dz;
    if (d2 > T.thr_far[l]) {
      if (FILL && lo_ + nl < lrn_end) {
        if (!slot) D.lrn_leaf[lo_ + nl] = t;
        D.lrn_cell[lo_ + nl] = g;
      }
      ++nl;
      return true;
    }
    if (l == L) {
      if (FILL && no + nn < near_end) D.near_idx[no + nn] = g - T.base[L];
      near_pairs += static_cast<long long>(tcount) * T.count[g];
      ++nn;
      return true;
    }
    return false;
  };
  int stack[96];
  int sp = 0;
  for (int c = T.ncell[0] - 1; c >= 0; --c) stack[sp++] = T.base[0] + c;
  while (sp > 0) {
    const int e = stack[--sp];
    const int g = e & ((1 << 27) - 1), l = e >> 27;
    const int4 c = T.cen[g];
    const int dx = px - c.x, dy = py - c.y, dz = pz - c.z;
    const int d2 = dx * dx + dy * dy + dz * dz;
    if (d2 > T.thr_par[l]) {
      if (first) {
        if (FILL && po + np < par_end) {
          if (!slot) D.par_par[po + np] = p;
          D.par_cell[po + np] = g;
        }
        ++np;
      }
      continue;
    }
    if (l < L - 1) {
      // accepted by every child of P (the octant of P nearest to A passes the
      // leaf test; the decision depends on P and A only): a pair of T's own,
      // as the per-leaf traversal would make it; otherwise A is opened
      const int ax = abs(dx) - 1, ay = abs(dy) - 1, az = abs(dz) - 1;
      if (ax * ax + ay * ay + az * az > T.thr_far[l]) {
        leaf_visit(g, l);
        continue;
      }
      const int clo = c.w >> 4, chi = clo + (c.w & 15);
      for (int q = chi - 1; q >= clo; --q) {
        if (sp < 96)
          stack[sp++] = (T.base[l + 1] + q) | ((l + 1) << 27);
        else
          atomicOr(overflow, 1u);
      }
      continue;
    }
    // A of P's size (level L-1) or a leaf: against T itself
    if (leaf_visit(g, l)) continue;
    const int clo = c.w >> 4, chi = clo + (c.w & 15);  // A at level L-1: leaves below
    for (int q = clo; q < chi; ++q) leaf_visit(T.base[L] + q, L);
  }
  if (!FILL || slot) {
    D.near_cnt[t] = nn;
    D.lrn_cnt[t] = nl;
    if (first) D.par_cnt[p] = np;
  }
  if (FILL) {
    if (no + nn > near_end || lo_ + nl > lrn_end || (first && po + np > par_end))
      atomicOr(overflow, slot ? 4u : 2u);
    unsigned long long* work = reinterpret_cast<unsigned long long*>(overflow + 2);
    atomicAdd(work, static_cast<unsigned long long>(near_pairs));
  }
}

// ---- one-pass two-level lists in two phases --------------------------------------
// The per-leaf traversal above tests every cell against the leaf's parent
// first; the eight siblings repeat those tests.  Here the parent-level walk
// runs once per parent, by a warp (phase 1), and leaves only the residual
// cells to each child leaf (phase 2).  The lists are the same sets as the
// per-leaf traversal's (the parent list of the parent, near leaves and local
// cells of each leaf); their order within a leaf or parent differs.
constexpr int kParWarps = 4;     // phase 1: warps (parents) per CTA
constexpr int kParStack = 2048;  // phase 1: stack entries per warp (shared memory)

// Phase 1: warp per parent of leaves P.  A shared stack is walked 32 entries
// per round (lane 0 takes the top).  A cell that P accepts goes to P's list;
// a cell accepted by every child of P (the octant test of the per-leaf
// traversal), or a leaf- or parent-level cell that P does not accept, goes to
// P's residual list; any other cell is opened.  Any capacity overflow sets
// overflow bit 4 (the host then builds the lists with the counting passes).
__global__ void __launch_bounds__(kParWarps * 32) traverse_parents_kernel(
    TreeView T, int* __restrict__ par_cnt, int* __restrict__ par_cell, int slot_par,
    int* __restrict__ res_cnt, int* __restrict__ res, int slot_res,
    unsigned* __restrict__ overflow) {
  __shared__ int s_stack[kParWarps][kParStack];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = T.L;
  const int p = blockIdx.x * kParWarps + w;
  if (p >= T.ncell[L - 1]) return;  // whole warps
  int* st = s_stack[w];
  const int4 cP = T.cen[T.base[L - 1] + p];
  const unsigned below = (1u << lane) - 1u;
  const int nroot = T.ncell[0];
  bool bad = nroot > kParStack;
  int sp = 0;
  if (!bad) {
    for (int i = lane; i < nroot; i += 32) st[nroot - 1 - i] = T.base[0] + i;  // root 0 on top
    sp = nroot;
  }
  __syncwarp();
  int np = 0, nr = 0;
  while (sp > 0 && !bad) {
    const int n = sp < 32 ? sp : 32;
    const int e = lane < n ? st[sp - 1 - lane] : -1;
    sp -= n;
    __syncwarp();
    int cat = 0, kids = 0;  // 1: parent list, 2: residual, 3: open
    if (e >= 0) {
      const int g = e & ((1 << 27) - 1), l = e >> 27;
      const int4 c = T.cen[g];
      const int dx = cP.x - c.x, dy = cP.y - c.y, dz = cP.z - c.z;
      const int d2 = dx * dx + dy * dy + dz * dz;
      if (d2 > T.thr_par[l]) {
        cat = 1;
      } else if (l < L - 1) {
        const int ax = abs(dx) - 1, ay = abs(dy) - 1, az = abs(dz) - 1;
        if (ax * ax + ay * ay + az * az > T.thr_far[l]) {
          cat = 2;
        } else {
          cat = 3;
          kids = c.w;
        }
      } else {
        cat = 2;
      }
    }
    const unsigned m1 = __ballot_sync(full, cat == 1);
    if (cat == 1) {
      const int k = np + __popc(m1 & below);
      if (k < slot_par) par_cell[static_cast<int64_t>(p) * slot_par + k] = e & ((1 << 27) - 1);
    }
    np += __popc(m1);
    const unsigned m2 = __ballot_sync(full, cat == 2);
    if (cat == 2) {
      const int k = nr + __popc(m2 & below);
      if (k < slot_res) res[static_cast<int64_t>(p) * slot_res + k] = e;
    }
    nr += __popc(m2);
    // children: lower lanes' nearer the top, child 0 of a cell on top
    const int cnt = cat == 3 ? (kids & 15) : 0;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(full, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(full, incl, 31);
    if (sp + total > kParStack) {
      bad = true;
    } else {
      if (cnt > 0) {
        const int l1 = (e >> 27) + 1, clo = kids >> 4;
        const int top = sp + total - incl + cnt - 1;  // this lane's highest slot
        for (int q = 0; q < cnt; ++q) st[top - q] = (T.base[l1] + clo + q) | (l1 << 27);
      }
      sp += total;
    }
    __syncwarp();
  }
  if (lane == 0) {
    par_cnt[p] = np;
    res_cnt[p] = nr;
    if (bad || np > slot_par || nr > slot_res) atomicOr(overflow, 4u);
  }
}

// Phase 2: warp per parent P: P's residual cells finished against each of its
// child leaves.  Lanes take 32 residual cells at a time (their records, and
// for a parent-level cell its leaves' records, loaded once for all children);
// per child leaf, the accepted cells become local-expansion pairs and the
// leaf-level ones near leaves, emitted in lane order (ballot prefixes).
__global__ void __launch_bounds__(kParWarps * 32) traverse_residual_kernel(
    TreeView T, DualLists D, const int* __restrict__ res_cnt, const int* __restrict__ res,
    int slot_res, unsigned* __restrict__ overflow) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = T.L;
  const int p = blockIdx.x * kParWarps + w;
  if (p >= T.ncell[L - 1]) return;  // whole warps
  const unsigned below = (1u << lane) - 1u;
  const int kidsP = T.cen[T.base[L - 1] + p].w;
  const int t0 = kidsP >> 4, nkP = kidsP & 15;  // the child leaves t0 .. t0 + nkP - 1
  int4 cL[8];
  int tc[8], nn[8], nl[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    nn[q] = nl[q] = 0;
    tc[q] = 0;
    cL[q] = make_int4(0, 0, 0, 0);
    if (q < nkP) {
      cL[q] = T.cen[T.base[L] + t0 + q];
      tc[q] = T.count[T.base[L] + t0 + q];
    }
  }
  long long near_pairs = 0;
  const int nr = min(res_cnt[p], slot_res);
  const int* rp = res + static_cast<int64_t>(p) * slot_res;
  // emit the lanes' flagged cells g into child q's list (lrn or near)
  auto emit = [&](int q, bool lrn, bool near, int g) {
    const unsigned ml = __ballot_sync(full, lrn), mn = __ballot_sync(full, near);
    const int t = t0 + q;
    if (lrn) {
      const int k = nl[q] + __popc(ml & below);
      if (k < D.slot_lrn) D.lrn_cell[static_cast<int64_t>(t) * D.slot_lrn + k] = g;
    }
    if (near) {
      const int k = nn[q] + __popc(mn & below);
      if (k < D.slot_near) D.near_idx[static_cast<int64_t>(t) * D.slot_near + k] = g - T.base[L];
      near_pairs += static_cast<long long>(tc[q]) * T.count[g];
    }
    nl[q] += __popc(ml);
    nn[q] += __popc(mn);
  };
  for (int i0 = 0; i0 < nr; i0 += 32) {
    const int e = i0 + lane < nr ? rp[i0 + lane] : -1;
    const int g = e & ((1 << 27) - 1), l = e >> 27;
    int4 c = make_int4(0, 0, 0, 0);
    if (e >= 0) c = T.cen[g];
    // a parent-level cell's leaves
    const int nk = (e >= 0 && l == L - 1) ? (c.w & 15) : 0, clo = c.w >> 4;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q >= nkP) break;  // uniform
      bool acc = false, near = false, expand = false;
      if (e >= 0) {
        const int dx = cL[q].x - c.x, dy = cL[q].y - c.y, dz = cL[q].z - c.z;
        const int d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > T.thr_far[l])
          acc = true;  // (for l < L - 1 always: accepted for every child of P)
        else if (l == L)
          near = true;
        else if (l == L - 1)
          expand = true;
      }
      emit(q, acc, near, g);
      // parent-level cells that leaf q does not accept: their leaves, four
      // cells per pass (eight lanes each), in lane order then child order
      unsigned mexp = __ballot_sync(full, expand);
      while (mexp) {
        // this lane's cell: the (lane / 8)-th set bit of mexp
        unsigned m = mexp;
        for (int r = 0; r < (lane >> 3); ++r) m &= m - 1;
        const int src = m ? __ffs(m) - 1 : 32;
        const int sl = src < 32 ? src : 0, ch = lane & 7;
        const int sclo = __shfl_sync(full, clo, sl), snk = __shfl_sync(full, nk, sl);
        bool a2 = false, n2 = false;
        int gl = 0;
        if (src < 32 && ch < snk) {
          gl = T.base[L] + sclo + ch;
          const int4 c2 = T.cen[gl];
          const int dx = cL[q].x - c2.x, dy = cL[q].y - c2.y, dz = cL[q].z - c2.z;
          a2 = dx * dx + dy * dy + dz * dz > T.thr_far[L];
          n2 = !a2;
        }
        emit(q, a2, n2, gl);
#pragma unroll
        for (int r = 0; r < 4; ++r) mexp &= mexp - 1;  // the four cells done
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (q < nkP && lane == 0) {
      const int t = t0 + q;
      D.near_cnt[t] = nn[q];
      D.lrn_cnt[t] = nl[q];
      if (nn[q] > D.slot_near || nl[q] > D.slot_lrn) atomicOr(overflow, 4u);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) near_pairs += __shfl_xor_sync(full, near_pairs, o);
  if (lane == 0) {
    unsigned long long* work = reinterpret_cast<unsigned long long*>(overflow + 2);
    atomicAdd(work, static_cast<unsigned long long>(near_pairs));
  }
}

// slot-mode lists -> flat (target, cell) pair lists ordered by target: warp
// per target, lanes over its slot; off = the exclusive scan of the counts
__global__ void compact_slots_kernel(int ntgt, int cap, const int* __restrict__ cnt,
                                     const int* __restrict__ off, const int* __restrict__ slots,
                                     int* __restrict__ tgt, int* __restrict__ cell) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ntgt) return;
  const int c = cnt[w], o = off[w];
  for (int q = lane; q < c; q += 32) {
    tgt[o + q] = w;
    cell[o + q] = slots[static_cast<int64_t>(w) * cap + q];
  }
}

__global__ void iota_scaled_kernel(int n, int step, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i * step;
}

// ---- evaluation -----------------------------------------------------------------------
struct EvalArgs {
  float h;  // leaf size
  const int* leaf_start;
  const int* leaf_count;
  const uint32_t* leaf_key;
  const int* near_off;
  const int* near_cnt;
  const int* near_idx;
  const int* far_off;
  const int* far_cnt;
  const int* far_idx;
  const float* rec;  // global cell records
  const float4* sp;
  const float4* sa;
  const float4* sg;
  const int* perm;
  double* out_a;
  double* out_b;
  const float* leaf_local;  // [leaves][32] learned local expansions, or null
  const float* parent_local;  // [parents][32] expansions shared by a parent's leaves, or null
  const int* leaf_parent;     // parent index of each leaf (with parent_local)
  int nleaf;
  int* leaf_next;             // leaf counter of the resident evaluation warps (zeroed)
  const int* leaf_order;      // the order the warps take the leaves in
};

// Learned local expansion of the leaf at offset d = x - c_T (u, J = du/dx,
// H_i,kn = d2 u_i / dx_k dx_n with 6 unique (k, n) per component).
template <int MODE>
__device__ __forceinline__ void l2p(float* acc, const float* L, float dx, float dy, float dz,
                                    float gx, float gy, float gz) {
  const float d[3] = {dx, dy, dz};
  float J[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float* Hi = L + 12 + 6 * i;  // xx xy xz yy yz zz
    const float Hm[3][3] = {{Hi[0], Hi[1], Hi[2]}, {Hi[1], Hi[3], Hi[4]}, {Hi[2], Hi[4], Hi[5]}};
#pragma unroll
    for (int n = 0; n < 3; ++n)
      J[i][n] = L[3 + 3 * i + n] + Hm[n][0] * d[0] + Hm[n][1] * d[1] + Hm[n][2] * d[2];
    if (MODE == FVX_PAIR_VELOCITY || MODE == FVX_PAIR_VELOCITY_STRETCH) {
      // u_i = L_i + J0_in d_n + 1/2 d H_i d = L_i + 1/2 (J0_in + J_in) d_n
      float u = L[i];
#pragma unroll
      for (int n = 0; n < 3; ++n) u += 0.5f * (L[3 + 3 * i + n] + J[i][n]) * d[n];
      acc[i] += u;
    }
  }
  if (MODE == FVX_PAIR_STRETCH || MODE == FVX_PAIR_VELOCITY_STRETCH) {
    constexpr int o = MODE == FVX_PAIR_STRETCH ? 0 : 3;
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[o + i] += J[i][0] * gx + J[i][1] * gy + J[i][2] * gz;
  }
  if (MODE == FVX_PAIR_VORTICITY) {
    acc[0] += J[2][1] - J[1][2];
    acc[1] += J[0][2] - J[2][0];
    acc[2] += J[1][0] - J[0][1];
  }
}

template <typename T>
__device__ __forceinline__ void fold(T& hi, T& lo, T p) {
  T s = hi + p;
  T bp = s - hi;
  T err = (hi - (s - bp)) + (p - bp);
  hi = s;
  lo += err;
}

// Far field of one cell record R at offset r = x - c (moments of C-scaled
// strengths; see the derivation in oracle/treecode.py): adds to acc.
template <int MODE>
__device__ __forceinline__ void m2p(float* acc, const float* R, float rx, float ry, float rz,
                                    float gx, float gy, float gz) {
  const float r[3] = {rx, ry, rz};
  const float r2 = rx * rx + ry * ry + rz * rz;
  const float ir = rsqrtf(r2);
  const float ir2 = ir * ir;
  const float ir3 = ir * ir2, ir5 = ir3 * ir2, ir7 = ir5 * ir2;
  const float* M0 = R + 4;
  const float* tr = R + 7;
  const float* M1 = R + 10;
  const float* M2 = R + 19;
  float a[3], w[3][3], q[3], s[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    a[m] = M1[3 * m] * rx + M1[3 * m + 1] * ry + M1[3 * m + 2] * rz;
    const float* Q = M2 + 6 * m;  // xx xy xz yy yz zz
    w[m][0] = Q[0] * rx + Q[1] * ry + Q[2] * rz;
    w[m][1] = Q[1] * rx + Q[3] * ry + Q[4] * rz;
    w[m][2] = Q[2] * rx + Q[4] * ry + Q[5] * rz;
    q[m] = w[m][0] * rx + w[m][1] * ry + w[m][2] * rz;
    s[m] = -M0[m] * ir3 - 3.f * ir5 * a[m] - 7.5f * ir7 * q[m] + 1.5f * ir5 * tr[m];
  }
  if (MODE == FVX_PAIR_VELOCITY || MODE == FVX_PAIR_VELOCITY_STRETCH) {
    float X[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int j = 0; j < 3; ++j) X[m][j] = s[m] * r[j] + ir3 * M1[3 * m + j] + 3.f * ir5 * w[m][j];
    acc[0] += X[1][2] - X[2][1];
    acc[1] += X[2][0] - X[0][2];
    acc[2] += X[0][1] - X[1][0];
  }
  if (MODE == FVX_PAIR_STRETCH || MODE == FVX_PAIR_VELOCITY_STRETCH ||
      MODE == FVX_PAIR_VORTICITY) {
    const float ir9 = ir7 * ir2;
    float P[3], V[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      P[m] = 3.f * M0[m] * ir5 + 15.f * ir7 * a[m] + 52.5f * ir9 * q[m] - 7.5f * ir7 * tr[m];
#pragma unroll
      for (int n = 0; n < 3; ++n) V[m][n] = 3.f * ir5 * M1[3 * m + n] + 15.f * ir7 * w[m][n];
    }
    if (MODE == FVX_PAIR_VORTICITY) {
      const float rP = rx * P[0] + ry * P[1] + rz * P[2];
      const float trV = V[0][0] + V[1][1] + V[2][2];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float Vr = V[0][i] * rx + V[1][i] * ry + V[2][i] * rz;
        // sum_j M2_j(i,j)
        const float m2 = M2[6 * 0 + m2i(i, 0)] + M2[6 * 1 + m2i(i, 1)] + M2[6 * 2 + m2i(i, 2)];
        acc[i] -= r[i] * rP + s[i] - Vr - r[i] * trV + 3.f * ir5 * m2;
      }
    } else {
      constexpr int o = MODE == FVX_PAIR_STRETCH ? 0 : 3;
      const float g[3] = {gx, gy, gz};
      const float rG = rx * gx + ry * gy + rz * gz;
      float hm[3][3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const float VG = V[m][0] * gx + V[m][1] * gy + V[m][2] * gz;
        const float* Q = M2 + 6 * m;
        const float MG[3] = {Q[0] * gx + Q[1] * gy + Q[2] * gz, Q[1] * gx + Q[3] * gy + Q[4] * gz,
                             Q[2] * gx + Q[4] * gy + Q[5] * gz};
#pragma unroll
        for (int j = 0; j < 3; ++j)
          hm[m][j] = rG * r[j] * P[m] + g[j] * s[m] - (VG * r[j] + V[m][j] * rG) +
                     3.f * ir5 * MG[j];
      }
      acc[o + 0] -= hm[2][1] - hm[1][2];
      acc[o + 1] -= hm[0][2] - hm[2][0];
      acc[o + 2] -= hm[1][0] - hm[0][1];
    }
  }
}

// ---- paired FP32 (f32x2) arithmetic: two targets per instruction -------------
namespace x2 {
__device__ __forceinline__ uint64_t pack(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ uint64_t dup(float a) { return pack(a, a); }
__device__ __forceinline__ void unpack(uint64_t v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
}  // namespace x2

// The packed near tile: kNearTile staged sources, one per row, in planes of
// 16-byte words (plane w of row k at w * kNearTile + k), so that a warp
// staging consecutive rows writes consecutive words without bank conflicts:
//   direct:   {-x, -y, -z, s2}, {c1, ax, ay, az}
//   factored: {x, y, z, S},     {c1, ax, ay, az}, {cx, cy, cz, 0}
// with c1 = 1.5 s2, x_s = (x, y, z) the source relative to the target leaf's
// centre, S = |x_s|^2 + s2 and c = x_s x a.  Each lane holds two targets in
// the halves of its paired registers and reads one row per step, duplicating
// each value into both halves: a broadcast 16-byte load costs the
// shared-memory pipe two wavefronts, so one source for two targets per load
// takes half the wavefronts of two sources for one target.
constexpr int kPlanes = 3;

// Near pairs of one staged tile (rows grp, grp + g, ... : nit of them) for the
// thread's two targets (Winckelmans core, velocity or stretching) in paired
// FP32 arithmetic.  With q = r^2 + s^2, t = q^-1/2 and u = 1.5 s^2 t^2,
//   f   = (r^2 + 2.5 s^2) t^5  = t^3 (1 + u),
//   fpr = -(3 r^2 + 10.5 s^2) t^7 = -5 t^5 (u + 0.6),
// so q comes from three fused multiply-adds seeded with s^2, r^2 is never
// formed, and every factor stays bounded (no FP32 overflow for cores down to
// the integrator's 1e-6 floor).  The cross products with the strengths are
// summed as two sums per component (sum e_y a_z and sum e_z a_y, ...),
// subtracted once per tile.
// Per-target constants: T = t, G = the target's strength, G5 = -5 G.
template <int MODE>
__device__ __forceinline__ void near_tile_direct(const float4* __restrict__ row, int nit, int g,
                                                 uint64_t TX, uint64_t TY, uint64_t TZ,
                                                 uint64_t GX, uint64_t GY, uint64_t GZ,
                                                 uint64_t G5X, uint64_t G5Y, uint64_t G5Z,
                                                 uint64_t* acc) {
  const uint64_t ONE = x2::pack(1.f, 1.f), C06 = x2::pack(0.6f, 0.6f);
  uint64_t PS[3] = {0ull, 0ull, 0ull}, MS[3] = {0ull, 0ull, 0ull};
#pragma unroll 4
  for (int i = 0; i < nit; ++i) {
    const float4* r = row + i * g;
    const float4 u0 = r[0], u1 = r[kNearTile];
    const uint64_t DX = x2::add(TX, x2::dup(u0.x)), DY = x2::add(TY, x2::dup(u0.y)),
                   DZ = x2::add(TZ, x2::dup(u0.z));
    uint64_t Q = x2::fma(DX, DX, x2::dup(u0.w));
    Q = x2::fma(DY, DY, Q);
    Q = x2::fma(DZ, DZ, Q);
    float qa, qb;
    x2::unpack(Q, qa, qb);
    const uint64_t T = x2::pack(rsqrt_ftz(qa), rsqrt_ftz(qb));
    const uint64_t T2 = x2::mul(T, T);
    const uint64_t T3 = x2::mul(T2, T);
    const uint64_t C1 = x2::dup(u1.x);
    const uint64_t AX = x2::dup(u1.y), AY = x2::dup(u1.z), AZ = x2::dup(u1.w);
    uint64_t EX, EY, EZ;
    if (MODE == FVX_PAIR_VELOCITY) {
      const uint64_t F = x2::mul(T3, x2::fma(C1, T2, ONE));
      EX = x2::mul(F, DX);
      EY = x2::mul(F, DY);
      EZ = x2::mul(F, DZ);
    } else {
      // e = f G + w d, w = fpr (d . G)
      const uint64_t T5 = x2::mul(T3, T2);
      const uint64_t F = x2::fma(C1, T5, T3);
      uint64_t DG5 = x2::mul(DX, G5X);
      DG5 = x2::fma(DY, G5Y, DG5);
      DG5 = x2::fma(DZ, G5Z, DG5);
      const uint64_t W = x2::mul(x2::mul(x2::fma(C1, T2, C06), T5), DG5);
      EX = x2::fma(W, DX, x2::mul(F, GX));
      EY = x2::fma(W, DY, x2::mul(F, GY));
      EZ = x2::fma(W, DZ, x2::mul(F, GZ));
    }
    PS[0] = x2::fma(EY, AZ, PS[0]);
    MS[0] = x2::fma(EZ, AY, MS[0]);
    PS[1] = x2::fma(EZ, AX, PS[1]);
    MS[1] = x2::fma(EX, AZ, MS[1]);
    PS[2] = x2::fma(EX, AY, PS[2]);
    MS[2] = x2::fma(EY, AX, MS[2]);
  }
  acc[0] = x2::sub(PS[0], MS[0]);
  acc[1] = x2::sub(PS[1], MS[1]);
  acc[2] = x2::sub(PS[2], MS[2]);
}

// Gaussian-erf vorticity of one staged tile (rows {-x, -y, -z, 1/s},
// {a, 1/s^2}) for the thread's two targets, in paired FP32:
//   omega += d (fpr (d . a)) - a (fpr r^2 + 2 f)
// with the core of core_f32<GAUSSIANERF>: x = r^2 / s^2 = rho^2,
// e = exp(-x / 2), g = erf(rho / sqrt2) - sqrt(2/pi) rho e, f = g / r^3,
// fpr = (sqrt(2/pi) x e / s - 3 g / r) / r^4.  erf takes the rational form of
// Abramowitz & Stegun (Handbook of Mathematical Functions, 7.1.26; absolute
// error <= 1.5e-7): erf(z) = 1 - t (a1 + t (a2 + ... + t a5)) exp(-z^2),
// t = 1 / (1 + p z), whose exponential at z = rho / sqrt2 is the same e, so a
// pair takes one ex2, one reciprocal and one reciprocal square root on the
// MUFU.  A row in which any lane has a pair with x < 0.25 (the self pair and
// close neighbours, where g cancels) also takes core_f32's series there,
// selected per target.  Sums d s1 and a s2 are kept apart and subtracted
// once per tile.
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ void near_tile_vort_gauss(const float4* __restrict__ row, int nit,
                                                     int g, uint64_t TX, uint64_t TY,
                                                     uint64_t TZ, uint64_t* acc) {
  using namespace pair;
  const uint64_t ONE = x2::dup(1.f);
  const uint64_t KP = x2::dup(static_cast<float>(0.3275911 * kInvSqrt2));  // p on rho
  // -a1..-a5: the polynomial enters as 1 - t P e
  const uint64_t NA1 = x2::dup(-0.254829592f), NA2 = x2::dup(0.284496736f),
                 NA3 = x2::dup(-1.421413741f), NA4 = x2::dup(1.453152027f),
                 NA5 = x2::dup(-1.061405429f);
  const uint64_t NHL2E = x2::dup(static_cast<float>(-0.5 * 1.4426950408889634));  // -log2(e)/2
  const uint64_t CS = x2::dup(static_cast<float>(kSqrt2OverPi)),
                 NCS = x2::dup(static_cast<float>(-kSqrt2OverPi)), M3 = x2::dup(-3.f),
                 TWO = x2::dup(2.f);
  uint64_t PS[3] = {0ull, 0ull, 0ull}, QS[3] = {0ull, 0ull, 0ull};
#pragma unroll 2
  for (int i = 0; i < nit; ++i) {
    const float4* r = row + i * g;
    const float4 u0 = r[0], u1 = r[kNearTile];
    const uint64_t DX = x2::add(TX, x2::dup(u0.x)), DY = x2::add(TY, x2::dup(u0.y)),
                   DZ = x2::add(TZ, x2::dup(u0.z));
    const uint64_t IS = x2::dup(u0.w), IS2 = x2::dup(u1.w);
    const uint64_t AX = x2::dup(u1.x), AY = x2::dup(u1.y), AZ = x2::dup(u1.z);
    uint64_t R2 = x2::mul(DZ, DZ);
    R2 = x2::fma(DY, DY, R2);
    R2 = x2::fma(DX, DX, R2);
    uint64_t DA = x2::mul(DZ, AZ);
    DA = x2::fma(DY, AY, DA);
    DA = x2::fma(DX, AX, DA);
    const uint64_t X = x2::mul(R2, IS2);
    float r2a, r2b;
    x2::unpack(R2, r2a, r2b);
    const uint64_t IR = x2::pack(rsqrt_ftz(r2a), rsqrt_ftz(r2b));
    const uint64_t RHO = x2::mul(x2::mul(R2, IR), IS);
    float ea, eb;
    x2::unpack(x2::mul(X, NHL2E), ea, eb);
    const uint64_t E = x2::pack(ex2_ftz(ea), ex2_ftz(eb));
    float ta, tb;
    x2::unpack(x2::fma(RHO, KP, ONE), ta, tb);
    const uint64_t T = x2::pack(rcp_ftz(ta), rcp_ftz(tb));
    uint64_t P = x2::fma(NA5, T, NA4);
    P = x2::fma(P, T, NA3);
    P = x2::fma(P, T, NA2);
    P = x2::fma(P, T, NA1);
    P = x2::mul(P, T);
    const uint64_t G = x2::fma(x2::mul(RHO, E), NCS, x2::fma(P, E, ONE));
    const uint64_t IR2 = x2::mul(IR, IR), IR3 = x2::mul(IR2, IR);
    uint64_t F = x2::mul(G, IR3);
    uint64_t FPR = x2::mul(x2::fma(x2::mul(x2::mul(X, E), IS), CS, x2::mul(x2::mul(G, IR), M3)),
                           x2::mul(IR3, IR));
    float xa, xb;
    x2::unpack(X, xa, xb);
    if (__any_sync(0xffffffffu, xa < 0.25f || xb < 0.25f)) {
      // the series of core_f32 for x < 0.25
      uint64_t H = x2::fma(x2::dup(static_cast<float>(FVX_GA6)), X,
                           x2::dup(static_cast<float>(FVX_GA5)));
      H = x2::fma(H, X, x2::dup(static_cast<float>(FVX_GA4)));
      H = x2::fma(H, X, x2::dup(static_cast<float>(FVX_GA3)));
      H = x2::fma(H, X, x2::dup(static_cast<float>(FVX_GA2)));
      H = x2::fma(H, X, x2::dup(static_cast<float>(FVX_GA1)));
      H = x2::fma(H, X, x2::dup(static_cast<float>(FVX_GA0)));
      uint64_t DD = x2::fma(x2::dup(static_cast<float>(12.0 * FVX_GA6)), X,
                            x2::dup(static_cast<float>(10.0 * FVX_GA5)));
      DD = x2::fma(DD, X, x2::dup(static_cast<float>(8.0 * FVX_GA4)));
      DD = x2::fma(DD, X, x2::dup(static_cast<float>(6.0 * FVX_GA3)));
      DD = x2::fma(DD, X, x2::dup(static_cast<float>(4.0 * FVX_GA2)));
      DD = x2::fma(DD, X, x2::dup(static_cast<float>(2.0 * FVX_GA1)));
      const uint64_t IS3 = x2::mul(x2::mul(IS, IS), IS);
      const uint64_t FS = x2::mul(x2::mul(CS, H), IS3);
      const uint64_t FPRS = x2::mul(x2::mul(x2::mul(x2::mul(CS, DD), IS3), IS), IS);
      float fa, fb, pa, pb, sa, sb, qa, qb;
      x2::unpack(F, fa, fb);
      x2::unpack(FPR, pa, pb);
      x2::unpack(FS, sa, sb);
      x2::unpack(FPRS, qa, qb);
      if (xa < 0.25f) {
        fa = sa;
        pa = qa;
      }
      if (xb < 0.25f) {
        fb = sb;
        pb = qb;
      }
      F = x2::pack(fa, fb);
      FPR = x2::pack(pa, pb);
    }
    const uint64_t S1 = x2::mul(FPR, DA);
    const uint64_t S2 = x2::fma(FPR, R2, x2::mul(F, TWO));
    PS[0] = x2::fma(DX, S1, PS[0]);
    PS[1] = x2::fma(DY, S1, PS[1]);
    PS[2] = x2::fma(DZ, S1, PS[2]);
    QS[0] = x2::fma(AX, S2, QS[0]);
    QS[1] = x2::fma(AY, S2, QS[1]);
    QS[2] = x2::fma(AZ, S2, QS[2]);
  }
  acc[0] = x2::sub(PS[0], QS[0]);
  acc[1] = x2::sub(PS[1], QS[1]);
  acc[2] = x2::sub(PS[2], QS[2]);
}

// The same sums in the factored form (FACT): d x a = t x a - x_s x a with
// c = x_s x a staged per source, and d never formed: q = |t|^2 + S - 2 t . x_s
// and d . G = t . G - x_s . G take three fused multiply-adds each from
// per-target constants.  Velocity sums f a and f c (14 paired operations per
// pair of pairs, 19 in the direct form), stretching f a, w' a and w' c with
// w = -5 w' (23, 28 in the direct form); the factor -5 and the cross products
// with t and G are applied once per tile.  The sums cancel where |d| is far
// below |x_s| or |t|, so a sweep takes this form only when the leaf size is
// at most 4 times the smallest core (|t|, |x_s| of order h, q >= s^2 >=
// h^2 / 16, and the rounding stays within a few tens of FP32 units of q and
// of a source's peak contribution).
// Per-target constants: M2 = -2 t, TT = |t|^2, NG = -G, TG = t . G.
template <int MODE, int NP>
__device__ __forceinline__ void near_tile_factored(const float4* __restrict__ row, int nit, int g,
                                                   const uint64_t* M2X, const uint64_t* M2Y,
                                                   const uint64_t* M2Z, const uint64_t* TT,
                                                   const uint64_t* NGX, const uint64_t* NGY,
                                                   const uint64_t* NGZ, const uint64_t* TG,
                                                   uint64_t (*acc)[3]) {
  const uint64_t ONE = x2::pack(1.f, 1.f), C06 = x2::pack(0.6f, 0.6f);
  uint64_t FA[NP][3], WA[NP][3], WC[NP][3];
#pragma unroll
  for (int p = 0; p < NP; ++p)
#pragma unroll
    for (int c = 0; c < 3; ++c) FA[p][c] = WA[p][c] = WC[p][c] = 0ull;
  // unrolled 4 x for one pair of velocity targets, 2 x for two pairs and for
  // the longer stretching body (4.61 -> 4.49 ms per sweep at 2^20; 1 x and
  // 8 x are no better)
  constexpr int kUnroll = MODE == FVX_PAIR_STRETCH || NP > 1 ? 2 : 4;
#pragma unroll kUnroll
  for (int i = 0; i < nit; ++i) {
    const float4* r = row + i * g;
    const float4 u0 = r[0], u1 = r[kNearTile], u2 = r[2 * kNearTile];
    const uint64_t X = x2::dup(u0.x), Y = x2::dup(u0.y), Z = x2::dup(u0.z), S = x2::dup(u0.w);
    const uint64_t C1 = x2::dup(u1.x);
    const uint64_t AX = x2::dup(u1.y), AY = x2::dup(u1.z), AZ = x2::dup(u1.w);
    const uint64_t CX = x2::dup(u2.x), CY = x2::dup(u2.y), CZ = x2::dup(u2.z);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      uint64_t Q = x2::add(TT[p], S);
      Q = x2::fma(M2X[p], X, Q);
      Q = x2::fma(M2Y[p], Y, Q);
      Q = x2::fma(M2Z[p], Z, Q);
      float qa, qb;
      x2::unpack(Q, qa, qb);
      const uint64_t T = x2::pack(rsqrt_ftz(qa), rsqrt_ftz(qb));
      const uint64_t T2 = x2::mul(T, T);
      const uint64_t T3 = x2::mul(T2, T);
      if (MODE == FVX_PAIR_VELOCITY) {
        const uint64_t F = x2::mul(T3, x2::fma(C1, T2, ONE));
        FA[p][0] = x2::fma(F, AX, FA[p][0]);
        FA[p][1] = x2::fma(F, AY, FA[p][1]);
        FA[p][2] = x2::fma(F, AZ, FA[p][2]);
        WC[p][0] = x2::fma(F, CX, WC[p][0]);
        WC[p][1] = x2::fma(F, CY, WC[p][1]);
        WC[p][2] = x2::fma(F, CZ, WC[p][2]);
      } else {
        const uint64_t T5 = x2::mul(T3, T2);
        const uint64_t F = x2::fma(C1, T5, T3);
        uint64_t DG = x2::fma(NGX[p], X, TG[p]);
        DG = x2::fma(NGY[p], Y, DG);
        DG = x2::fma(NGZ[p], Z, DG);
        const uint64_t W = x2::mul(x2::mul(x2::fma(C1, T2, C06), T5), DG);
        FA[p][0] = x2::fma(F, AX, FA[p][0]);
        FA[p][1] = x2::fma(F, AY, FA[p][1]);
        FA[p][2] = x2::fma(F, AZ, FA[p][2]);
        WA[p][0] = x2::fma(W, AX, WA[p][0]);
        WA[p][1] = x2::fma(W, AY, WA[p][1]);
        WA[p][2] = x2::fma(W, AZ, WA[p][2]);
        WC[p][0] = x2::fma(W, CX, WC[p][0]);
        WC[p][1] = x2::fma(W, CY, WC[p][1]);
        WC[p][2] = x2::fma(W, CZ, WC[p][2]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    if (MODE == FVX_PAIR_VELOCITY) {
      // sum f (d x a) = t x FA - sum f c, t = -M2 / 2 (exact)
      const uint64_t MH = x2::pack(-0.5f, -0.5f);
      const uint64_t TX = x2::mul(M2X[p], MH), TY = x2::mul(M2Y[p], MH), TZ = x2::mul(M2Z[p], MH);
      acc[p][0] = x2::sub(x2::mul(TY, FA[p][2]), x2::fma(TZ, FA[p][1], WC[p][0]));
      acc[p][1] = x2::sub(x2::mul(TZ, FA[p][0]), x2::fma(TX, FA[p][2], WC[p][1]));
      acc[p][2] = x2::sub(x2::mul(TX, FA[p][1]), x2::fma(TY, FA[p][0], WC[p][2]));
    } else {
      // G x FA + t x (sum w a) - sum w c = -(NG x FA) + 2.5 (M2 x WA) + 5 WC
      const uint64_t MONE = x2::pack(-1.f, -1.f), P25 = x2::pack(2.5f, 2.5f),
                     P5 = x2::pack(5.f, 5.f);
      const uint64_t GX = x2::mul(NGX[p], MONE), GY = x2::mul(NGY[p], MONE),
                     GZ = x2::mul(NGZ[p], MONE);
      const uint64_t HX = x2::mul(M2X[p], P25), HY = x2::mul(M2Y[p], P25),
                     HZ = x2::mul(M2Z[p], P25);
      acc[p][0] = x2::add(x2::sub(x2::mul(GY, FA[p][2]), x2::mul(GZ, FA[p][1])),
                          x2::fma(P5, WC[p][0], x2::sub(x2::mul(HY, WA[p][2]), x2::mul(HZ, WA[p][1]))));
      acc[p][1] = x2::add(x2::sub(x2::mul(GZ, FA[p][0]), x2::mul(GX, FA[p][2])),
                          x2::fma(P5, WC[p][1], x2::sub(x2::mul(HZ, WA[p][0]), x2::mul(HX, WA[p][2]))));
      acc[p][2] = x2::add(x2::sub(x2::mul(GX, FA[p][1]), x2::mul(GY, FA[p][0])),
                          x2::fma(P5, WC[p][2], x2::sub(x2::mul(HX, WA[p][1]), x2::mul(HY, WA[p][0]))));
    }
  }
}

// Shared memory of an evaluation warp: the near tile (plain or paired layout)
// and the far-cell records share the storage.
template <int MODE, int KERNEL, int TPT>
struct EvalSmem {
  // paired path: Winckelmans velocity / stretching with two or four targets
  // per thread, the Gaussian-erf vorticity with two
  static constexpr bool VORT_GAUSS = KERNEL == FVX_KERNEL_GAUSSIANERF && MODE == FVX_PAIR_VORTICITY;
  static constexpr bool PACKED =
      ((TPT == 2 || TPT == 4) && KERNEL == FVX_KERNEL_WINCKELMANS &&
       (MODE == FVX_PAIR_VELOCITY || MODE == FVX_PAIR_STRETCH)) ||
      (TPT == 2 && VORT_GAUSS);
  // paired: the tile's planes, then the lanes' running near-field sums
  // (hi, lo of TPT targets x three components, 6 TPT x 32 floats)
  static constexpr int kNearBytes = PACKED ? kPlanes * kNearTile * 16 + 6 * TPT * kEvalThreads * 4
                                           : kNearTile * 2 * static_cast<int>(sizeof(float4));
  static constexpr int kFarBytes = kFarTile * kRecFloats * 4;
  static constexpr int bytes = kNearBytes > kFarBytes ? kNearBytes : kFarBytes;
};

// Leaf t: its targets against its near leaves and far cells, plus the local
// expansions (one warp).
template <int MODE, int KERNEL, int TPT, bool FACT>
__device__ __forceinline__ void eval_leaf(const EvalArgs& A, int t, unsigned char* s_raw) {
  using namespace pair;
  constexpr int NC = ModeInfo<MODE>::ncomp;
  constexpr int NA = ModeInfo<MODE>::na;
  constexpr bool NEED_FPR = ModeInfo<MODE>::need_fpr;
  constexpr bool NEED_TG = ModeInfo<MODE>::need_tg;
  constexpr bool PACKED = EvalSmem<MODE, KERNEL, TPT>::PACKED;
  float4* s_p = reinterpret_cast<float4*>(s_raw);
  float4* s_a = s_p + kNearTile;
  float* s_rec = reinterpret_cast<float*>(s_raw);

  const int tstart = A.leaf_start[t], tcount = A.leaf_count[t];
  const float3 cT = cell_center_rel(A.leaf_key[t], A.h);
  const int nno = A.near_off[t], nnc = A.near_cnt[t];
  const int fno = A.far_off[t], fnc = A.far_cnt[t];
  // Paired path: TPT = 2 or 4 targets per lane (one or two pairs of paired
  // registers), the leaf's targets in chunks of at most 16 TPT.  A chunk of c
  // targets puts TPT in each of m = ceil(c/TPT) lanes and splits the sources
  // over g = floor(32/m) groups of m lanes (group j sums rows j, j + g, ...);
  // the groups' partial sums are added into group 0 at the end of the near
  // field.  Lanes past the g groups mirror group 0 and are not counted.  The
  // other paths take TPT targets per lane.
  constexpr int NP = TPT / 2;  // pairs of targets per lane (paired path)
  const int chunk_step = PACKED ? (kEvalThreads / 2) * TPT : kEvalThreads * TPT;
  const int lane = threadIdx.x;

  for (int chunk = 0; chunk < tcount; chunk += chunk_step) {
    const int cend = min(tcount, chunk + chunk_step);
    int m = kEvalThreads, g = 1, grp = 0, tl = lane;
    bool spare = false;
    if constexpr (PACKED) {
      m = (cend - chunk + TPT - 1) / TPT;
      g = kEvalThreads / m;
      grp = lane / m;
      tl = lane - grp * m;
      spare = grp >= g;
      if (spare) grp = 0;
    }
    float ox[TPT], oy[TPT], oz[TPT], gx[TPT], gy[TPT], gz[TPT];
    float hi[TPT][NC], lo[TPT][NC];
    bool act[TPT];
    int kk[TPT];
    // the lane's targets (reloaded after the paired near field rather than
    // held through it)
    auto load_targets = [&]() {
#pragma unroll
      for (int j = 0; j < TPT; ++j) {
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f), gv = p;
        if (kk[j] < cend) {
          p = A.sp[tstart + kk[j]];
          if (NEED_TG) gv = A.sg[tstart + kk[j]];
        }
        ox[j] = p.x;
        oy[j] = p.y;
        oz[j] = p.z;
        gx[j] = gv.x;
        gy[j] = gv.y;
        gz[j] = gv.z;
      }
    };
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      kk[j] = chunk + tl + j * m;
      act[j] = kk[j] < cend && grp == 0 && !spare;
#pragma unroll
      for (int c = 0; c < NC; ++c) hi[j][c] = lo[j][c] = 0.f;
    }
    load_targets();
    // near field: direct pairs with every near leaf
    if constexpr (PACKED) {
      // Tiles of up to kNearTile sources filled from up to 32 near leaves at
      // a time: lane l holds near leaf l's start, count and exact centre
      // difference c_T - c_S, a warp prefix sum places the leaves' sources
      // one after another, and each staged source is stored relative to the
      // target leaf's centre (the centre difference folded in while staging,
      // the same two roundings as forming the target relative to the source
      // leaf), so one tile mixes leaves and its barriers, loads and fold are
      // paid per 128 sources instead of per near leaf.
      const unsigned full = 0xffffffffu;
      // per-target constants, pair p holding the lane's targets 2p and 2p + 1:
      // direct form t, G, -5 G; factored form -2 t, |t|^2, -G, t . G
      uint64_t TX[NP], TY[NP], TZ[NP], GX[NP], GY[NP], GZ[NP], G5X[NP], G5Y[NP], G5Z[NP];
      uint64_t M2X[NP], M2Y[NP], M2Z[NP], TT[NP], NGX[NP], NGY[NP], NGZ[NP], TG[NP];
      const float m5 = -5.f, m2 = -2.f;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const int a = 2 * p, b = 2 * p + 1;
        TX[p] = x2::pack(ox[a], ox[b]);
        TY[p] = x2::pack(oy[a], oy[b]);
        TZ[p] = x2::pack(oz[a], oz[b]);
        GX[p] = x2::pack(gx[a], gx[b]);
        GY[p] = x2::pack(gy[a], gy[b]);
        GZ[p] = x2::pack(gz[a], gz[b]);
        G5X[p] = x2::pack(m5 * gx[a], m5 * gx[b]);
        G5Y[p] = x2::pack(m5 * gy[a], m5 * gy[b]);
        G5Z[p] = x2::pack(m5 * gz[a], m5 * gz[b]);
        M2X[p] = x2::pack(m2 * ox[a], m2 * ox[b]);
        M2Y[p] = x2::pack(m2 * oy[a], m2 * oy[b]);
        M2Z[p] = x2::pack(m2 * oz[a], m2 * oz[b]);
        TT[p] = x2::pack(fmaf(ox[a], ox[a], fmaf(oy[a], oy[a], oz[a] * oz[a])),
                         fmaf(ox[b], ox[b], fmaf(oy[b], oy[b], oz[b] * oz[b])));
        NGX[p] = x2::pack(-gx[a], -gx[b]);
        NGY[p] = x2::pack(-gy[a], -gy[b]);
        NGZ[p] = x2::pack(-gz[a], -gz[b]);
        TG[p] = x2::pack(fmaf(ox[a], gx[a], fmaf(oy[a], gy[a], oz[a] * gz[a])),
                         fmaf(ox[b], gx[b], fmaf(oy[b], gy[b], oz[b] * gz[b])));
      }
      float4* s_r = reinterpret_cast<float4*>(s_raw);
      // the running sums stay in shared memory through the near field (each
      // lane its own column), not in registers
      float* s_sum = reinterpret_cast<float*>(s_raw + kPlanes * kNearTile * 16) + lane;
#pragma unroll
      for (int e = 0; e < 6 * TPT; ++e) s_sum[e * kEvalThreads] = 0.f;
      for (int q0 = 0; q0 < nnc; q0 += kEvalThreads) {
        int mss = 0, msn = 0;
        float mdx = 0.f, mdy = 0.f, mdz = 0.f;
        if (q0 + lane < nnc) {
          const int S = A.near_idx[nno + q0 + lane];
          mss = A.leaf_start[S];
          msn = A.leaf_count[S];
          const float3 cS = cell_center_rel(A.leaf_key[S], A.h);
          mdx = cT.x - cS.x;
          mdy = cT.y - cS.y;
          mdz = cT.z - cS.z;
        }
        int incl = msn;
#pragma unroll
        for (int o = 1; o < kEvalThreads; o <<= 1) {
          const int v = __shfl_up_sync(full, incl, o);
          if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(full, incl, kEvalThreads - 1);
        const int excl = incl - msn;
        // a tile holds a multiple of g sources (at most kNearTile), so that
        // padding its last one to a multiple of g stays within the planes
        const int tile_src = kNearTile / g * g;
        for (int b0 = 0; b0 < total; b0 += tile_src) {
          const int nt = min(tile_src, total - b0);
          // rows: nt sources padded with zero-strength ones to a multiple of g
          const int rows = (nt + g - 1) / g * g;
          __syncthreads();
          for (int r0 = 0; r0 < rows; r0 += kEvalThreads) {
            const int k = r0 + lane;
            // each staged source's near leaf, from the leaves' start offsets in
            // this window of 32 sources: one bit per start (near leaves are
            // never empty, so starts are distinct), and a source's leaf is the
            // number of starts up to it, minus one
            const int pl = excl - (b0 + r0);
            const unsigned bits = __reduce_or_sync(full, (pl >= 0 && pl < 32) ? 1u << pl : 0u);
            const int before = __popc(__ballot_sync(full, pl < 0));
            const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
            const int li = before + __popc(bits & upto) - 1;
            const int lss = __shfl_sync(full, mss, li), lex = __shfl_sync(full, excl, li);
            const float ldx = __shfl_sync(full, mdx, li), ldy = __shfl_sync(full, mdy, li),
                        ldz = __shfl_sync(full, mdz, li);
            float4 p = make_float4(0.f, 0.f, 0.f, 1.f), av = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < nt) {
              const int src = lss + b0 + k - lex;
              const float4 pv = A.sp[src];
              p = make_float4(pv.x - ldx, pv.y - ldy, pv.z - ldz, pv.w);
              av = A.sa[src];
            }
            if (k < rows) {
              float4* row = s_r + k;
              if constexpr (EvalSmem<MODE, KERNEL, TPT>::VORT_GAUSS) {
                // {-x, 1/s}, {a, 1/s^2} (a padding row: 1/s = 0, no strength)
                row[0] = make_float4(-p.x, -p.y, -p.z, av.w);
                row[kNearTile] = make_float4(av.x, av.y, av.z, av.w * av.w);
              } else {
                if constexpr (FACT) {
                  const float S2 = fmaf(p.x, p.x, fmaf(p.y, p.y, fmaf(p.z, p.z, p.w)));
                  row[0] = make_float4(p.x, p.y, p.z, S2);
                  row[2 * kNearTile] =
                      make_float4(p.y * av.z - p.z * av.y, p.z * av.x - p.x * av.z,
                                  p.x * av.y - p.y * av.x, 0.f);
                } else {
                  row[0] = make_float4(-p.x, -p.y, -p.z, p.w);
                }
                row[kNearTile] = make_float4(1.5f * p.w, av.x, av.y, av.z);
              }
            }
          }
          __syncthreads();
          uint64_t acc2[NP][3];
          const float4* row = s_r + grp;
          if constexpr (FACT) {
            near_tile_factored<MODE, NP>(row, rows / g, g, M2X, M2Y, M2Z, TT, NGX, NGY, NGZ, TG,
                                         acc2);
          } else if constexpr (EvalSmem<MODE, KERNEL, TPT>::VORT_GAUSS) {
            near_tile_vort_gauss(row, rows / g, g, TX[0], TY[0], TZ[0], acc2[0]);
          } else {
            static_assert(FACT || NP == 1, "the direct form takes two targets per lane");
            near_tile_direct<MODE>(row, rows / g, g, TX[0], TY[0], TZ[0], GX[0], GY[0], GZ[0],
                                   G5X[0], G5Y[0], G5Z[0], acc2[0]);
          }
#pragma unroll
          for (int p = 0; p < NP; ++p)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              float a[2];
              x2::unpack(acc2[p][c], a[0], a[1]);
#pragma unroll
              for (int h2 = 0; h2 < 2; ++h2) {
                float* e = s_sum + (2 * (c * TPT + 2 * p + h2)) * kEvalThreads;
                float hv = e[0], lv = e[kEvalThreads];
                fold(hv, lv, a[h2]);
                e[0] = hv;
                e[kEvalThreads] = lv;
              }
            }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int j = 0; j < TPT; ++j) {
          hi[j][c] = s_sum[(2 * (c * TPT + j)) * kEvalThreads];
          lo[j][c] = s_sum[(2 * (c * TPT + j) + 1) * kEvalThreads];
        }
      load_targets();
      // the groups' partial sums into group 0 (lanes tl + j m, j < g), read
      // from copies: every lane updates its own sums while others read them
      float ph[TPT][3], pq[TPT][3];
#pragma unroll
      for (int s2 = 0; s2 < TPT; ++s2)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          ph[s2][c] = hi[s2][c];
          pq[s2][c] = lo[s2][c];
        }
      for (int j = 1; j < g; ++j) {
        const int src = tl + j * m;
#pragma unroll
        for (int s2 = 0; s2 < TPT; ++s2)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float vh = __shfl_sync(full, ph[s2][c], src);
            const float vl = __shfl_sync(full, pq[s2][c], src);
            fold(hi[s2][c], lo[s2][c], vh);
            lo[s2][c] += vl;
          }
      }
    }
    for (int q = 0; q < (PACKED ? 0 : nnc); ++q) {
      const int S = A.near_idx[nno + q];
      const int ss = A.leaf_start[S], sn = A.leaf_count[S];
      const float3 cS = cell_center_rel(A.leaf_key[S], A.h);
      const float dcx = cT.x - cS.x, dcy = cT.y - cS.y, dcz = cT.z - cS.z;
      float tx[TPT], ty[TPT], tz[TPT];
#pragma unroll
      for (int j = 0; j < TPT; ++j) {
        tx[j] = ox[j] + dcx;
        ty[j] = oy[j] + dcy;
        tz[j] = oz[j] + dcz;
      }
      for (int k0 = 0; k0 < sn; k0 += kNearTile) {
        const int nt = min(kNearTile, sn - k0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += kEvalThreads) {
          s_p[k] = A.sp[ss + k0 + k];
          s_a[k] = A.sa[ss + k0 + k];
        }
        __syncthreads();
        float part[TPT][NC];
#pragma unroll
        for (int j = 0; j < TPT; ++j)
#pragma unroll
          for (int c = 0; c < NC; ++c) part[j][c] = 0.f;
        for (int k = 0; k < nt; ++k) {
          const float4 pv = s_p[k];
          const float4 av = s_a[k];
#pragma unroll
          for (int j = 0; j < TPT; ++j) {
            const float dx = tx[j] - pv.x, dy = ty[j] - pv.y, dz = tz[j] - pv.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            float f, fpr = 0.f;
            core_f32<KERNEL, NEED_FPR>(r2, pv.w, av.w, f, fpr);
            accumulate<MODE, float>(part[j], dx, dy, dz, r2, av.x, av.y, av.z, f, fpr, gx[j],
                                    gy[j], gz[j]);
          }
        }
#pragma unroll
        for (int j = 0; j < TPT; ++j)
#pragma unroll
          for (int c = 0; c < NC; ++c) fold(hi[j][c], lo[j][c], part[j][c]);
      }
    }
    // far field: multipole expansions of the accepted cells
    for (int f0 = 0; f0 < fnc; f0 += kFarTile) {
      const int nt = min(kFarTile, fnc - f0);
      __syncthreads();
      for (int x = threadIdx.x; x < nt * kRecFloats; x += kEvalThreads) {
        const int c = x / kRecFloats, o = x - c * kRecFloats;
        s_rec[x] = A.rec[static_cast<int64_t>(A.far_idx[fno + f0 + c]) * kRecFloats + o];
      }
      __syncthreads();
      float part[TPT][NC];
#pragma unroll
      for (int j = 0; j < TPT; ++j)
#pragma unroll
        for (int c = 0; c < NC; ++c) part[j][c] = 0.f;
      for (int c = 0; c < nt; ++c) {
        const float* R = s_rec + c * kRecFloats;
        const float dcx = cT.x - R[0], dcy = cT.y - R[1], dcz = cT.z - R[2];
#pragma unroll
        for (int j = 0; j < TPT; ++j)
          m2p<MODE>(part[j], R, ox[j] + dcx, oy[j] + dcy, oz[j] + dcz, gx[j], gy[j], gz[j]);
      }
#pragma unroll
      for (int j = 0; j < TPT; ++j)
#pragma unroll
        for (int c = 0; c < NC; ++c) fold(hi[j][c], lo[j][c], part[j][c]);
    }
    if (A.parent_local) {
      // the parent's expansion about its own centre (parent key = leaf key >> 3)
      const float3 cP = cell_center_rel(A.leaf_key[t] >> 3, 2.f * A.h);
      const float qx = cT.x - cP.x, qy = cT.y - cP.y, qz = cT.z - cP.z;
      const float* L = A.parent_local + static_cast<int64_t>(A.leaf_parent[t]) * 32;
      float Ls[30];
#pragma unroll
      for (int c = 0; c < 30; ++c) Ls[c] = L[c];
#pragma unroll
      for (int j = 0; j < TPT; ++j) {
        float part[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) part[c] = 0.f;
        l2p<MODE>(part, Ls, ox[j] + qx, oy[j] + qy, oz[j] + qz, gx[j], gy[j], gz[j]);
#pragma unroll
        for (int c = 0; c < NC; ++c) fold(hi[j][c], lo[j][c], part[c]);
      }
    }
    if (A.leaf_local) {
      const float* L = A.leaf_local + static_cast<int64_t>(t) * 32;
      float Ls[30];
#pragma unroll
      for (int c = 0; c < 30; ++c) Ls[c] = L[c];
#pragma unroll
      for (int j = 0; j < TPT; ++j) {
        float part[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) part[c] = 0.f;
        l2p<MODE>(part, Ls, ox[j], oy[j], oz[j], gx[j], gy[j], gz[j]);
#pragma unroll
        for (int c = 0; c < NC; ++c) fold(hi[j][c], lo[j][c], part[c]);
      }
    }
#pragma unroll
    for (int j = 0; j < TPT; ++j) {
      if (!act[j]) continue;
      const int i = A.perm[tstart + kk[j]];
#pragma unroll
      for (int c = 0; c < NA; ++c)
        A.out_a[static_cast<int64_t>(i) * NA + c] =
            static_cast<double>(hi[j][c]) + static_cast<double>(lo[j][c]);
#pragma unroll
      for (int c = NA; c < NC; ++c)
        A.out_b[static_cast<int64_t>(i) * (NC - NA) + (c - NA)] =
            static_cast<double>(hi[j][c]) + static_cast<double>(lo[j][c]);
    }
  }
}

// Resident evaluation warps (one per CTA) take leaves from a shared counter
// until none are left: the SMs stay at their occupancy limit to the end, and
// no CTA is launched per leaf.  The leaves come in decreasing order of their
// near-field work, so the last ones taken are the shortest.
template <int MODE, int KERNEL, int TPT, bool FACT>
__device__ __forceinline__ void eval_leaves(const EvalArgs& A) {
  __shared__ __align__(16) unsigned char s_raw[EvalSmem<MODE, KERNEL, TPT>::bytes];
  for (;;) {
    int c = 0;
    if (threadIdx.x == 0) c = atomicAdd(A.leaf_next, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= A.nleaf) break;
    eval_leaf<MODE, KERNEL, TPT, FACT>(A, A.leaf_order[c], s_raw);
    __syncthreads();  // the next leaf restages the shared buffer
  }
}

template <int MODE, int KERNEL, int TPT>
__global__ void __launch_bounds__(kEvalThreads) eval_kernel(EvalArgs A) {
  eval_leaves<MODE, KERNEL, TPT, false>(A);
}

// The factored loops (paired Winckelmans): stretching with two targets per
// lane held to 24 resident warps per SM (at most 80 registers); velocity with
// four targets per lane, so that each staged value serves four pairs (the
// velocity loop was bound by the shared-memory pipe: 3.09 -> 2.93 ms per sweep
// at 2^20), held to 20 warps (96 registers; 16 and 24 warps are no faster).
template <int MODE, int KERNEL, int TPT>
__global__ void __launch_bounds__(kEvalThreads, TPT == 4 ? 20 : 24)
    eval_kernel_factored(EvalArgs A) {
  eval_leaves<MODE, KERNEL, TPT, true>(A);
}

// ---- the FP64 judge of the local-expansion path ------------------------------------
// (pair classes: judge_class in fvx_common.cuh)

// Both lists of local-expansion pairs (rows: list 0's, then list 1's).
struct JudgeLists {
  const int* tgt[2];
  const int* cell[2];
  const uint32_t* key[2];
  float h[2];
  int n0, n;
};

// Class of every pair (cls[row]) and the class sizes (hist, accumulated).
__global__ void judge_classify_kernel(JudgeLists J, const float* __restrict__ rec,
                                      float inv_theta2, uint8_t* __restrict__ cls,
                                      unsigned* __restrict__ hist) {
  __shared__ unsigned sh[kJudgeClasses];
  if (threadIdx.x < kJudgeClasses) sh[threadIdx.x] = 0u;
  __syncthreads();
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < J.n; r += gridDim.x * blockDim.x) {
    const int li = r >= J.n0 ? 1 : 0;
    const int i = r - li * J.n0;
    const int t = J.tgt[li][i], c = J.cell[li][i];
    const float3 cT = cell_center_rel(J.key[li][t], J.h[li]);
    const float4 cs = __ldg(reinterpret_cast<const float4*>(rec + static_cast<int64_t>(c) * kRecFloats));
    const float dx = cT.x - cs.x, dy = cT.y - cs.y, dz = cT.z - cs.z;
    const int k = judge_class(li, J.h[li], cs.w, dx * dx + dy * dy + dz * dz, inv_theta2);
    cls[r] = static_cast<uint8_t>(k);
    atomicAdd(&sh[k], 1u);
  }
  __syncthreads();
  if (threadIdx.x < kJudgeClasses && sh[threadIdx.x]) atomicAdd(hist + threadIdx.x, sh[threadIdx.x]);
}

// Judge state on the device, one block of words (zeroed per judged sweep).
struct JudgeWords {
  unsigned checked, repaired, err_sum_bits, err_max_bits, applied;
  unsigned class_pairs[kJudgeClasses], class_samples[kJudgeClasses];
  unsigned fail_learned[kJudgeClasses], fail_analytic[kJudgeClasses];
  unsigned action[kJudgeClasses], taken[kJudgeClasses];
  int cnt[2];
  float unrepaired;
};

struct JudgeSampleBufs {
  int* row[2];       // index of the sampled pair in its list
  int* tgt[2];       // its target (leaf or parent)
  int* cell[2];
  uint32_t* key[2];
  uint8_t* cls[2];
  int cap;
};

__host__ __device__ __forceinline__ uint32_t judge_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// Stratified random sample: a pair of class k (n_k pairs) is taken with
// probability s_k / n_k, s_k = min(n_k, per_class) (every pair of a class with
// at most per_class pairs), from a hash of (row, seed); at most 2 per_class
// per class are kept.
__global__ void judge_select_kernel(JudgeLists J, const uint8_t* __restrict__ cls,
                                    const unsigned* __restrict__ hist, int per_class,
                                    uint32_t seed, JudgeWords* W, JudgeSampleBufs B) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < J.n; r += gridDim.x * blockDim.x) {
    const int k = cls[r];
    const unsigned nk = hist[k];
    const unsigned sk = nk < static_cast<unsigned>(per_class) ? nk : per_class;
    if (judge_hash(static_cast<uint32_t>(r) ^ seed) % nk >= sk) continue;
    if (atomicAdd(&W->taken[k], 1u) >= 2u * per_class) continue;
    const int li = r >= J.n0 ? 1 : 0;
    const int i = r - li * J.n0;
    const int q = atomicAdd(&W->cnt[li], 1);
    if (q >= B.cap) continue;  // cannot happen: 2 x per_class x 8 classes per list
    const int t = J.tgt[li][i];
    B.row[li][q] = i;
    B.tgt[li][q] = t;
    B.cell[li][q] = J.cell[li][i];
    B.key[li][q] = J.key[li][t];
    B.cls[li][q] = static_cast<uint8_t>(k);
  }
}

// Unused slots get a valid pair (the list's first), so that the translation
// and network kernels can run over all cap slots; pair_tgt is the identity.
__global__ void judge_pad_kernel(JudgeLists J, JudgeWords* W, JudgeSampleBufs B, int* iota) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= B.cap) return;
  iota[q] = q;
  for (int li = 0; li < 2; ++li) {
    const int nl = li ? J.n - J.n0 : J.n0;
    if (nl <= 0) continue;
    if (q < W->cnt[li]) continue;
    const int t = J.tgt[li][0];
    B.row[li][q] = 0;
    B.tgt[li][q] = t;
    B.cell[li][q] = J.cell[li][0];
    B.key[li][q] = J.key[li][t];
    B.cls[li][q] = 0;
  }
}

__device__ __forceinline__ float expansion_error(const float* p, const double* t, float rho) {
  float dn[3] = {0.f, 0.f, 0.f}, tn[3] = {0.f, 0.f, 0.f};
  for (int c = 0; c < 30; ++c) {
    const float tc = static_cast<float>(t[c]);
    const int g = c < 3 ? 0 : (c < 12 ? 1 : 2);
    dn[g] += (p[c] - tc) * (p[c] - tc);
    tn[g] += tc * tc;
  }
  const float w1 = rho, w2 = 0.5f * rho * rho;
  const float num = sqrtf(dn[0]) + w1 * sqrtf(dn[1]) + w2 * sqrtf(dn[2]);
  const float den = sqrtf(tn[0]) + w1 * sqrtf(tn[1]) + w2 * sqrtf(tn[2]);
  return num / fmaxf(den, 1e-30f);
}

// Per sample: the exact expansion T (FP64 sums), the
// analytic translation A and the network residual Y (physical units, from
// the same kernels the sweep runs), and the error of the expansion applied
// across the target: with rho = sqrt(3)/2 h_T / d (the target's half
// diagonal over the distance),
//   e = (|du| + rho |dJ| + rho^2/2 |dH|) / (|u| + rho |J| + rho^2/2 |H|),
// for A + Y (err_l) and for A alone (err_a); failures counted per class.
__global__ void judge_errors_kernel(JudgeSampleBufs B, const float* __restrict__ rec,
                                    const double* __restrict__ sums,
                                    const float* __restrict__ A, const float* __restrict__ Y,
                                    float h0, float h1, float tol, JudgeWords* W,
                                    float* __restrict__ err) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= 2 * B.cap) return;
  const int li = slot >= B.cap ? 1 : 0;
  const int q = slot - li * B.cap;
  if (q >= W->cnt[li]) return;
  double t[30];
  for (int c = 0; c < 30; ++c) t[c] = sums[static_cast<int64_t>(slot) * 30 + c];
  const float hT = li ? h1 : h0;
  const float3 cT = cell_center_rel(B.key[li][q], hT);
  const float* cs = rec + static_cast<int64_t>(B.cell[li][q]) * kRecFloats;
  const float dx = cT.x - cs[0], dy = cT.y - cs[1], dz = cT.z - cs[2];
  const float rho = 0.8660254f * hT * rsqrtf(dx * dx + dy * dy + dz * dz);
  float pa[30], pl[30];
  for (int c = 0; c < 30; ++c) {
    pa[c] = A[static_cast<int64_t>(slot) * 32 + c];
    pl[c] = pa[c] + (Y ? Y[static_cast<int64_t>(slot) * 32 + c] : 0.f);
  }
  const float el = expansion_error(pl, t, rho), ea = expansion_error(pa, t, rho);
  err[2 * slot] = el;
  err[2 * slot + 1] = ea;
  const int k = B.cls[li][q];
  atomicAdd(&W->checked, 1u);
  atomicAdd(&W->class_samples[k], 1u);
  if (!(el <= tol)) atomicAdd(&W->fail_learned[k], 1u);
  if (!(ea <= tol)) atomicAdd(&W->fail_analytic[k], 1u);
}

// Per class, from its sampled failure fractions (f_l with the network, f_a
// without): f_l <= kJudgeFailFraction keeps the network (action 0); else
// f_a <= kJudgeFailFraction drops the network for the class (1); else every
// pair of the class is summed directly in FP64 (2).  act is the table the
// sweep's translation and network kernels read (kept for the sweeps that are
// not judged).  unrepaired: the expected fraction of the pairs left above
// the tolerance, sum over the expanded classes of n_k f_k over sum n_k.
constexpr float kJudgeFailFraction = 0.25f;
__global__ void judge_decide_kernel(JudgeWords* W, const unsigned* __restrict__ hist,
                                    uint8_t* __restrict__ act, int learned) {
  const int k = threadIdx.x;
  float num = 0.f, den = 0.f;
  if (k < kJudgeClasses) {
    const unsigned ns = W->class_samples[k], nk = hist[k];
    int a = 0;
    float f = 0.f;
    if (ns > 0) {
      const float fl = static_cast<float>(W->fail_learned[k]) / ns;
      const float fa = static_cast<float>(W->fail_analytic[k]) / ns;
      if (fl <= kJudgeFailFraction) {
        a = 0;
        f = fl;
      } else if (learned && fa <= kJudgeFailFraction) {
        a = 1;
        f = fa;
      } else {
        a = 2;
      }
    }
    act[k] = static_cast<uint8_t>(a);
    W->action[k] = a;
    W->class_pairs[k] = nk;
    num = f * nk;
    den = static_cast<float>(nk);
  }
  for (int o = 16; o > 0; o >>= 1) {
    num += __shfl_xor_sync(0xffffffffu, num, o);
    den += __shfl_xor_sync(0xffffffffu, den, o);
  }
  if (k == 0) W->unrepaired = den > 0.f ? num / den : 0.f;
}

// After the sweep's expansions: a sampled pair of an expanded class whose
// applied expansion (A + Y, or A where the network was dropped) misses the
// tolerance is taken out of its target's expansion and queued for the FP64
// direct sum.  The applied error is summed for the report.
__global__ void judge_repair_kernel(JudgeSampleBufs B, const float* __restrict__ A,
                                    const float* __restrict__ Y, const float* __restrict__ err,
                                    float tol, const uint8_t* __restrict__ act, float* local0,
                                    float* local1, JudgeWords* W, FarJudge J) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= 2 * B.cap) return;
  const int li = slot >= B.cap ? 1 : 0;
  const int q = slot - li * B.cap;
  if (q >= W->cnt[li]) return;
  const int a = act[B.cls[li][q]];
  if (a == 2) return;  // already queued whole by the translation kernel
  const float e = err[2 * slot + (a == 0 ? 0 : 1)];
  atomicAdd(&W->applied, 1u);
  atomicAdd(reinterpret_cast<float*>(&W->err_sum_bits), e);
  atomicMax(&W->err_max_bits, __float_as_uint(e));
  if (e <= tol) return;
  const int t = B.tgt[li][q];
  float* L = (li ? local1 : local0) + static_cast<int64_t>(t) * 32;
  for (int c = 0; c < 30; ++c) {
    float p = A[static_cast<int64_t>(slot) * 32 + c];
    if (a == 0 && Y) p += Y[static_cast<int64_t>(slot) * 32 + c];
    atomicAdd(L + c, -p);
  }
  atomicAdd(&W->repaired, 1u);
  const int f = atomicAdd(J.nfb, 1);
  if (f < J.fb_cap)
    J.fb[f] = make_int2(t | (li << 30), B.cell[li][q]);
  else
    flag_status(kStatusCapacity);
}

// FP64 direct sums of the queued (target, cell) pairs at every particle of
// the target (a leaf, or a parent of leaves), added to the outputs.
// Persistent CTAs stride over (pair, slice, target phase) items: each pair's
// cell is cut into S slices of at least a minimum size (the surplus items of
// a small cell are skipped at once), and its targets into TP phases of eight
// (one per warp).  A short queue (the judge's repairs: a few pairs, some of
// them parents of hundreds of particles against cells of thousands) takes
// S = 64 slices of at least 32 particles and TP = 8 phases, so that a single
// pair spreads over hundreds of CTAs: FP64 runs at 1/64 of the FP32 rate, and
// one CTA per slice left a parent pair at ~0.2 ms.  A long queue (whole
// classes) takes S = 8 slices of at least 128 and one phase.  Each warp takes
// whole targets: its lanes stride over the slice, reduce by shuffles and add
// one atomic per output component, with no block-wide barrier per target.
constexpr int kFallbackThreads = 256;
constexpr int kFallbackShortQueue = 2048;
struct FallbackTargets {
  const int* start[2];
  const int* count[2];
};
template <int MODE, int KERNEL>
__global__ void __launch_bounds__(kFallbackThreads) fallback_kernel(
    const int2* __restrict__ fallback, const int* __restrict__ n_fallback, int fb_cap,
    FallbackTargets tg, const int* __restrict__ cell_start, const int* __restrict__ cell_count,
    const int* __restrict__ perm, const double* __restrict__ pos,
    const double* __restrict__ alpha, const double* __restrict__ sigma,
    const double* __restrict__ tgt_gamma, double* __restrict__ out_a,
    double* __restrict__ out_b) {
  using namespace pair;
  constexpr int NC = ModeInfo<MODE>::ncomp;
  constexpr int NA = ModeInfo<MODE>::na;
  constexpr bool NEED_FPR = ModeInfo<MODE>::need_fpr;
  constexpr bool NEED_TG = ModeInfo<MODE>::need_tg;
  constexpr double kC = -0.07957747154594767;
  const int nq = min(*n_fallback, fb_cap);
  const bool short_q = nq < kFallbackShortQueue;
  const int S = short_q ? 64 : 8, TP = short_q ? 8 : 1, min_slice = short_q ? 32 : 128;
  const int64_t items = static_cast<int64_t>(nq) * S * TP;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int kWarps = kFallbackThreads / 32;
  for (int64_t w = blockIdx.x; w < items; w += gridDim.x) {
    const int2 pr = fallback[w / (S * TP)];
    const int rem = static_cast<int>(w % (S * TP));
    const int sl = rem / TP, tp = rem - sl * TP;
    const int li = (pr.x >> 30) & 1, tgt = pr.x & ((1 << 30) - 1);
    const int t0 = (li ? tg.start[1] : tg.start[0])[tgt];
    const int nt = (li ? tg.count[1] : tg.count[0])[tgt];
    const int c0 = cell_start[pr.y], cn = cell_count[pr.y];
    const int per = max(min_slice, (cn + S - 1) / S);
    const int64_t s0_64 = c0 + static_cast<int64_t>(sl) * per;
    if (s0_64 >= c0 + cn) continue;
    const int s0 = static_cast<int>(s0_64);
    const int ns = min(per, c0 + cn - s0);
    for (int ti = tp * kWarps + wid; ti < nt; ti += kWarps * TP) {
      const int i = perm[t0 + ti];
      const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
      double gx = 0.0, gy = 0.0, gz = 0.0;
      if (NEED_TG) {
        gx = tgt_gamma[3 * i];
        gy = tgt_gamma[3 * i + 1];
        gz = tgt_gamma[3 * i + 2];
      }
      double acc[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = 0.0;
      for (int q = lane; q < ns; q += 32) {
        const int j = perm[s0 + q];
        const double dx = x - pos[3 * j], dy = y - pos[3 * j + 1], dz = z - pos[3 * j + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double sg = sigma[j];
        const double s2 = sg * sg;
        const double k2 = KERNEL == FVX_KERNEL_WINCKELMANS ? 2.5 * s2 : 1.0 / sg;
        double f, fpr = 0.0;
        core_f64<KERNEL, NEED_FPR>(r2, s2, k2, f, fpr);
        accumulate<MODE, double>(acc, dx, dy, dz, r2, kC * alpha[3 * j], kC * alpha[3 * j + 1],
                                 kC * alpha[3 * j + 2], f, fpr, gx, gy, gz);
      }
#pragma unroll
      for (int c = 0; c < NC; ++c)
        for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (lane != c) continue;
        if (c < NA)
          atomicAdd(out_a + static_cast<int64_t>(i) * NA + c, acc[c]);
        else
          atomicAdd(out_b + static_cast<int64_t>(i) * (NC - NA) + (c - NA), acc[c]);
      }
    }
  }
}

}  // namespace tree

// ---- host orchestration --------------------------------------------------------------
namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

int grow(DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return FVX_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t c = bytes + bytes / 4 + 4096;
  FVX_CUDA_TRY(cudaMalloc(&b.p, c));
  b.cap = c;
  return FVX_OK;
}

template <typename T>
T* P(DevBuf& b, size_t off = 0) {
  return reinterpret_cast<T*>(static_cast<char*>(b.p) + off);
}

// Same arithmetic as fluxvortex_gb300/tree_params.py:grid_params.
void grid_params(const double lo[3], const double hi[3], int64_t n, int leaf_target, int* L_out,
                 double* h_out, double origin[3]) {
  double ext[3], emax = 0.0;
  for (int c = 0; c < 3; ++c) {
    ext[c] = fmax(hi[c] - lo[c], 1e-12);
    emax = fmax(emax, ext[c]);
  }
  double vol = 1.0;
  for (int c = 0; c < 3; ++c) vol *= fmax(ext[c], emax * 1e-3);
  const double h_target = pow(vol * leaf_target / static_cast<double>(n > 0 ? n : 1), 1.0 / 3.0);
  // leaf size c 2^k, c in {1, 5/4, 3/2, 7/4}: the candidate nearest to
  // h_target in ratio (boundaries at the geometric means, compared squared)
  int e = 0;
  const double x = 2.0 * frexp(h_target, &e);  // h_target = x 2^(e-1), x in [1, 2)
  const double cand[5] = {1.0, 1.25, 1.5, 1.75, 2.0};
  int ci = 0;
  while (ci < 4 && x * x > cand[ci] * cand[ci + 1]) ++ci;
  double h = ldexp(cand[ci], e - 1);
  int L = 1;
  for (;;) {
    double span = 0.0;
    for (int c = 0; c < 3; ++c) {
      origin[c] = floor(lo[c] / h) * h;
      span = fmax(span, hi[c] - origin[c]);
    }
    L = 1;
    while (h * static_cast<double>(1 << L) <= span) ++L;
    if (L <= 10) break;
    h *= 2.0;
  }
  *L_out = L;
  *h_out = h;
}

}  // namespace

int mlp_farfield_launch(const FarPairs& a, const FarPairs& b, const float* rec, const void* W,
                        const float* bias, cudaStream_t s, const FarJudge& judge = FarJudge{});
int mlp_pair_targets_launch(int npairs, int stride, const int* pair_leaf, const int* pair_cell,
                            const uint32_t* tgt_key, float h_tgt, const uint32_t* leaf_key,
                            const float* rec, const int* cell_start,
                            const int* cell_count, const float4* sp, const float4* sa,
                            const int* leaf_of_particle, float h, void* X, float* T,
                            float* A, float* scale, double* partial, int slices,
                            cudaStream_t s);
int m2l_farfield_launch(const FarPairs& a, const FarPairs& b, const float* rec, cudaStream_t s,
                        const FarJudge& judge = FarJudge{});
int judge_sums_launch(const JudgeSampleView& S, const uint32_t* leaf_key, const int* cell_start,
                      const int* cell_count, const float4* sp, const float4* sa,
                      const int* leaf_of_particle, float h, double* sums, int* off,
                      cudaStream_t s);

}  // namespace fvx

struct fvx_tree {
  int device = 0;
  fvx::DevBuf keys0, keys1, idx0, idx1, table, scan_tmp, flags, cid, levels, counts, rec, sp, sa,
      sg, lists_meta, near_list, far_list, bbox;
  int64_t stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the last evaluation launch
  // far-field method of the pairs beyond theta_l (FVX_FAR_*)
  int far_method = FVX_FAR_M2P;
  double sigma_min = 0.0;  // smallest core at the last full build
  const void* mlp_W = nullptr;
  const float* mlp_b = nullptr;
  double theta_l = 0.0;
  cudaEvent_t ev2 = nullptr, ev3 = nullptr;  // around the local-expansion stage
  // the FP64 judge of the local-expansion path and its FP64 fallback: samples
  // per judged sweep (spread over the classes), the tolerance, the per-mode
  // class actions (kept between judged sweeps), the pair classes, the sample
  // buffers, the fallback queue
  int val_samples = 256;
  double val_tol = 0.1;
  bool judge_armed = false;      // a judged sweep has set the action tables
  uint32_t judge_seq = 0;        // seeds the samples of each judged sweep
  fvx::DevBuf judge_act, judge_cls, judge_hist, judge_words, judge_samp, judge_A, judge_Y,
      judge_err, fb_queue, fb_count;
  int last_judged = 0;           // samples judged by the last judged sweep
  // two-level traversal: per-parent lists and expansions
  fvx::DevBuf dual_meta, par_par, par_cell, parent_local;
  fvx::DevBuf cen;  // cell centres in units of h/2 (dual traversal)
  fvx::DevBuf eval_next;  // leaf counter of the evaluation kernel
  fvx::DevBuf leaf_order, order_table;  // evaluation order of the leaves (+ sort scratch)
  fvx::DevBuf pair_partial;  // slices of the FP64 exact-expansion sums
  int n_parent_pairs = 0;
  fvx::DevBuf lrn_meta, lrn_leaf, lrn_cell, leaf_local;
  fvx::DevBuf lrn_slot, par_slot;  // one-pass (slot) form of the two-level lists
  fvx::DevBuf res_slot, res_cnt;   // per parent: residual cells for its leaves
  int slot_near = 512, slot_lrn = 1024, slot_par = 1024;  // 0: counting pass always
  int n_learned = 0;
  // the structure of the last full build (grid, sort, cells, interaction
  // lists), reused by a sweep hinted to have the same positions
  bool reuse_next = false;
  struct Structure {
    bool valid = false;
    const double* pos = nullptr;
    int n = 0, leaf_target = 0, far_method = 0;
    double theta = 0.0, theta_l = 0.0;
    int L = 0, total_cells = 0, nleaf = 0;
    double h = 0.0, origin[3] = {0.0, 0.0, 0.0};
    int cap[11] = {}, base[12] = {}, ncells[11] = {};
    const int* perm = nullptr;
    int64_t near_total = 0, far_total = 0, lrn_total = 0, par_total = 0;
  } st;
  // the last sweep's tree, for sampling training pairs
  int last_L = 0, last_nleaf = 0;
  double last_h = 0.0;
  const uint32_t* last_leaf_key = nullptr;
  const uint32_t* last_par_key = nullptr;  // level L-1 keys (two-level lists)
  const int* last_cell_start = nullptr;
  const int* last_cell_count = nullptr;
  const int* last_cid = nullptr;
};

namespace fvx {
namespace {

template <int KERNEL>
void launch_gather(int n, const int* perm, const int* leaf_of, const uint32_t* leaf_key,
                   tree::Grid g, const double* pos, const double* alpha, const double* sigma,
                   const double* tgam, float4* sp, float4* sa, float4* sg, cudaStream_t s) {
  tree::gather_kernel<KERNEL><<<(n + 255) / 256, 256, 0, s>>>(n, perm, leaf_of, leaf_key, g, pos,
                                                             alpha, sigma, tgam, sp, sa, sg);
}

// Resident CTAs: the occupancy limit per SM times the SMs (at most one per leaf).
template <typename K>
int resident_grid(K kernel, int nleaf) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, tree::kEvalThreads, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int64_t g = static_cast<int64_t>(per_sm) * device_sm_count();
  return static_cast<int>(g < nleaf ? g : nleaf);
}

// Targets per thread: leaves of at most ~40 particles on average fill one
// 32-target chunk per warp better than two.
template <int KERNEL, int TPT>
void launch_eval_tpt(int mode, int nleaf, const tree::EvalArgs& A, bool factored,
                     cudaStream_t s) {
  using namespace tree;
  constexpr bool F = KERNEL == FVX_KERNEL_WINCKELMANS && TPT == 2;  // the paired kernels
  switch (mode) {
    case FVX_PAIR_VELOCITY: {
      auto k = eval_kernel<FVX_PAIR_VELOCITY, KERNEL, TPT>;
      if constexpr (F)
        if (factored) k = eval_kernel_factored<FVX_PAIR_VELOCITY, KERNEL, 4>;
      k<<<resident_grid(k, nleaf), kEvalThreads, 0, s>>>(A);
      break;
    }
    case FVX_PAIR_STRETCH: {
      auto k = eval_kernel<FVX_PAIR_STRETCH, KERNEL, TPT>;
      if constexpr (F)
        if (factored) k = eval_kernel_factored<FVX_PAIR_STRETCH, KERNEL, TPT>;
      k<<<resident_grid(k, nleaf), kEvalThreads, 0, s>>>(A);
      break;
    }
    case FVX_PAIR_VELOCITY_STRETCH: {
      auto k = eval_kernel<FVX_PAIR_VELOCITY_STRETCH, KERNEL, TPT>;
      k<<<resident_grid(k, nleaf), kEvalThreads, 0, s>>>(A);
      break;
    }
    default: {
      auto k = eval_kernel<FVX_PAIR_VORTICITY, KERNEL, TPT>;
      k<<<resident_grid(k, nleaf), kEvalThreads, 0, s>>>(A);
      break;
    }
  }
}

template <int KERNEL>
void launch_eval(int mode, int nleaf, int n, const tree::EvalArgs& A, bool factored,
                 cudaStream_t s) {
  // Winckelmans velocity and stretching and the Gaussian-erf vorticity: the
  // paired f32x2 kernels, whose source phases keep small leaves' slots busy.
  // Otherwise two targets per thread once leaves average more than ~40
  // particles; at fewer, one target per thread wastes fewer lanes.
  const bool paired = (KERNEL == FVX_KERNEL_WINCKELMANS &&
                       (mode == FVX_PAIR_VELOCITY || mode == FVX_PAIR_STRETCH)) ||
                      (KERNEL == FVX_KERNEL_GAUSSIANERF && mode == FVX_PAIR_VORTICITY);
  if (!paired && n <= 40 * nleaf)
    launch_eval_tpt<KERNEL, 1>(mode, nleaf, A, false, s);
  else
    launch_eval_tpt<KERNEL, 2>(mode, nleaf, A, factored, s);
}

template <int KERNEL>
void launch_fallback(int mode, int grid, const int2* fb, const int* nfb, int fb_cap,
                     tree::FallbackTargets tgs, const int* cell_start, const int* cell_count,
                     const int* perm, const double* pos, const double* alpha,
                     const double* sigma, const double* tg, double* out_a, double* out_b,
                     cudaStream_t s) {
  using namespace tree;
#define FVX_FB(M)                                                                        \
  fallback_kernel<M, KERNEL><<<grid, kFallbackThreads, 0, s>>>(fb, nfb, fb_cap, tgs,     \
                                                               cell_start, cell_count,   \
                                                               perm, pos, alpha, sigma,  \
                                                               tg, out_a, out_b)
  switch (mode) {
    case FVX_PAIR_VELOCITY:
      FVX_FB(FVX_PAIR_VELOCITY);
      break;
    case FVX_PAIR_STRETCH:
      FVX_FB(FVX_PAIR_STRETCH);
      break;
    case FVX_PAIR_VELOCITY_STRETCH:
      FVX_FB(FVX_PAIR_VELOCITY_STRETCH);
      break;
    default:
      FVX_FB(FVX_PAIR_VORTICITY);
      break;
  }
#undef FVX_FB
}

}  // namespace

int tree_sweep(fvx_tree* T, int mode, int kernel, const double* pos, const double* alpha,
               const double* sigma, const double* tgt_gamma, int64_t n64, double theta,
               int leaf_target, double* out_a, double* out_b, int64_t* stats, cudaStream_t s) {
  using namespace tree;
  FVX_ARG_CHECK(T != nullptr, "null tree handle");
  FVX_ARG_CHECK(mode == FVX_PAIR_VELOCITY || mode == FVX_PAIR_STRETCH ||
                    mode == FVX_PAIR_VELOCITY_STRETCH || mode == FVX_PAIR_VORTICITY,
                "treecode supports the velocity, stretch, velocity+stretch and vorticity sweeps");
  FVX_ARG_CHECK(kernel == FVX_KERNEL_WINCKELMANS || kernel == FVX_KERNEL_GAUSSIANERF,
                "unknown kernel %d", kernel);
  FVX_ARG_CHECK(theta > 0.0 && theta < 1.0 && leaf_target >= 1, "bad theta / leaf size");
  FVX_ARG_CHECK(n64 >= 0 && n64 <= (int64_t(1) << 22), "treecode supports up to 2^22 particles");
  const int n = static_cast<int>(n64);
  if (n == 0) return FVX_OK;
  const bool need_tg = mode == FVX_PAIR_STRETCH || mode == FVX_PAIR_VELOCITY_STRETCH;
  FVX_ARG_CHECK(pos && alpha && sigma && out_a && (!need_tg || tgt_gamma) &&
                    (mode != FVX_PAIR_VELOCITY_STRETCH || out_b),
                "null array");
  int rc;
  // A sweep hinted to have the last full build's positions (same array,
  // count, opening angles, leaf size and far-field method) reuses its grid,
  // sort, cells and interaction lists; strengths, cores and target strengths
  // are gathered anew and the moments, expansions and evaluation recomputed.
  auto& ST = T->st;
  const bool reuse = T->reuse_next && ST.valid && ST.pos == pos && ST.n == n &&
                     ST.theta == theta && ST.leaf_target == leaf_target &&
                     ST.far_method == T->far_method && ST.theta_l == T->theta_l;
  T->reuse_next = false;
  int L = 0, total_cells = 0, nleaf = 0;
  double h = 0.0, origin[3] = {0.0, 0.0, 0.0};
  int cap[11] = {}, base[12] = {}, ncells[11] = {};
  const int* perm = nullptr;
  int* lvb = nullptr;
  auto level = [&](int l) {
    Level v;
    v.start = lvb + base[l];
    v.count = lvb + total_cells + base[l];
    v.key = reinterpret_cast<uint32_t*>(lvb + 2 * total_cells + base[l]);
    v.child_lo = lvb + 3 * total_cells + base[l];
    v.child_hi = lvb + 4 * total_cells + base[l];
    return v;
  };
  if (reuse) {
    L = ST.L;
    total_cells = ST.total_cells;
    nleaf = ST.nleaf;
    h = ST.h;
    for (int c = 0; c < 3; ++c) origin[c] = ST.origin[c];
    for (int l = 0; l < 11; ++l) {
      cap[l] = ST.cap[l];
      ncells[l] = ST.ncells[l];
    }
    for (int l = 0; l < 12; ++l) base[l] = ST.base[l];
    perm = ST.perm;
    lvb = P<int>(T->levels);
  } else {
  ST.valid = false;
  // 1. bounding box -> grid
  const int nbb = 256;
  if ((rc = grow(T->bbox, sizeof(double) * (7 * nbb + 8)))) return rc;
  unsigned* nonfinite = reinterpret_cast<unsigned*>(P<double>(T->bbox) + 7 * nbb + 7);
  FVX_CUDA_TRY(cudaMemsetAsync(nonfinite, 0, sizeof(unsigned), s));
  bbox_partial_kernel<<<nbb, 256, 0, s>>>(n, pos, sigma, P<double>(T->bbox), nonfinite);
  FVX_LAUNCH_CHECK();
  bbox_final_kernel<<<1, kBboxFinalThreads, 0, s>>>(nbb, P<double>(T->bbox),
                                                    P<double>(T->bbox) + 7 * nbb);
  FVX_LAUNCH_CHECK();
  double lohi[7];
  unsigned nbad = 0;
  FVX_CUDA_TRY(cudaMemcpyAsync(lohi, P<double>(T->bbox) + 7 * nbb, sizeof(lohi),
                               cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&nbad, nonfinite, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  // a non-finite position would otherwise collapse the grid (all keys in one
  // cell) and turn the sweep into an all-pairs sum on a few CTAs
  FVX_ARG_CHECK(nbad == 0, "treecode: %u particles with non-finite positions", nbad);
  grid_params(lohi, lohi + 3, n, leaf_target, &L, &h, origin);
  T->sigma_min = lohi[6];
  // level capacities and bases
  cap[L] = n;
  for (int l = L - 1; l >= 0; --l) {
    const int64_t full = int64_t(1) << (3 * l);
    cap[l] = static_cast<int>(full < cap[l + 1] ? full : cap[l + 1]);
  }
  base[0] = 0;
  for (int l = 0; l <= L; ++l) base[l + 1] = base[l] + cap[l];
  total_cells = base[L + 1];
  const int nblk = (n + kSortItems - 1) / kSortItems;
  if ((rc = grow(T->keys0, 4 * size_t(n))) || (rc = grow(T->keys1, 4 * size_t(n))) ||
      (rc = grow(T->idx0, 4 * size_t(n))) || (rc = grow(T->idx1, 4 * size_t(n))) ||
      (rc = grow(T->table, 4 * size_t(256) * nblk * 2)) ||
      (rc = grow(T->scan_tmp, 4 * size_t(2 * kScanBlock))) ||
      (rc = grow(T->flags, 4 * size_t(n))) || (rc = grow(T->cid, 4 * size_t(n))) ||
      (rc = grow(T->levels, 4 * size_t(total_cells) * 5)) ||
      (rc = grow(T->counts, 4 * 16)) ||
      (rc = grow(T->rec, 4 * size_t(total_cells) * kRecFloats)) ||
      (rc = grow(T->sp, 16 * size_t(n))) || (rc = grow(T->sa, 16 * size_t(n))) ||
      (rc = grow(T->sg, 16 * size_t(n))))
    return rc;
  // 2. keys + stable radix sort: a pass per 8 bits of the 3L-bit keys (the result in
  //    ka / ia, the other pair free)
  keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, origin[0], origin[1], origin[2], 1.0 / h, L,
                                              P<uint32_t>(T->keys0), P<int>(T->idx0));
  FVX_LAUNCH_CHECK();
  uint32_t *ka = P<uint32_t>(T->keys0), *kb = P<uint32_t>(T->keys1);
  int *ia = P<int>(T->idx0), *ib = P<int>(T->idx1);
  int* table = P<int>(T->table);
  int* table_ex = table + 256 * nblk;
  const int passes = (3 * L + 7) / 8;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = 8 * pass;
    radix_hist_kernel<<<nblk, 256, 0, s>>>(ka, n, shift, nblk, table);
    FVX_LAUNCH_CHECK();
    if ((rc = scan_ints(table, 256 * nblk, table_ex, 0, P<int>(T->scan_tmp), s))) return rc;
    radix_scatter_kernel<<<nblk, 256, 0, s>>>(ka, ia, n, shift, nblk, table_ex, kb, ib);
    FVX_LAUNCH_CHECK();
    uint32_t* tk = ka;
    ka = kb;
    kb = tk;
    int* ti = ia;
    ia = ib;
    ib = ti;
  }
  const uint32_t* keys = ka;  // sorted
  perm = ia;
  // 3. cells: leaves from particles, parents from children
  lvb = P<int>(T->levels);
  int* ncells_d = P<int>(T->counts);
  int* flag = P<int>(T->flags);
  int* cid = P<int>(T->cid);
  flags_kernel<<<(n + 255) / 256, 256, 0, s>>>(keys, nullptr, n, 0, flag);
  FVX_LAUNCH_CHECK();
  if ((rc = scan_ints(flag, n, cid, 1, P<int>(T->scan_tmp), s))) return rc;
  Level leaves = level(L);
  leaf_cells_kernel<<<(n + 255) / 256, 256, 0, s>>>(keys, n, flag, cid, leaves, ncells_d + L);
  FVX_LAUNCH_CHECK();
  cell_counts_kernel<<<(n + 255) / 256, 256, 0, s>>>(leaves, ncells_d + L, n);
  FVX_LAUNCH_CHECK();
  // parent levels reuse flag (as flags) and the scan buffer; the leaf ids of
  // the particles (cid) are kept for the gather
  int* pflag = reinterpret_cast<int*>(kb);  // the sort's free pair
  int* pid = ib;
  for (int l = L - 1; l >= 0; --l) {
    Level ch = level(l + 1), par = level(l);
    const int cc = cap[l + 1];
    parent_flags_kernel<<<(cc + 255) / 256, 256, 0, s>>>(ch, ncells_d + l + 1, cc, pflag);
    FVX_LAUNCH_CHECK();
    if ((rc = scan_ints(pflag, cc, pid, 1, P<int>(T->scan_tmp), s))) return rc;
    parent_cells_kernel<<<(cc + 255) / 256, 256, 0, s>>>(ch, ncells_d + l + 1, pflag, pid, par,
                                                         ncells_d + l);
    FVX_LAUNCH_CHECK();
    parent_counts_kernel<<<(cap[l] + 255) / 256, 256, 0, s>>>(ch, par, ncells_d + l);
    FVX_LAUNCH_CHECK();
  }
  FVX_CUDA_TRY(cudaMemcpyAsync(ncells, ncells_d, sizeof(int) * (L + 1), cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  nleaf = ncells[L];
  }
  int* ncells_d = P<int>(T->counts);
  int* cid = P<int>(T->cid);
  Level leaves = level(L);
  // 4. sorted FP32 records
  Grid g{origin[0], origin[1], origin[2], h, L};
  float4 *sp = P<float4>(T->sp), *sa = P<float4>(T->sa), *sg = P<float4>(T->sg);
  if (kernel == FVX_KERNEL_WINCKELMANS)
    launch_gather<FVX_KERNEL_WINCKELMANS>(n, perm, cid, leaves.key, g, pos, alpha, sigma,
                                          need_tg ? tgt_gamma : nullptr, sp, sa, sg, s);
  else
    launch_gather<FVX_KERNEL_GAUSSIANERF>(n, perm, cid, leaves.key, g, pos, alpha, sigma,
                                          need_tg ? tgt_gamma : nullptr, sp, sa, sg, s);
  FVX_LAUNCH_CHECK();
  // 5. moments: leaves, then M2M up the levels
  float* rec = P<float>(T->rec);
  leaf_moments_kernel<<<(nleaf * 32 + 255) / 256, 256, 0, s>>>(
      leaves, ncells_d + L, static_cast<float>(h), sp, sa, rec + int64_t(base[L]) * kRecFloats);
  FVX_LAUNCH_CHECK();
  for (int l = L - 1; l >= 0; --l) {
    const float hl = static_cast<float>(h * static_cast<double>(1 << (L - l)));
    m2m_kernel<<<(ncells[l] + 127) / 128, 128, 0, s>>>(
        level(l), ncells_d + l, hl, rec + int64_t(base[l + 1]) * kRecFloats,
        rec + int64_t(base[l]) * kRecFloats);
    FVX_LAUNCH_CHECK();
  }
  // 6. interaction lists
  TreeView V;
  V.L = L;
  V.h = h;
  V.mac_k = 0.75 / (theta * theta);
  for (int l = 0; l <= L + 1 && l < 11; ++l) V.base[l] = base[l];
  for (int l = 0; l <= L; ++l) V.ncell[l] = ncells[l];
  V.start = lvb;
  V.count = lvb + total_cells;
  V.key = reinterpret_cast<const uint32_t*>(lvb + 2 * total_cells);
  V.child_lo = lvb + 3 * total_cells;
  V.child_hi = lvb + 4 * total_cells;
  V.cen = nullptr;
  const bool learned = T->far_method != FVX_FAR_M2P && T->theta_l > 0.0;
  V.mac_kl = learned ? 0.75 / (T->theta_l * T->theta_l) : 0.0;
  // integer acceptance thresholds per source level: (h_T + h_S)^2 in (h/2)^2
  // units is 4 (1 + 2^(L-l))^2; d2 > k x that <=> d2 > floor(k x that)
  for (int l = 0; l <= L; ++l) {
    const double hs2 = 4.0 * (1.0 + static_cast<double>(1 << (L - l))) *
                       (1.0 + static_cast<double>(1 << (L - l)));
    const double tf = floor(V.mac_k * hs2), tl = floor(V.mac_kl * hs2);
    V.thr_far[l] = tf < 2147483647.0 ? static_cast<int>(tf) : 2147483647;
    V.thr_lrn[l] = learned ? (tl < 2147483647.0 ? static_cast<int>(tl) : 2147483647)
                           : 2147483647;
  }
  V.learned_only = learned ? 1 : 0;
  // two-level traversal when every accepted cell takes the local expansion
  bool dual = learned && L >= 1;
  for (int l = 0; l <= L; ++l) {
    if (V.thr_lrn[l] != V.thr_far[l]) dual = false;
    // (h_P + h_S)^2 in (h/2)^2 units for a parent of leaves (size 2h)
    const double hp2 = 4.0 * (2.0 + static_cast<double>(1 << (L - l))) *
                       (2.0 + static_cast<double>(1 << (L - l)));
    const double tp = floor(V.mac_k * hp2);
    V.thr_par[l] = tp < 2147483647.0 ? static_cast<int>(tp) : 2147483647;
  }
  const int npar = dual ? ncells[L - 1] : 0;
  if ((rc = grow(T->lists_meta, 4 * size_t(nleaf) * 4 + 64))) return rc;
  if (learned && (rc = grow(T->lrn_meta, 4 * size_t(nleaf) * 2 + 64))) return rc;
  if (dual && (rc = grow(T->dual_meta, 4 * (2 * size_t(npar) + size_t(nleaf)) + 64))) return rc;
  LearnedLists LL{nullptr, nullptr, nullptr, nullptr, 0};
  if (learned) {
    LL.cnt = P<int>(T->lrn_meta);
    LL.off = P<int>(T->lrn_meta) + nleaf;
  }
  int* near_cnt = P<int>(T->lists_meta);
  int* far_cnt = near_cnt + nleaf;
  int* near_off = far_cnt + nleaf;
  int* far_off = near_off + nleaf;
  unsigned* ovf = reinterpret_cast<unsigned*>(far_off + nleaf);  // + 2 x u64 work counters
  int* par_cnt = dual ? P<int>(T->dual_meta) : nullptr;
  int* par_off = dual ? par_cnt + npar : nullptr;
  int* leaf_parent = dual ? par_off + npar : nullptr;
  int64_t near_total = 0, far_total = 0, lrn_total = 0, par_total = 0;
  if (reuse) {
    near_total = ST.near_total;
    far_total = ST.far_total;
    lrn_total = ST.lrn_total;
    par_total = ST.par_total;
  } else {
  // Two-level lists in one pass: each leaf's near leaves and local cells and
  // each parent's cells go to fixed-capacity slots (no counting pass); the
  // local-expansion pairs are then compacted into flat lists ordered by
  // target.  A slot overflow falls back to the counting pass and exact lists.
  if (dual) {
    // what every leaf's traversal reads: cell centres and its parent
    if ((rc = grow(T->cen, 16 * size_t(total_cells)))) return rc;
    V.cen = P<int4>(T->cen);
    cell_centres_kernel<<<(total_cells + 255) / 256, 256, 0, s>>>(V, total_cells, P<int4>(T->cen));
    FVX_LAUNCH_CHECK();
    leaf_parents_kernel<<<(npar + 127) / 128, 128, 0, s>>>(V, leaf_parent);
    FVX_LAUNCH_CHECK();
  }
  bool slotted = false;
  if (dual && T->slot_near > 0 && T->slot_lrn > 0 && T->slot_par > 0) {
    const int kSlotNear = T->slot_near, kSlotLrn = T->slot_lrn, kSlotPar = T->slot_par;
    if ((rc = grow(T->near_list, 4 * size_t(nleaf) * kSlotNear)) ||
        (rc = grow(T->lrn_slot, 4 * size_t(nleaf) * kSlotLrn)) ||
        (rc = grow(T->par_slot, 4 * size_t(npar) * kSlotPar)))
      return rc;
    FVX_CUDA_TRY(cudaMemsetAsync(ovf, 0, 24, s));
    FVX_CUDA_TRY(cudaMemsetAsync(far_cnt, 0, sizeof(int) * size_t(nleaf), s));
    DualLists D{};
    D.near_cnt = near_cnt;
    D.lrn_cnt = LL.cnt;
    D.par_cnt = par_cnt;
    D.near_idx = P<int>(T->near_list);
    D.lrn_cell = P<int>(T->lrn_slot);
    D.par_cell = P<int>(T->par_slot);
    D.leaf_parent = leaf_parent;
    D.slot_near = kSlotNear;
    D.slot_lrn = kSlotLrn;
    D.slot_par = kSlotPar;
    // parent-level walk once per parent, then each leaf's residual cells
    constexpr int kSlotRes = 1024;
    if ((rc = grow(T->res_slot, 4 * size_t(npar) * kSlotRes)) ||
        (rc = grow(T->res_cnt, 4 * size_t(npar))))
      return rc;
    traverse_parents_kernel<<<(npar + kParWarps - 1) / kParWarps, kParWarps * 32, 0, s>>>(
        V, par_cnt, P<int>(T->par_slot), kSlotPar, P<int>(T->res_cnt), P<int>(T->res_slot),
        kSlotRes, ovf);
    FVX_LAUNCH_CHECK();
    traverse_residual_kernel<<<(npar + kParWarps - 1) / kParWarps, kParWarps * 32, 0, s>>>(
        V, D, P<int>(T->res_cnt), P<int>(T->res_slot), kSlotRes, ovf);
    FVX_LAUNCH_CHECK();
    iota_scaled_kernel<<<(nleaf + 255) / 256, 256, 0, s>>>(nleaf, kSlotNear, near_off);
    FVX_LAUNCH_CHECK();
    if ((rc = scan_ints(LL.cnt, nleaf, P<int>(T->lrn_meta) + nleaf, 0, P<int>(T->scan_tmp), s)))
      return rc;
    if ((rc = scan_ints(par_cnt, npar, par_off, 0, P<int>(T->scan_tmp), s))) return rc;
    // the near total through a scan into far_off (no far cells on this path)
    if ((rc = scan_ints(near_cnt, nleaf, far_off, 0, P<int>(T->scan_tmp), s))) return rc;
    int tl[6] = {0, 0, 0, 0, 0, 0};
    unsigned flags = 0;
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[0], LL.cnt + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[1], LL.off + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[2], par_cnt + npar - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[3], par_off + npar - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[4], near_cnt + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&tl[5], far_off + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&flags, ovf, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaStreamSynchronize(s));
    if (!(flags & 4u)) {
      near_total = int64_t(tl[4]) + tl[5];
      far_total = 0;
      lrn_total = int64_t(tl[0]) + tl[1];
      par_total = int64_t(tl[2]) + tl[3];
      if ((rc = grow(T->lrn_leaf, 4 * size_t(lrn_total + 1))) ||
          (rc = grow(T->lrn_cell, 4 * size_t(lrn_total + 1))) ||
          (rc = grow(T->par_par, 4 * size_t(par_total + 1))) ||
          (rc = grow(T->par_cell, 4 * size_t(par_total + 1))))
        return rc;
      compact_slots_kernel<<<(nleaf * 32 + 255) / 256, 256, 0, s>>>(
          nleaf, kSlotLrn, LL.cnt, LL.off, P<int>(T->lrn_slot), P<int>(T->lrn_leaf),
          P<int>(T->lrn_cell));
      FVX_LAUNCH_CHECK();
      compact_slots_kernel<<<(npar * 32 + 255) / 256, 256, 0, s>>>(
          npar, kSlotPar, par_cnt, par_off, P<int>(T->par_slot), P<int>(T->par_par),
          P<int>(T->par_cell));
      FVX_LAUNCH_CHECK();
      T->n_learned = static_cast<int>(lrn_total);
      T->n_parent_pairs = static_cast<int>(par_total);
      slotted = true;
    }
  }
  if (!slotted) {
  FVX_CUDA_TRY(cudaMemsetAsync(ovf, 0, 24, s));
  DualLists D{};
  if (dual) {
    // no per-target far cells on this path
    FVX_CUDA_TRY(cudaMemsetAsync(far_cnt, 0, sizeof(int) * size_t(nleaf), s));
    D.near_cnt = near_cnt;
    D.lrn_cnt = LL.cnt;
    D.par_cnt = par_cnt;
    D.near_off = near_off;
    D.lrn_off = LL.off;
    D.par_off = par_off;
    D.leaf_parent = leaf_parent;
    traverse_dual_kernel<false><<<(nleaf + 127) / 128, 128, 0, s>>>(V, D, ovf);
  } else {
    traverse_kernel<false><<<(nleaf + 127) / 128, 128, 0, s>>>(
        V, nullptr, nullptr, near_cnt, far_cnt, nullptr, nullptr, 0, 0, ovf, LL);
  }
  FVX_LAUNCH_CHECK();
  if ((rc = scan_ints(near_cnt, nleaf, near_off, 0, P<int>(T->scan_tmp), s))) return rc;
  if ((rc = scan_ints(far_cnt, nleaf, far_off, 0, P<int>(T->scan_tmp), s))) return rc;
  int ltail[4] = {0, 0, 0, 0};
  if (learned) {
    if ((rc = scan_ints(LL.cnt, nleaf, P<int>(T->lrn_meta) + nleaf, 0, P<int>(T->scan_tmp), s)))
      return rc;
    FVX_CUDA_TRY(cudaMemcpyAsync(&ltail[0], LL.cnt + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&ltail[1], LL.off + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
  }
  if (dual) {
    if ((rc = scan_ints(par_cnt, npar, par_off, 0, P<int>(T->scan_tmp), s))) return rc;
    FVX_CUDA_TRY(cudaMemcpyAsync(&ltail[2], par_cnt + npar - 1, 4, cudaMemcpyDeviceToHost, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(&ltail[3], par_off + npar - 1, 4, cudaMemcpyDeviceToHost, s));
  }
  int tail[4];
  FVX_CUDA_TRY(cudaMemcpyAsync(&tail[0], near_cnt + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&tail[1], near_off + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&tail[2], far_cnt + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&tail[3], far_off + nleaf - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  near_total = int64_t(tail[0]) + tail[1];
  far_total = int64_t(tail[2]) + tail[3];
  FVX_ARG_CHECK(near_total < (int64_t(1) << 31) && far_total < (int64_t(1) << 31),
                "interaction lists too long");
  if ((rc = grow(T->near_list, 4 * size_t(near_total + 1))) ||
      (rc = grow(T->far_list, 4 * size_t(far_total + 1))))
    return rc;
  lrn_total = int64_t(ltail[0]) + ltail[1];
  par_total = int64_t(ltail[2]) + ltail[3];
  FVX_ARG_CHECK(lrn_total < (int64_t(1) << 31) && par_total < (int64_t(1) << 31),
                "local-expansion pair list too long");
  if (learned) {
    if ((rc = grow(T->lrn_leaf, 4 * size_t(lrn_total + 1))) ||
        (rc = grow(T->lrn_cell, 4 * size_t(lrn_total + 1))))
      return rc;
    LL.leaf = P<int>(T->lrn_leaf);
    LL.cell = P<int>(T->lrn_cell);
    LL.cap = static_cast<int>(lrn_total);
  }
  if (dual) {
    if ((rc = grow(T->par_par, 4 * size_t(par_total + 1))) ||
        (rc = grow(T->par_cell, 4 * size_t(par_total + 1))))
      return rc;
  }
  T->n_learned = static_cast<int>(lrn_total);
  T->n_parent_pairs = static_cast<int>(par_total);
  if (dual) {
    D.near_idx = P<int>(T->near_list);
    D.lrn_leaf = LL.leaf;
    D.lrn_cell = LL.cell;
    D.par_par = P<int>(T->par_par);
    D.par_cell = P<int>(T->par_cell);
    D.near_cap = static_cast<int>(near_total);
    D.lrn_cap = static_cast<int>(lrn_total);
    D.par_cap = static_cast<int>(par_total);
    traverse_dual_kernel<true><<<(nleaf + 127) / 128, 128, 0, s>>>(V, D, ovf);
  } else {
    traverse_kernel<true><<<(nleaf + 127) / 128, 128, 0, s>>>(
        V, near_off, far_off, nullptr, nullptr, P<int>(T->near_list), P<int>(T->far_list),
        static_cast<int>(near_total), static_cast<int>(far_total), ovf, LL);
  }
  FVX_LAUNCH_CHECK();

  }
  ST.pos = pos;
  ST.n = n;
  ST.leaf_target = leaf_target;
  ST.far_method = T->far_method;
  ST.theta = theta;
  ST.theta_l = T->theta_l;
  ST.L = L;
  ST.total_cells = total_cells;
  ST.nleaf = nleaf;
  ST.h = h;
  for (int c = 0; c < 3; ++c) ST.origin[c] = origin[c];
  for (int l = 0; l < 11; ++l) {
    ST.cap[l] = cap[l];
    ST.ncells[l] = ncells[l];
  }
  for (int l = 0; l < 12; ++l) ST.base[l] = base[l];
  ST.perm = perm;
  ST.near_total = near_total;
  ST.far_total = far_total;
  ST.lrn_total = lrn_total;
  ST.par_total = par_total;
  // the evaluation order: leaves by decreasing near-field work
  if ((rc = grow(T->leaf_order, 4 * 4 * size_t(nleaf))) ||
      (rc = grow(T->order_table, 4 * size_t(sort_table_ints(nleaf)))))
    return rc;
  {
    uint32_t* ok0 = P<uint32_t>(T->leaf_order) + 2 * size_t(nleaf);
    int* oi0 = P<int>(T->leaf_order);
    order_keys_kernel<<<(nleaf + 255) / 256, 256, 0, s>>>(
        nleaf, near_cnt, lvb + total_cells + base[L], ok0, oi0);
    FVX_LAUNCH_CHECK();
    if ((rc = sort_pairs_u32(ok0, oi0, ok0 + nleaf, oi0 + nleaf, nleaf, P<int>(T->order_table),
                             P<int>(T->scan_tmp), s, 2)))
      return rc;
  }
  ST.valid = true;
  }
  // 7. evaluation
  EvalArgs A;
  A.h = static_cast<float>(h);
  A.leaf_start = leaves.start;
  A.leaf_count = leaves.count;
  A.leaf_key = leaves.key;
  A.near_off = near_off;
  A.near_cnt = near_cnt;
  A.near_idx = P<int>(T->near_list);
  A.far_off = far_off;
  A.far_cnt = far_cnt;
  A.far_idx = P<int>(T->far_list);
  A.rec = rec;
  A.sp = sp;
  A.sa = sa;
  A.sg = sg;
  A.perm = perm;
  A.out_a = out_a;
  A.out_b = out_b;
  A.leaf_local = nullptr;
  A.parent_local = nullptr;
  A.leaf_parent = leaf_parent;
  const uint32_t* par_key = dual ? V.key + base[L - 1] : nullptr;
  // ---- the FP64 judge of the local-expansion path --------------------------------
  // A judged sweep (val_samples > 0) classifies every pair, samples each class,
  // sums the samples' exact expansions in FP64, runs the sweep's own
  // translation and network kernels on them and decides per class whether the
  // network stays, is dropped, or the whole class is summed directly in FP64;
  // the decision is kept (per mode) for the sweeps in between, which only
  // classify their pairs.
  const int64_t nloc = learned ? lrn_total + par_total : 0;
  const bool network = T->far_method == FVX_FAR_LEARNED;
  const bool judged = nloc > 0 && T->val_samples > 0;
  const bool use_judge = nloc > 0 && (judged || T->judge_armed);
  const int mslot = mode & 7;
  FarJudge FJ{};
  tree::JudgeLists JL{};
  tree::JudgeSampleBufs JB{};
  tree::JudgeWords* JW = nullptr;
  int jcap = 0;
  uint8_t* act = nullptr;
  if (use_judge) {
    const bool fresh_table = T->judge_act.p == nullptr;
    if ((rc = grow(T->judge_act, 8 * kJudgeClasses)) || (rc = grow(T->fb_count, 16))) return rc;
    if (fresh_table || !T->judge_armed)
      FVX_CUDA_TRY(cudaMemsetAsync(T->judge_act.p, 0, 8 * kJudgeClasses, s));
    act = P<uint8_t>(T->judge_act) + mslot * kJudgeClasses;
    FVX_CUDA_TRY(cudaMemsetAsync(T->fb_count.p, 0, 16, s));
  }
  if (judged) {
    // every pair's class and the class sizes (the sweep's kernels work the
    // class out again themselves; the judge needs the sizes and the sample)
    if ((rc = grow(T->judge_cls, size_t(nloc))) || (rc = grow(T->judge_hist, 4 * kJudgeClasses)))
      return rc;
    FVX_CUDA_TRY(cudaMemsetAsync(T->judge_hist.p, 0, 4 * kJudgeClasses, s));
    JL.tgt[0] = P<int>(T->lrn_leaf);
    JL.cell[0] = P<int>(T->lrn_cell);
    JL.key[0] = leaves.key;
    JL.h[0] = static_cast<float>(h);
    JL.tgt[1] = dual ? P<int>(T->par_par) : JL.tgt[0];
    JL.cell[1] = dual ? P<int>(T->par_cell) : JL.cell[0];
    JL.key[1] = dual ? par_key : JL.key[0];
    JL.h[1] = static_cast<float>(2.0 * h);
    JL.n0 = static_cast<int>(lrn_total);
    JL.n = static_cast<int>(nloc);
    const int cgrid = static_cast<int>(std::min<int64_t>((nloc + 255) / 256, 8 * device_sm_count()));
    tree::judge_classify_kernel<<<cgrid, 256, 0, s>>>(
        JL, rec, static_cast<float>(1.0 / (T->theta_l * T->theta_l)), P<uint8_t>(T->judge_cls),
        P<unsigned>(T->judge_hist));
    FVX_LAUNCH_CHECK();
  }
  if (judged) {
    const int per_class = std::max(1, T->val_samples / kJudgeClasses);
    jcap = 16 * per_class;  // per list: 8 classes, at most 2 per_class samples each
    if ((rc = grow(T->judge_words, sizeof(tree::JudgeWords))) ||
        (rc = grow(T->judge_samp, (9 * sizeof(int) + 2) * size_t(jcap) + 256)) ||
        (rc = grow(T->judge_A, sizeof(float) * 64 * size_t(jcap))) ||
        (rc = grow(T->judge_Y, sizeof(float) * 64 * size_t(jcap))) ||
        (rc = grow(T->judge_err, sizeof(float) * 4 * size_t(jcap))) ||
        (rc = grow(T->pair_partial, sizeof(double) * 30 * 2 * size_t(jcap) + 8 * size_t(jcap) + 64)))
      return rc;
    JW = P<tree::JudgeWords>(T->judge_words);
    FVX_CUDA_TRY(cudaMemsetAsync(JW, 0, sizeof(tree::JudgeWords), s));
    FVX_CUDA_TRY(cudaMemsetAsync(T->judge_A.p, 0, sizeof(float) * 64 * size_t(jcap), s));
    FVX_CUDA_TRY(cudaMemsetAsync(T->judge_Y.p, 0, sizeof(float) * 64 * size_t(jcap), s));
    int* ib = P<int>(T->judge_samp);
    for (int l = 0; l < 2; ++l) {
      JB.row[l] = ib + (4 * l + 0) * jcap;
      JB.tgt[l] = ib + (4 * l + 1) * jcap;
      JB.cell[l] = ib + (4 * l + 2) * jcap;
      JB.key[l] = reinterpret_cast<uint32_t*>(ib + (4 * l + 3) * jcap);
      JB.cls[l] = reinterpret_cast<uint8_t*>(ib + 9 * jcap) + l * jcap;
    }
    int* iota = ib + 8 * jcap;
    JB.cap = jcap;
    const uint32_t seed = tree::judge_hash(0x9e3779b9u * (++T->judge_seq));
    const int cgrid = static_cast<int>(std::min<int64_t>((nloc + 255) / 256, 8 * device_sm_count()));
    tree::judge_select_kernel<<<cgrid, 256, 0, s>>>(JL, P<uint8_t>(T->judge_cls),
                                                    P<unsigned>(T->judge_hist), per_class, seed,
                                                    JW, JB);
    FVX_LAUNCH_CHECK();
    tree::judge_pad_kernel<<<(jcap + 127) / 128, 128, 0, s>>>(JL, JW, JB, iota);
    FVX_LAUNCH_CHECK();
    // exact FP64 expansions of the samples
    const int* jcnt = reinterpret_cast<const int*>(reinterpret_cast<const char*>(JW) +
                                                   offsetof(tree::JudgeWords, cnt));
    JudgeSampleView SV{jcnt, jcap, {JB.cell[0], JB.cell[1]}, {JB.key[0], JB.key[1]},
                       {JL.h[0], JL.h[1]}};
    int* joff = reinterpret_cast<int*>(P<double>(T->pair_partial) + 30 * 2 * size_t(jcap));
    if ((rc = judge_sums_launch(SV, leaves.key, lvb, lvb + total_cells, sp, sa, cid,
                                static_cast<float>(h), P<double>(T->pair_partial), joff, s)))
      return rc;
    // the sweep's own translation (and network) on the samples, one target each
    float* jA = P<float>(T->judge_A);
    float* jY = P<float>(T->judge_Y);
    const int n1s = dual && par_total > 0 ? jcap : 0;
    const int n0s = lrn_total > 0 ? jcap : 0;
    FarPairs sa0{iota, JB.cell[0], JB.key[0], JL.h[0], jA, n0s};
    FarPairs sa1{iota, JB.cell[1], JB.key[1], JL.h[1], jA + 32 * jcap, n1s};
    if ((rc = m2l_farfield_launch(sa0, sa1, rec, s))) return rc;
    if (network) {
      FarPairs sy0{iota, JB.cell[0], JB.key[0], JL.h[0], jY, n0s};
      FarPairs sy1{iota, JB.cell[1], JB.key[1], JL.h[1], jY + 32 * jcap, n1s};
      if ((rc = mlp_farfield_launch(sy0, sy1, rec, T->mlp_W, T->mlp_b, s))) return rc;
    }
    tree::judge_errors_kernel<<<(2 * jcap + 127) / 128, 128, 0, s>>>(
        JB, rec, P<double>(T->pair_partial), jA, network ? jY : nullptr, JL.h[0],
        JL.h[1], static_cast<float>(T->val_tol), JW, P<float>(T->judge_err));
    FVX_LAUNCH_CHECK();
    tree::judge_decide_kernel<<<1, 32, 0, s>>>(JW, P<unsigned>(T->judge_hist), act,
                                               network ? 1 : 0);
    FVX_LAUNCH_CHECK();
    T->judge_armed = true;
  }
  if (use_judge) {
    const int64_t cap = nloc + 2 * int64_t(jcap);
    if ((rc = grow(T->fb_queue, sizeof(int2) * size_t(cap)))) return rc;
    FJ.act = act;
    FJ.inv_theta2 = static_cast<float>(1.0 / (T->theta_l * T->theta_l));
    FJ.fb = P<int2>(T->fb_queue);
    FJ.nfb = P<int>(T->fb_count);
    FJ.fb_cap = static_cast<int>(cap);
  }
  if (learned && nloc > 0) {
    if (!T->ev2) {
      FVX_CUDA_TRY(cudaEventCreate(&T->ev2));
      FVX_CUDA_TRY(cudaEventCreate(&T->ev3));
    }
    FVX_CUDA_TRY(cudaEventRecord(T->ev2, s));
    // zeroed expansions of the leaves (and parents), then the analytic
    // translation and (learned) the network's residual of both lists, each in
    // one launch, under the judge's class actions
    auto zeroed = [&](DevBuf& buf, int ntgt) -> int {
      int r = grow(buf, sizeof(float) * 32 * size_t(ntgt));
      if (r) return r;
      FVX_CUDA_TRY(cudaMemsetAsync(buf.p, 0, sizeof(float) * 32 * size_t(ntgt), s));
      return FVX_OK;
    };
    if ((rc = zeroed(T->leaf_local, nleaf))) return rc;
    FarPairs la{P<int>(T->lrn_leaf), P<int>(T->lrn_cell), leaves.key, static_cast<float>(h),
                P<float>(T->leaf_local), static_cast<int>(lrn_total)};
    FarPairs lb{};
    if (dual) {
      if ((rc = zeroed(T->parent_local, npar))) return rc;
      lb = FarPairs{P<int>(T->par_par), P<int>(T->par_cell), par_key, static_cast<float>(2.0 * h),
                    P<float>(T->parent_local), static_cast<int>(par_total)};
    }
    if ((rc = m2l_farfield_launch(la, lb, rec, s, FJ))) return rc;
    if (network && (rc = mlp_farfield_launch(la, lb, rec, T->mlp_W, T->mlp_b, s, FJ))) return rc;
    A.leaf_local = P<float>(T->leaf_local);
    if (dual) A.parent_local = P<float>(T->parent_local);
    FVX_CUDA_TRY(cudaEventRecord(T->ev3, s));
  }
  if (judged) {
    // sampled pairs that miss the tolerance: out of their expansions, queued
    tree::judge_repair_kernel<<<(2 * jcap + 127) / 128, 128, 0, s>>>(
        JB, P<float>(T->judge_A), network ? P<float>(T->judge_Y) : nullptr,
        P<float>(T->judge_err), static_cast<float>(T->val_tol), act, P<float>(T->leaf_local),
        dual ? P<float>(T->parent_local) : nullptr, JW, FJ);
    FVX_LAUNCH_CHECK();
    T->last_judged = 2 * jcap;
  }
  T->last_L = L;
  T->last_nleaf = nleaf;
  T->last_h = h;
  T->last_leaf_key = leaves.key;
  T->last_par_key = par_key;
  T->last_cell_start = lvb;
  T->last_cell_count = lvb + total_cells;
  T->last_cid = cid;
  if (!T->ev0) {
    FVX_CUDA_TRY(cudaEventCreate(&T->ev0));
    FVX_CUDA_TRY(cudaEventCreate(&T->ev1));
  }
  // the resident evaluation warps' leaf counter
  if ((rc = grow(T->eval_next, 16))) return rc;
  FVX_CUDA_TRY(cudaMemsetAsync(T->eval_next.p, 0, sizeof(int), s));
  A.nleaf = nleaf;
  A.leaf_next = P<int>(T->eval_next);
  A.leaf_order = P<int>(T->leaf_order);
  FVX_CUDA_TRY(cudaEventRecord(T->ev0, s));
  // the factored stretching loop where leaves are at most 4 smallest cores
  // wide (the cores of the last full build; see near_tile_x2_factored)
  const bool factored = h <= 4.0 * T->sigma_min;
  if (kernel == FVX_KERNEL_WINCKELMANS)
    launch_eval<FVX_KERNEL_WINCKELMANS>(mode, nleaf, n, A, factored, s);
  else
    launch_eval<FVX_KERNEL_GAUSSIANERF>(mode, nleaf, n, A, factored, s);
  FVX_LAUNCH_CHECK();
  FVX_CUDA_TRY(cudaEventRecord(T->ev1, s));
  // FP64 direct sums of the queued pairs (whole classes and sampled repairs)
  // at every particle of their leaf or parent
  if (use_judge) {
    tree::FallbackTargets tgs{{A.leaf_start, dual ? V.start + base[L - 1] : A.leaf_start},
                              {A.leaf_count, dual ? V.count + base[L - 1] : A.leaf_count}};
    const int fgrid = 4 * device_sm_count();
    if (kernel == FVX_KERNEL_WINCKELMANS)
      launch_fallback<FVX_KERNEL_WINCKELMANS>(mode, fgrid, FJ.fb, FJ.nfb, FJ.fb_cap, tgs, lvb,
                                              lvb + total_cells, perm, pos, alpha, sigma,
                                              tgt_gamma, out_a, out_b, s);
    else
      launch_fallback<FVX_KERNEL_GAUSSIANERF>(mode, fgrid, FJ.fb, FJ.nfb, FJ.fb_cap, tgs, lvb,
                                              lvb + total_cells, perm, pos, alpha, sigma,
                                              tgt_gamma, out_a, out_b, s);
    FVX_LAUNCH_CHECK();
  }
  unsigned ovf_h[6] = {0, 0, 0, 0, 0, 0};
  FVX_CUDA_TRY(cudaMemcpyAsync(ovf_h, ovf, 24, cudaMemcpyDeviceToHost, s));
  T->stats[0] = L;
  T->stats[1] = nleaf;
  T->stats[2] = near_total;
  T->stats[3] = far_total;
  T->stats[4] = lrn_total + par_total;
  if (stats) {
    FVX_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned long long work[2];
    memcpy(work, ovf_h + 2, sizeof(work));
    T->stats[5] = ovf_h[0];
    T->stats[6] = static_cast<int64_t>(work[0]);
    T->stats[7] = static_cast<int64_t>(work[1]);
    for (int k = 0; k < 8; ++k) stats[k] = T->stats[k];
    FVX_ARG_CHECK(ovf_h[0] == 0, "treecode traversal overflow (code %u)", ovf_h[0]);
  }
  return FVX_OK;
}

}  // namespace fvx

extern "C" {

int fvx_tree_set_list_slots(fvx_tree* T, int near, int lrn, int par) {
  FVX_ARG_CHECK(T != nullptr && near >= 0 && lrn >= 0 && par >= 0, "bad slot capacities");
  T->slot_near = near;
  T->slot_lrn = lrn;
  T->slot_par = par;
  T->st.valid = false;
  return FVX_OK;
}

int fvx_tree_hint_same_positions(fvx_tree* T) {
  FVX_ARG_CHECK(T != nullptr, "null tree handle");
  T->reuse_next = true;
  return FVX_OK;
}

int fvx_tree_create(fvx_tree** out) {
  FVX_ARG_CHECK(out != nullptr, "null handle pointer");
  *out = new fvx_tree();
  cudaGetDevice(&(*out)->device);
  return FVX_OK;
}

void fvx_tree_destroy(fvx_tree* T) {
  if (!T) return;
  if (T->ev0) cudaEventDestroy(T->ev0);
  if (T->ev1) cudaEventDestroy(T->ev1);
  if (T->ev2) cudaEventDestroy(T->ev2);
  if (T->ev3) cudaEventDestroy(T->ev3);
  fvx::DevBuf* bufs[] = {&T->keys0,   &T->keys1,     &T->idx0,     &T->idx1,     &T->table,
                         &T->scan_tmp, &T->flags,   &T->cid,      &T->levels,   &T->counts,
                         &T->rec,     &T->sp,       &T->sa,       &T->sg,       &T->lists_meta,
                         &T->near_list, &T->far_list, &T->bbox,   &T->lrn_meta, &T->lrn_leaf,
                         &T->lrn_cell, &T->leaf_local, &T->judge_act, &T->judge_cls,
                         &T->judge_hist, &T->judge_words, &T->judge_samp, &T->judge_A,
                         &T->judge_Y, &T->judge_err, &T->fb_queue, &T->fb_count,
                         &T->dual_meta, &T->par_par, &T->par_cell, &T->parent_local,
                         &T->cen, &T->res_slot, &T->res_cnt, &T->eval_next,
                         &T->leaf_order, &T->order_table,
                         &T->lrn_slot, &T->par_slot,
                         &T->pair_partial};
  for (auto* b : bufs)
    if (b->p) cudaFree(b->p);
  delete T;
}

int fvx_tree_sweep(fvx_tree* T, int mode, int kernel, const double* pos, const double* alpha,
                   const double* sigma, const double* tgt_gamma, int64_t n, double theta,
                   int leaf_target, double* out_a, double* out_b, int64_t* stats, void* stream) {
  return fvx::tree_sweep(T, mode, kernel, pos, alpha, sigma, tgt_gamma, n, theta, leaf_target,
                         out_a, out_b, stats, static_cast<cudaStream_t>(stream));
}

int fvx_tree_set_far_field(fvx_tree* T, int method, const void* W, const float* b,
                           double theta_local) {
  FVX_ARG_CHECK(T != nullptr, "null tree handle");
  FVX_ARG_CHECK(method == FVX_FAR_M2P || method == FVX_FAR_M2L || method == FVX_FAR_LEARNED,
                "unknown far-field method %d", method);
  FVX_ARG_CHECK(method == FVX_FAR_M2P || (theta_local > 0.0 && theta_local < 1.0),
                "bad theta_local");
  FVX_ARG_CHECK(method != FVX_FAR_LEARNED || (W != nullptr && b != nullptr),
                "the learned far field needs weights and biases");
  T->far_method = method;
  T->mlp_W = method == FVX_FAR_LEARNED ? W : nullptr;
  T->mlp_b = method == FVX_FAR_LEARNED ? b : nullptr;
  T->theta_l = method == FVX_FAR_M2P ? 0.0 : theta_local;
  T->judge_armed = false;  // a new far field starts with every class expanded
  T->last_judged = 0;
  return FVX_OK;
}

int fvx_tree_set_validation(fvx_tree* T, int samples, double tol) {
  FVX_ARG_CHECK(T != nullptr, "null tree handle");
  FVX_ARG_CHECK(samples >= 0 && samples <= (1 << 16), "samples out of range");
  FVX_ARG_CHECK(tol > 0.0, "tolerance must be positive");
  T->val_samples = samples;
  T->val_tol = tol;
  return FVX_OK;
}

int fvx_tree_last_validation(fvx_tree* T, double* out) {
  FVX_ARG_CHECK(T && out, "null argument");
  double rec[8 + 5 * fvx::kJudgeClasses];
  int rc = fvx_tree_last_judge(T, rec, 8 + 5 * fvx::kJudgeClasses);
  if (rc) return rc;
  out[0] = rec[0];
  out[1] = rec[2];
  out[2] = rec[3];
  out[3] = rec[4];
  return FVX_OK;
}

int fvx_tree_last_judge(fvx_tree* T, double* out, int n_out) {
  FVX_ARG_CHECK(T && out && n_out >= 0, "null argument");
  const int n_rec = 8 + 5 * fvx::kJudgeClasses;
  for (int k = 0; k < n_out; ++k) out[k] = 0.0;
  if (T->last_judged <= 0) return FVX_OK;
  fvx::tree::JudgeWords W;
  int nfb = 0;
  FVX_CUDA_TRY(cudaMemcpy(&W, T->judge_words.p, sizeof(W), cudaMemcpyDeviceToHost));
  FVX_CUDA_TRY(cudaMemcpy(&nfb, T->fb_count.p, sizeof(int), cudaMemcpyDeviceToHost));
  double rec[8 + 5 * fvx::kJudgeClasses];
  float esum;
  memcpy(&esum, &W.err_sum_bits, sizeof(float));
  float emax;
  memcpy(&emax, &W.err_max_bits, sizeof(float));
  double pairs = 0.0;
  for (int k = 0; k < fvx::kJudgeClasses; ++k) pairs += W.class_pairs[k];
  rec[0] = W.checked;
  rec[1] = W.repaired;
  rec[2] = nfb;
  rec[3] = W.applied ? esum / W.applied : 0.0;
  rec[4] = emax;
  rec[5] = W.unrepaired;
  rec[6] = pairs;
  rec[7] = 0.0;
  for (int k = 0; k < fvx::kJudgeClasses; ++k) {
    rec[8 + 5 * k + 0] = W.class_pairs[k];
    rec[8 + 5 * k + 1] = W.class_samples[k];
    rec[8 + 5 * k + 2] = W.fail_learned[k];
    rec[8 + 5 * k + 3] = W.fail_analytic[k];
    rec[8 + 5 * k + 4] = W.action[k];
  }
  for (int k = 0; k < n_out && k < n_rec; ++k) out[k] = rec[k];
  return FVX_OK;
}

int fvx_tree_last_local_ms(fvx_tree* T, float* ms) {
  FVX_ARG_CHECK(T && ms, "null argument");
  *ms = 0.f;
  if (!T->ev2 || T->n_learned <= 0) return FVX_OK;
  FVX_CUDA_TRY(cudaEventSynchronize(T->ev3));
  FVX_CUDA_TRY(cudaEventElapsedTime(ms, T->ev2, T->ev3));
  return FVX_OK;
}

int fvx_tree_sample_pairs(fvx_tree* T, int list, int max_pairs, void* X, float* Tgt, float* A,
                          int* n_out, void* stream) {
  FVX_ARG_CHECK(T && X && Tgt && n_out && max_pairs > 0, "bad arguments");
  FVX_ARG_CHECK(list == 0 || list == 1, "list is 0 (leaf pairs) or 1 (parent pairs)");
  *n_out = 0;
  FVX_ARG_CHECK(T->theta_l > 0.0, "sampling needs the local-expansion path on the last sweep");
  const int n = list == 0 ? T->n_learned : T->n_parent_pairs;
  if (n <= 0) return FVX_OK;
  const int stride = n > max_pairs ? n / max_pairs : 1;
  const int np = n / stride < max_pairs ? n / stride : max_pairs;
  const int slices = np < 4096 ? 8 : (np < 32768 ? 4 : 2);
  int rc = fvx::grow(T->pair_partial, sizeof(double) * 30 * size_t(np) * slices);
  if (rc) return rc;
  const int* tgt = list == 0 ? fvx::P<int>(T->lrn_leaf) : fvx::P<int>(T->par_par);
  const int* cell = list == 0 ? fvx::P<int>(T->lrn_cell) : fvx::P<int>(T->par_cell);
  const uint32_t* tkey = list == 0 ? T->last_leaf_key : T->last_par_key;
  const float th = static_cast<float>(list == 0 ? T->last_h : 2.0 * T->last_h);
  rc = fvx::mlp_pair_targets_launch(
      np, stride, tgt, cell, tkey, th, T->last_leaf_key, fvx::P<float>(T->rec),
      T->last_cell_start, T->last_cell_count, fvx::P<float4>(T->sp), fvx::P<float4>(T->sa),
      T->last_cid, static_cast<float>(T->last_h), X, Tgt, A, nullptr,
      fvx::P<double>(T->pair_partial), slices, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  *n_out = np;
  return FVX_OK;
}

int fvx_tree_last_eval_ms(fvx_tree* T, float* ms) {
  FVX_ARG_CHECK(T && ms, "null argument");
  *ms = 0.f;
  if (!T->ev0) return FVX_OK;
  FVX_CUDA_TRY(cudaEventSynchronize(T->ev1));
  FVX_CUDA_TRY(cudaEventElapsedTime(ms, T->ev0, T->ev1));
  return FVX_OK;
}

}  // extern "C"
