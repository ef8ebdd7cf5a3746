// fvx_particles.cu -- all-pairs vortex-particle sweeps (velocity, stretching,
// velocity gradient, vorticity) with the Winckelmans or Gaussian-erf core.
//
// Replaces src/fluxvortex/kernel.py:69-190 (NumPy, 512 x 512 chunks) and its
// unused Warp ports src/fluxvortex/warp_vpm.py:20-141 (one thread per pair,
// one atomic per pair and component).
//
// Closed forms used (C = -1/(4 pi) folded into alpha on staging; d = x_t - x_s;
// f(r) = g(r/sigma)/r^3 and fpr = f'(r)/r, both finite at r = 0):
//   u      += f (d x a)                                      kernel.py:103-114
//   J_ij   += fpr (d x a)_i d_j + f eps_ijl a_l              kernel.py:156-188
//   S       = J . G_t = f (G_t x a) + fpr (d . G_t)(d x a)   particles.py:148-151
//   omega_i = eps_ijk J_kj = fpr (d (d . a) - a r^2) - 2 f a particles.py:219-225
// Winckelmans: f = (r^2 + 2.5 s^2) q^-5/2, fpr = -(3 r^2 + 10.5 s^2) q^-7/2,
//   q = r^2 + s^2 (kernel.py:42-55 rewritten without r_bar = r/sigma).
// Gaussian-erf: for r/sigma >= 0.5 the kernel.py:16-31 formula; below it the
//   Taylor series of g(r)/r^3 (the reference's erf - c r exp form cancels
//   there and is pure rounding noise at its r = 1e-12 self-pair clamp).
//
// Layout and tiling: a CTA owns 128 (FP64) or 256-512 (FP32, two or four per
// thread) targets held in registers.  Source tiles of 128 particles (AoS pos, alpha,
// sigma exactly as the caller stores them) are staged by 1-D TMA bulk copies
// (cp.async.bulk) into a double-buffered raw area, then converted by all
// threads into a compute tile (alpha pre-scaled by C, sigma^2 and the core's
// second constant precomputed; FP32 positions re-centred on the CTA's first
// target in FP64 before rounding).  Every thread then sweeps the tile reading
// shared memory by broadcast.  FP32 sums are kept per tile and folded into a
// two-sum (hi, lo) pair per component.  When targets alone cannot fill the
// SMs the source range is split over gridDim.y; partial sums go to scratch
// and a second kernel adds them in fixed order.
#include <type_traits>

#include "fvx_common.cuh"
#include "fvx_pair_math.cuh"

namespace fvx {
namespace {

using namespace pair;

constexpr int kThreads = 128;
constexpr int kSrcTile = 128;
constexpr double kC = -0.07957747154594767;  // -1/(4 pi)

struct RawSrc {
  double pos[kSrcTile * 3];
  double alpha[kSrcTile * 3];
  double sigma[kSrcTile];
};

// Compute tile: two 4-vectors per source so that a thread fetches a source
// with two 128-bit shared loads (FP32) and reuses it for all its targets.
template <typename T>
struct alignas(4 * sizeof(T)) Vec4 {
  T x, y, z, w;
};
template <typename T>
struct SrcTile {
  Vec4<T> p[kSrcTile];  // x, y, z, sigma^2
  Vec4<T> a[kSrcTile];  // C*alpha_x, C*alpha_y, C*alpha_z, k2
};

// Targets per thread: more register blocking for the 3-component modes.
template <int MODE, bool F32>
struct Blocking {
  static constexpr int tpt = !F32 ? 1 : (ModeInfo<MODE>::ncomp <= 3 ? 4 : 2);
};

struct PairArgs {
  const double* tgt;
  const double* tgt_gamma;
  int64_t n_tgt;
  const double* pos;
  const double* alpha;
  const double* sigma;
  int64_t n_src;
  int64_t chunk;  // sources per split (even)
  double* out_a;
  double* out_b;
  double* partial;  // (S, M, ncomp) when gridDim.y > 1
  int use_tma;
};

__device__ void issue_src(const PairArgs& A, RawSrc& raw, int64_t j0, int cnt, uint64_t* bar) {
  BulkPlan pp = plan_bulk(A.pos, j0, cnt, 24, A.use_tma);
  BulkPlan pa = plan_bulk(A.alpha, j0, cnt, 24, A.use_tma);
  BulkPlan ps = plan_bulk(A.sigma, j0, cnt, 8, A.use_tma);
  mbar_arrive_expect_tx(bar, pp.bulk_bytes + pa.bulk_bytes + ps.bulk_bytes);
  if (pp.bulk_bytes) bulk_g2s(raw.pos, A.pos + 3 * j0, pp.bulk_bytes, bar);
  if (pa.bulk_bytes) bulk_g2s(raw.alpha, A.alpha + 3 * j0, pa.bulk_bytes, bar);
  if (ps.bulk_bytes) bulk_g2s(raw.sigma, A.sigma + j0, ps.bulk_bytes, bar);
}

__device__ void tail_src(const PairArgs& A, RawSrc& raw, int64_t j0, int cnt) {
  BulkPlan p = plan_bulk(A.pos, j0, cnt, 24, A.use_tma);
  if (p.tail_bytes) plain_copy8(raw.pos, A.pos + 3 * j0, p.bulk_bytes, p.tail_bytes);
  p = plan_bulk(A.alpha, j0, cnt, 24, A.use_tma);
  if (p.tail_bytes) plain_copy8(raw.alpha, A.alpha + 3 * j0, p.bulk_bytes, p.tail_bytes);
  p = plan_bulk(A.sigma, j0, cnt, 8, A.use_tma);
  if (p.tail_bytes) plain_copy8(raw.sigma, A.sigma + j0, p.bulk_bytes, p.tail_bytes);
}

template <typename T>
__device__ __forceinline__ void two_sum_fold(T& hi, T& lo, T p) {
  T s = hi + p;
  T bp = s - hi;
  T err = (hi - (s - bp)) + (p - bp);
  hi = s;
  lo += err;
}

template <int MODE, int KERNEL, bool F32>
__global__ void __launch_bounds__(kThreads) pairs_kernel(PairArgs A) {
  using T = typename std::conditional<F32, float, double>::type;
  constexpr int TPT = Blocking<MODE, F32>::tpt;  // targets per thread
  constexpr int NC = ModeInfo<MODE>::ncomp;
  constexpr bool NEED_FPR = ModeInfo<MODE>::need_fpr;
  constexpr bool NEED_TG = ModeInfo<MODE>::need_tg;

  __shared__ __align__(128) RawSrc raw[2];
  __shared__ __align__(16) SrcTile<T> tile;
  __shared__ __align__(8) uint64_t bar[2];

  const int64_t base = static_cast<int64_t>(blockIdx.x) * (kThreads * TPT);
  // Re-centring origin: the CTA's first target (FP32 only).
  double ox = 0.0, oy = 0.0, oz = 0.0;
  if (F32) {
    ox = A.tgt[3 * base + 0];
    oy = A.tgt[3 * base + 1];
    oz = A.tgt[3 * base + 2];
  }
  T tx[TPT], ty[TPT], tz[TPT], gx[TPT], gy[TPT], gz[TPT];
  bool act[TPT];
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    const int64_t i = base + threadIdx.x + j * kThreads;
    act[j] = i < A.n_tgt;
    double px = 0, py = 0, pz = 0, qx = 0, qy = 0, qz = 0;
    if (act[j]) {
      px = A.tgt[3 * i + 0] - ox;
      py = A.tgt[3 * i + 1] - oy;
      pz = A.tgt[3 * i + 2] - oz;
      if (NEED_TG) {
        qx = A.tgt_gamma[3 * i + 0];
        qy = A.tgt_gamma[3 * i + 1];
        qz = A.tgt_gamma[3 * i + 2];
      }
    }
    tx[j] = static_cast<T>(px);
    ty[j] = static_cast<T>(py);
    tz[j] = static_cast<T>(pz);
    gx[j] = static_cast<T>(qx);
    gy[j] = static_cast<T>(qy);
    gz[j] = static_cast<T>(qz);
  }

  const int64_t jb = static_cast<int64_t>(blockIdx.y) * A.chunk;
  const int64_t je = min(jb + A.chunk, A.n_src);
  const int ntiles = jb < je ? static_cast<int>((je - jb + kSrcTile - 1) / kSrcTile) : 0;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  T hi[TPT][NC], lo[TPT][NC];
#pragma unroll
  for (int j = 0; j < TPT; ++j)
#pragma unroll
    for (int c = 0; c < NC; ++c) hi[j][c] = lo[j][c] = T(0);

  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  if (ntiles > 0 && threadIdx.x == 0)
    issue_src(A, raw[0], jb, static_cast<int>(min64(kSrcTile, je - jb)), &bar[0]);
  int t = 0;
  for (; t < ntiles; ++t) {
    const int buf = t & 1;
    const int64_t j0 = jb + static_cast<int64_t>(t) * kSrcTile;
    const int n = static_cast<int>(min64(kSrcTile, je - j0));
    if (t + 1 < ntiles && threadIdx.x == 0) {
      const int64_t j1 = j0 + kSrcTile;
      issue_src(A, raw[buf ^ 1], j1, static_cast<int>(min64(kSrcTile, je - j1)),
                &bar[buf ^ 1]);
    }
    const bool got = mbar_wait(&bar[buf], phase[buf]);
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
    phase[buf] ^= 1u;
    tail_src(A, raw[buf], j0, n);
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += kThreads) {
      const double sg = raw[buf].sigma[k];
      Vec4<T> pv, av;
      pv.x = static_cast<T>(raw[buf].pos[3 * k + 0] - ox);
      pv.y = static_cast<T>(raw[buf].pos[3 * k + 1] - oy);
      pv.z = static_cast<T>(raw[buf].pos[3 * k + 2] - oz);
      pv.w = static_cast<T>(sg * sg);
      av.x = static_cast<T>(kC * raw[buf].alpha[3 * k + 0]);
      av.y = static_cast<T>(kC * raw[buf].alpha[3 * k + 1]);
      av.z = static_cast<T>(kC * raw[buf].alpha[3 * k + 2]);
      av.w = static_cast<T>(KERNEL == FVX_KERNEL_WINCKELMANS ? 2.5 * sg * sg : 1.0 / sg);
      tile.p[k] = pv;
      tile.a[k] = av;
    }
    __syncthreads();
    T part[TPT][NC];
#pragma unroll
    for (int j = 0; j < TPT; ++j)
#pragma unroll
      for (int c = 0; c < NC; ++c) part[j][c] = T(0);
#pragma unroll 2
    for (int k = 0; k < n; ++k) {
      const Vec4<T> pv = tile.p[k];
      const Vec4<T> av = tile.a[k];
      const T sx = pv.x, sy = pv.y, sz = pv.z, s2 = pv.w;
      const T ax = av.x, ay = av.y, az = av.z, k2 = av.w;
#pragma unroll
      for (int j = 0; j < TPT; ++j) {
        const T dx = tx[j] - sx, dy = ty[j] - sy, dz = tz[j] - sz;
        const T r2 = dx * dx + dy * dy + dz * dz;
        T f, fpr = T(0);
        if constexpr (F32)
          core_f32<KERNEL, NEED_FPR>(r2, s2, k2, f, fpr);
        else
          core_f64<KERNEL, NEED_FPR>(r2, s2, k2, f, fpr);
        accumulate<MODE, T>(part[j], dx, dy, dz, r2, ax, ay, az, f, fpr, gx[j], gy[j], gz[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < TPT; ++j)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if constexpr (F32)
          two_sum_fold(hi[j][c], lo[j][c], part[j][c]);
        else
          hi[j][c] += part[j][c];
      }
    __syncthreads();
  }
  if (!ok) {
    flag_status(kStatusTimeout);
    if (threadIdx.x == 0 && t + 1 < ntiles) mbar_wait(&bar[(t + 1) & 1], phase[(t + 1) & 1]);
    return;
  }
#pragma unroll
  for (int j = 0; j < TPT; ++j) {
    if (!act[j]) continue;
    const int64_t i = base + threadIdx.x + j * kThreads;
    double v[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c)
      v[c] = static_cast<double>(hi[j][c]) + static_cast<double>(lo[j][c]);
    if (gridDim.y > 1) {
      double* o = A.partial + (static_cast<int64_t>(blockIdx.y) * A.n_tgt + i) * NC;
#pragma unroll
      for (int c = 0; c < NC; ++c) o[c] = v[c];
    } else {
      constexpr int NA = ModeInfo<MODE>::na;
#pragma unroll
      for (int c = 0; c < NA; ++c) A.out_a[i * NA + c] = v[c];
#pragma unroll
      for (int c = NA; c < NC; ++c) A.out_b[i * (NC - NA) + (c - NA)] = v[c];
    }
  }
}

// The split partial sums of every output value, in a fixed order: a warp per
// value, lane l adding splits l, l + 32, ... in turn, then a fixed shuffle
// tree over the lanes.  (A thread per value would leave a few hundred values
// to a handful of CTAs, each thread waiting on one dependent load per split.)
__global__ void reduce_pairs_kernel(const double* __restrict__ partial, int64_t n_tgt, int nc,
                                    int na, int splits, double* __restrict__ out_a,
                                    double* __restrict__ out_b) {
  const int64_t idx = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n_vals = n_tgt * nc;
  if (idx >= n_vals) return;  // the whole warp: idx is the warp's
  double s = 0.0;
  for (int k = lane; k < splits; k += 32) s += partial[static_cast<int64_t>(k) * n_vals + idx];
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if (lane != 0) return;
  const int64_t i = idx / nc;
  const int c = static_cast<int>(idx - i * nc);
  if (c < na)
    out_a[i * na + c] = s;
  else
    out_b[i * (nc - na) + (c - na)] = s;
}

int mode_ncomp(int mode) {
  switch (mode) {
    case FVX_PAIR_VELOCITY:
    case FVX_PAIR_STRETCH:
    case FVX_PAIR_VORTICITY:
      return 3;
    case FVX_PAIR_VELOCITY_STRETCH:
      return 6;
    case FVX_PAIR_JACOBIAN:
      return 9;
    default:
      return -1;
  }
}

int mode_na(int mode) { return mode == FVX_PAIR_VELOCITY_STRETCH ? 3 : mode_ncomp(mode); }

int targets_per_cta(int mode, int precision) {
  if (precision != FVX_PREC_F32C) return kThreads;
  return kThreads * (mode_ncomp(mode) <= 3 ? 4 : 2);
}

int pair_splits(int mode, int precision, int64_t n_tgt, int64_t n_src, int64_t* chunk) {
  const int per_cta = targets_per_cta(mode, precision);
  const int64_t gx = (n_tgt + per_cta - 1) / per_cta;
  // six resident CTAs per SM (80 registers x 128 threads): few targets
  // (the panel points against every particle) split the sources that far
  const int64_t want = 6LL * device_sm_count();
  int64_t s = gx >= want ? 1 : (want + gx - 1) / gx;
  // keep at least two source tiles per split
  int64_t maxs = (n_src + 2 * kSrcTile - 1) / (2 * kSrcTile);
  if (s > maxs) s = maxs;
  if (s < 1) s = 1;
  int64_t c = (n_src + s - 1) / s;
  c = (c + 1) & ~int64_t(1);
  s = (n_src + c - 1) / c;
  *chunk = c;
  return static_cast<int>(s);
}

template <int MODE, int KERNEL>
void launch_mode(int precision, dim3 grid, cudaStream_t stream, const PairArgs& A) {
  if (precision == FVX_PREC_F32C)
    pairs_kernel<MODE, KERNEL, true><<<grid, kThreads, 0, stream>>>(A);
  else
    pairs_kernel<MODE, KERNEL, false><<<grid, kThreads, 0, stream>>>(A);
}

template <int KERNEL>
void launch_kernel(int mode, int precision, dim3 grid, cudaStream_t stream, const PairArgs& A) {
  switch (mode) {
    case FVX_PAIR_VELOCITY:
      launch_mode<FVX_PAIR_VELOCITY, KERNEL>(precision, grid, stream, A);
      break;
    case FVX_PAIR_STRETCH:
      launch_mode<FVX_PAIR_STRETCH, KERNEL>(precision, grid, stream, A);
      break;
    case FVX_PAIR_VELOCITY_STRETCH:
      launch_mode<FVX_PAIR_VELOCITY_STRETCH, KERNEL>(precision, grid, stream, A);
      break;
    case FVX_PAIR_JACOBIAN:
      launch_mode<FVX_PAIR_JACOBIAN, KERNEL>(precision, grid, stream, A);
      break;
    default:
      launch_mode<FVX_PAIR_VORTICITY, KERNEL>(precision, grid, stream, A);
      break;
  }
}

}  // namespace

size_t particle_pairs_scratch(int mode, int precision, int64_t n_tgt, int64_t n_src) {
  const int nc = mode_ncomp(mode);
  if (nc < 0 || n_tgt <= 0 || n_src <= 0) return 0;
  int64_t chunk = 0;
  const int s = pair_splits(mode, precision, n_tgt, n_src, &chunk);
  return s > 1 ? sizeof(double) * static_cast<size_t>(nc) * n_tgt * s : 0;
}

int particle_pairs_launch(int mode, int kernel, int precision, const double* tgt,
                          const double* tgt_gamma, int64_t n_tgt, const double* pos,
                          const double* alpha, const double* sigma, int64_t n_src,
                          double* out_a, double* out_b, void* scratch, size_t scratch_bytes,
                          cudaStream_t stream) {
  const int nc = mode_ncomp(mode);
  FVX_ARG_CHECK(nc > 0, "unknown pair mode %d", mode);
  FVX_ARG_CHECK(kernel == FVX_KERNEL_GAUSSIANERF || kernel == FVX_KERNEL_WINCKELMANS,
                "unknown kernel %d", kernel);
  FVX_ARG_CHECK(precision == FVX_PREC_F64 || precision == FVX_PREC_F32C,
                "unknown precision %d", precision);
  FVX_ARG_CHECK(n_tgt >= 0 && n_src >= 0, "negative size");
  if (n_tgt == 0) return FVX_OK;
  const int na = mode_na(mode);
  FVX_ARG_CHECK(tgt && out_a, "null targets/output");
  FVX_ARG_CHECK(na == nc || out_b, "mode needs out_b");
  const bool need_tg = mode == FVX_PAIR_STRETCH || mode == FVX_PAIR_VELOCITY_STRETCH;
  FVX_ARG_CHECK(!need_tg || tgt_gamma, "mode needs target strengths");
  if (n_src == 0) {
    FVX_CUDA_TRY(cudaMemsetAsync(out_a, 0, sizeof(double) * na * n_tgt, stream));
    if (nc > na) FVX_CUDA_TRY(cudaMemsetAsync(out_b, 0, sizeof(double) * (nc - na) * n_tgt, stream));
    return FVX_OK;
  }
  FVX_ARG_CHECK(pos && alpha && sigma, "null source array");
  int64_t chunk = 0;
  const int splits = pair_splits(mode, precision, n_tgt, n_src, &chunk);
  const size_t need = splits > 1 ? sizeof(double) * static_cast<size_t>(nc) * n_tgt * splits : 0;
  if (need > 0 && (scratch == nullptr || scratch_bytes < need)) {
    set_last_error("particle_pairs needs %zu scratch bytes, got %zu", need, scratch_bytes);
    return FVX_ERR_SCRATCH;
  }
  PairArgs A;
  A.tgt = tgt;
  A.tgt_gamma = tgt_gamma;
  A.n_tgt = n_tgt;
  A.pos = pos;
  A.alpha = alpha;
  A.sigma = sigma;
  A.n_src = n_src;
  A.chunk = chunk;
  A.out_a = out_a;
  A.out_b = out_b;
  A.partial = static_cast<double*>(scratch);
  A.use_tma = aligned16(pos) && aligned16(alpha) && aligned16(sigma);
  const int per_cta = targets_per_cta(mode, precision);
  const int64_t gx = (n_tgt + per_cta - 1) / per_cta;
  FVX_ARG_CHECK(gx < (1LL << 31), "too many targets");
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(splits));
  if (kernel == FVX_KERNEL_WINCKELMANS)
    launch_kernel<FVX_KERNEL_WINCKELMANS>(mode, precision, grid, stream, A);
  else
    launch_kernel<FVX_KERNEL_GAUSSIANERF>(mode, precision, grid, stream, A);
  FVX_LAUNCH_CHECK();
  if (splits > 1) {
    const int64_t nv = n_tgt * nc;  // a warp per value
    FVX_ARG_CHECK((nv * 32 + 255) / 256 < (1LL << 31), "too many output values");
    reduce_pairs_kernel<<<static_cast<unsigned>((nv * 32 + 255) / 256), 256, 0, stream>>>(
        static_cast<const double*>(scratch), n_tgt, nc, na, splits, out_a, out_b);
    FVX_LAUNCH_CHECK();
  }
  return FVX_OK;
}

}  // namespace fvx

extern "C" {

size_t fvx_particle_pairs_scratch_bytes(int mode, int precision, int64_t n_targets,
                                        int64_t n_sources) {
  return fvx::particle_pairs_scratch(mode, precision, n_targets, n_sources);
}

int fvx_particle_pairs(int mode, int kernel, int precision, const double* tgt_pos,
                       const double* tgt_gamma, int64_t n_targets, const double* src_pos,
                       const double* src_gamma, const double* src_sigma, int64_t n_sources,
                       double* out_a, double* out_b, void* scratch, size_t scratch_bytes,
                       void* stream) {
  return fvx::particle_pairs_launch(mode, kernel, precision, tgt_pos, tgt_gamma, n_targets,
                                    src_pos, src_gamma, src_sigma, n_sources, out_a, out_b,
                                    scratch, scratch_bytes, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
