// fvx_segments.cu -- line-vortex Biot-Savart for ring, chordwise-ring and
// horseshoe vortices with the PteraSoftware Lamb-Oseen + Squire core, FP64.
//
// Replaces the five functions of src/fluxvortex/warp_kernels.py:251-382 (one
// launch per leg with an atomic add per (point, vortex) pair, :188-246).
// Here all legs of a vortex are fused: corner offsets and their lengths are
// shared between the two legs that meet at a corner (the reference computes
// the same values twice, so sharing changes no bit), per-leg constants
// (|r0|^2, the 1e-10 |r0| tolerance, |r0|^2 r_c^2, Gamma/4pi) are hoisted
// into shared memory once per tile, and sums are reduced without atomics:
//
//   collapsed  CTA = 128 target points x one chunk of vortices.  Vortex tiles
//              (corners + strengths + core radii + ages) are staged into
//              shared memory by 1-D TMA bulk copies (cp.async.bulk), double
//              buffered on two mbarriers.  When the target blocks alone cannot
//              fill the SMs, the vortex range is split over gridDim.y and the
//              per-split partial sums go to scratch and are summed in fixed
//              split order by a second kernel (deterministic).
//   expanded   one thread per vortex, looping over a few target points, so
//              that a warp writes 32 consecutive (point, vortex, 3) records.
//
// Arithmetic per (point, leg) follows warp_kernels.py:46-96 operation by
// operation (FMA contraction aside); the four skip tests take the same
// decisions (the |r1 x r2| test compares squares and falls back to the
// reference's sqrt only within a factor 2 of the threshold).
#include "fvx_common.cuh"
#include "fvx_segment_math.cuh"

namespace fvx {
namespace {

using namespace seg;

constexpr int kCollThreads = 128;  // target points per collapsed CTA
constexpr int kTile = 64;          // vortices per shared-memory tile
constexpr int kExpThreads = 64;    // vortices per expanded CTA
__device__ __forceinline__ void flush_counts(int cnt[4], int64_t* counts) {
  if (counts == nullptr) return;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    unsigned v = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(cnt[k]));
    if ((threadIdx.x & 31) == 0 && v != 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(counts + k),
                static_cast<unsigned long long>(v));
  }
}

struct RawTile {
  double c[4][kTile * 3];
  double strength[kTile];
  double rc0[kTile];
  double age[kTile];
};

struct SegArgs {
  const double* points;
  const double* corner[4];
  const double* strengths;
  const double* rc0s;
  const double* ages;  // may be null
  double nu;
  int64_t n_points;
  int64_t n_vort;
  int64_t chunk;  // vortices per split (even)
  double* out;    // (N,3) when gridDim.y == 1, else partials (S,N,3)
  int64_t* counts;
  int use_tma;
};

// Issues the stage-in of vortices [v0, v0+cnt) into `raw`; thread 0 only.
__device__ void issue_tile(const SegArgs& A, RawTile& raw, int64_t v0, int cnt, uint64_t* bar) {
  uint32_t total = 0;
  BulkPlan pc[4], ps, pr, pa;
  for (int c = 0; c < 4; ++c) {
    pc[c] = plan_bulk(A.corner[c], v0, cnt, 24, A.use_tma);
    total += pc[c].bulk_bytes;
  }
  ps = plan_bulk(A.strengths, v0, cnt, 8, A.use_tma);
  pr = plan_bulk(A.rc0s, v0, cnt, 8, A.use_tma);
  pa = A.ages ? plan_bulk(A.ages, v0, cnt, 8, A.use_tma) : BulkPlan{0u, 0u};
  total += ps.bulk_bytes + pr.bulk_bytes + pa.bulk_bytes;
  mbar_arrive_expect_tx(bar, total);
  for (int c = 0; c < 4; ++c)
    if (pc[c].bulk_bytes) bulk_g2s(raw.c[c], A.corner[c] + 3 * v0, pc[c].bulk_bytes, bar);
  if (ps.bulk_bytes) bulk_g2s(raw.strength, A.strengths + v0, ps.bulk_bytes, bar);
  if (pr.bulk_bytes) bulk_g2s(raw.rc0, A.rc0s + v0, pr.bulk_bytes, bar);
  if (pa.bulk_bytes) bulk_g2s(raw.age, A.ages + v0, pa.bulk_bytes, bar);
}

// Plain copies of whatever the bulk copies of the tile did not cover.
__device__ void tail_tile(const SegArgs& A, RawTile& raw, int64_t v0, int cnt) {
  for (int c = 0; c < 4; ++c) {
    BulkPlan p = plan_bulk(A.corner[c], v0, cnt, 24, A.use_tma);
    if (p.tail_bytes) plain_copy8(raw.c[c], A.corner[c] + 3 * v0, p.bulk_bytes, p.tail_bytes);
  }
  BulkPlan p = plan_bulk(A.strengths, v0, cnt, 8, A.use_tma);
  if (p.tail_bytes) plain_copy8(raw.strength, A.strengths + v0, p.bulk_bytes, p.tail_bytes);
  p = plan_bulk(A.rc0s, v0, cnt, 8, A.use_tma);
  if (p.tail_bytes) plain_copy8(raw.rc0, A.rc0s + v0, p.bulk_bytes, p.tail_bytes);
  if (A.ages) {
    p = plan_bulk(A.ages, v0, cnt, 8, A.use_tma);
    if (p.tail_bytes) plain_copy8(raw.age, A.ages + v0, p.bulk_bytes, p.tail_bytes);
  }
}

template <int LEGS>
__global__ void __launch_bounds__(kCollThreads) collapsed_kernel(SegArgs A) {
  __shared__ __align__(128) RawTile raw[2];
  __shared__ __align__(16) VortexRec rec[kTile];
  __shared__ __align__(8) uint64_t bar[2];

  const int64_t i = static_cast<int64_t>(blockIdx.x) * kCollThreads + threadIdx.x;
  const bool active = i < A.n_points;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (active) {
    px = A.points[3 * i + 0];
    py = A.points[3 * i + 1];
    pz = A.points[3 * i + 2];
  }
  const int64_t vb = static_cast<int64_t>(blockIdx.y) * A.chunk;
  const int64_t ve = min(vb + A.chunk, A.n_vort);
  const int ntiles = vb < ve ? static_cast<int>((ve - vb + kTile - 1) / kTile) : 0;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  double vx = 0.0, vy = 0.0, vz = 0.0;
  int cnt[4] = {0, 0, 0, 0};
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  if (ntiles > 0 && threadIdx.x == 0)
    issue_tile(A, raw[0], vb, static_cast<int>(min64(kTile, ve - vb)), &bar[0]);

  int t = 0;
  for (; t < ntiles; ++t) {
    const int buf = t & 1;
    const int64_t v0 = vb + static_cast<int64_t>(t) * kTile;
    const int n = static_cast<int>(min64(kTile, ve - v0));
    if (t + 1 < ntiles && threadIdx.x == 0) {
      const int64_t v1 = v0 + kTile;
      issue_tile(A, raw[buf ^ 1], v1, static_cast<int>(min64(kTile, ve - v1)),
                 &bar[buf ^ 1]);
    }
    if (!mbar_wait(&bar[buf], phase[buf])) {
      ok = false;
      break;
    }
    phase[buf] ^= 1u;
    tail_tile(A, raw[buf], v0, n);
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += kCollThreads) {
      prep_vortex<LEGS>(rec[k], &raw[buf].c[0][3 * k], &raw[buf].c[1][3 * k],
                        &raw[buf].c[2][3 * k], &raw[buf].c[3][3 * k], raw[buf].strength[k],
                        raw[buf].rc0[k], A.ages ? raw[buf].age[k] : 0.0, A.nu);
    }
    __syncthreads();
    if (active) {
      for (int k = 0; k < n; ++k) vortex_velocity<LEGS>(rec[k], px, py, pz, vx, vy, vz, cnt);
    }
    __syncthreads();
  }
  if (!ok) {
    flag_status(kStatusTimeout);
    // Drain the copy that may still be in flight into the other buffer.
    if (threadIdx.x == 0 && t + 1 < ntiles) mbar_wait(&bar[(t + 1) & 1], phase[(t + 1) & 1]);
    return;
  }
  flush_counts(cnt, A.counts);
  if (active) {
    double* o = A.out + (static_cast<int64_t>(blockIdx.y) * A.n_points + i) * 3;
    o[0] = vx;
    o[1] = vy;
    o[2] = vz;
  }
}

// out[i] = sum_s partial[s][i], fixed order.
__global__ void reduce_splits_kernel(const double* __restrict__ partial, int64_t n_vals,
                                     int splits, double* __restrict__ out) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_vals) return;
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += partial[static_cast<int64_t>(k) * n_vals + i];
  out[i] = s;
}

template <int LEGS>
__global__ void __launch_bounds__(kExpThreads) expanded_kernel(SegArgs A, int points_per_cta) {
  extern __shared__ double pts[];  // points_per_cta x 3
  const int64_t m = static_cast<int64_t>(blockIdx.x) * kExpThreads + threadIdx.x;
  const int64_t p0 = static_cast<int64_t>(blockIdx.y) * points_per_cta;
  const int np = static_cast<int>(min64(points_per_cta, A.n_points - p0));
  for (int k = threadIdx.x; k < 3 * np; k += kExpThreads) pts[k] = A.points[3 * p0 + k];
  __syncthreads();
  if (np <= 0) return;
  int cnt[4] = {0, 0, 0, 0};
  if (m < A.n_vort) {
    VortexRec R;
    prep_vortex<LEGS>(R, A.corner[0] + 3 * m, A.corner[1] + 3 * m, A.corner[2] + 3 * m,
                      A.corner[3] + 3 * m, A.strengths[m], A.rc0s[m],
                      A.ages ? A.ages[m] : 0.0, A.nu);
    for (int k = 0; k < np; ++k) {
      double vx = 0.0, vy = 0.0, vz = 0.0;
      vortex_velocity<LEGS>(R, pts[3 * k], pts[3 * k + 1], pts[3 * k + 2], vx, vy, vz, cnt);
      double* o = A.out + ((p0 + k) * A.n_vort + m) * 3;
      o[0] = vx;
      o[1] = vy;
      o[2] = vz;
    }
  }
  flush_counts(cnt, A.counts);
}

// Split of the vortex range for a collapsed call: enough CTAs for about two
// per SM, at least two vortices (and an even count) per split.
int collapsed_splits(int64_t n_points, int64_t n_vort, int64_t* chunk) {
  const int64_t gx = (n_points + kCollThreads - 1) / kCollThreads;
  const int64_t want = 2LL * device_sm_count();
  int64_t s = gx >= want ? 1 : (want + gx - 1) / gx;
  int64_t maxs = (n_vort + 1) / 2;
  if (s > maxs) s = maxs;
  if (s < 1) s = 1;
  int64_t c = (n_vort + s - 1) / s;
  c = (c + 1) & ~int64_t(1);
  s = (n_vort + c - 1) / c;
  *chunk = c;
  return static_cast<int>(s);
}

int check_legs(int leg_set) {
  return leg_set == FVX_LEGS_RING || leg_set == FVX_LEGS_CHORDWISE ||
         leg_set == FVX_LEGS_HORSESHOE;
}

}  // namespace

// Internal launcher shared by the device, host and scratch-free entry points.
int segments_collapsed_launch(const double* points, int64_t n_points, const double* br,
                              const double* fr, const double* fl, const double* bl,
                              const double* strengths, const double* r_c0s, const double* ages,
                              double nu, int64_t n_vort, int leg_set, double* out,
                              int64_t* counts, void* scratch, size_t scratch_bytes,
                              cudaStream_t stream) {
  FVX_ARG_CHECK(check_legs(leg_set), "unknown leg set %d", leg_set);
  FVX_ARG_CHECK(n_points >= 0 && n_vort >= 0, "negative size");
  if (n_points == 0) return FVX_OK;
  FVX_ARG_CHECK(points && out, "null points/out");
  if (n_vort == 0) {
    FVX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * 3 * n_points, stream));
    return FVX_OK;
  }
  FVX_ARG_CHECK(br && fr && fl && bl && strengths && r_c0s, "null vortex array");
  int64_t chunk = 0;
  const int splits = collapsed_splits(n_points, n_vort, &chunk);
  const size_t need = splits > 1 ? sizeof(double) * 3 * n_points * splits : 0;
  if (need > 0 && (scratch == nullptr || scratch_bytes < need)) {
    set_last_error("segments_collapsed needs %zu scratch bytes, got %zu", need, scratch_bytes);
    return FVX_ERR_SCRATCH;
  }
  SegArgs A;
  A.points = points;
  A.corner[0] = br;
  A.corner[1] = fr;
  A.corner[2] = fl;
  A.corner[3] = bl;
  A.strengths = strengths;
  A.rc0s = r_c0s;
  A.ages = ages;
  A.nu = nu;
  A.n_points = n_points;
  A.n_vort = n_vort;
  A.chunk = chunk;
  A.out = splits > 1 ? static_cast<double*>(scratch) : out;
  A.counts = counts;
  A.use_tma = aligned16(br) && aligned16(fr) && aligned16(fl) && aligned16(bl) &&
              aligned16(strengths) && aligned16(r_c0s) && (!ages || aligned16(ages));
  dim3 grid(static_cast<unsigned>((n_points + kCollThreads - 1) / kCollThreads), splits);
  switch (leg_set) {
    case FVX_LEGS_RING:
      collapsed_kernel<FVX_LEGS_RING><<<grid, kCollThreads, 0, stream>>>(A);
      break;
    case FVX_LEGS_CHORDWISE:
      collapsed_kernel<FVX_LEGS_CHORDWISE><<<grid, kCollThreads, 0, stream>>>(A);
      break;
    default:
      collapsed_kernel<FVX_LEGS_HORSESHOE><<<grid, kCollThreads, 0, stream>>>(A);
      break;
  }
  FVX_LAUNCH_CHECK();
  if (splits > 1) {
    const int64_t nv = 3 * n_points;
    reduce_splits_kernel<<<static_cast<unsigned>((nv + 255) / 256), 256, 0, stream>>>(
        static_cast<const double*>(scratch), nv, splits, out);
    FVX_LAUNCH_CHECK();
  }
  return FVX_OK;
}

size_t segments_collapsed_scratch(int64_t n_points, int64_t n_vort) {
  if (n_points <= 0 || n_vort <= 0) return 0;
  int64_t chunk = 0;
  const int splits = collapsed_splits(n_points, n_vort, &chunk);
  return splits > 1 ? sizeof(double) * 3 * n_points * splits : 0;
}

int segments_expanded_launch(const double* points, int64_t n_points, const double* br,
                             const double* fr, const double* fl, const double* bl,
                             const double* strengths, const double* r_c0s, const double* ages,
                             double nu, int64_t n_vort, int leg_set, double* out,
                             int64_t* counts, cudaStream_t stream) {
  FVX_ARG_CHECK(check_legs(leg_set), "unknown leg set %d", leg_set);
  FVX_ARG_CHECK(n_points >= 0 && n_vort >= 0, "negative size");
  if (n_points == 0 || n_vort == 0) return FVX_OK;  // (N,M,3) is empty
  FVX_ARG_CHECK(points && out && br && fr && fl && bl && strengths && r_c0s, "null array");
  SegArgs A;
  A.points = points;
  A.corner[0] = br;
  A.corner[1] = fr;
  A.corner[2] = fl;
  A.corner[3] = bl;
  A.strengths = strengths;
  A.rc0s = r_c0s;
  A.ages = ages;
  A.nu = nu;
  A.n_points = n_points;
  A.n_vort = n_vort;
  A.chunk = 0;
  A.out = out;
  A.counts = counts;
  A.use_tma = 0;
  const int64_t gx = (n_vort + kExpThreads - 1) / kExpThreads;
  const int64_t want = 4LL * device_sm_count();
  int64_t gy = gx >= want ? 1 : (want + gx - 1) / gx;
  if (gy > n_points) gy = n_points;
  int ppc = static_cast<int>((n_points + gy - 1) / gy);
  if (ppc > 512) ppc = 512;
  gy = (n_points + ppc - 1) / ppc;
  FVX_ARG_CHECK(gy <= 65535, "too many target points for one expanded launch");
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  size_t smem = sizeof(double) * 3 * ppc;
  switch (leg_set) {
    case FVX_LEGS_RING:
      expanded_kernel<FVX_LEGS_RING><<<grid, kExpThreads, smem, stream>>>(A, ppc);
      break;
    case FVX_LEGS_CHORDWISE:
      expanded_kernel<FVX_LEGS_CHORDWISE><<<grid, kExpThreads, smem, stream>>>(A, ppc);
      break;
    default:
      expanded_kernel<FVX_LEGS_HORSESHOE><<<grid, kExpThreads, smem, stream>>>(A, ppc);
      break;
  }
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

}  // namespace fvx

extern "C" {

size_t fvx_segments_collapsed_scratch_bytes(int64_t n_points, int64_t n_vortices, int) {
  return fvx::segments_collapsed_scratch(n_points, n_vortices);
}

int fvx_segments_collapsed(const double* points, int64_t n_points, const double* br,
                           const double* fr, const double* fl, const double* bl,
                           const double* strengths, const double* r_c0s, const double* ages,
                           double nu, int64_t n_vortices, int leg_set, double* out,
                           int64_t* singularity_counts, void* scratch, size_t scratch_bytes,
                           void* stream) {
  return fvx::segments_collapsed_launch(points, n_points, br, fr, fl, bl, strengths, r_c0s,
                                        ages, nu, n_vortices, leg_set, out, singularity_counts,
                                        scratch, scratch_bytes,
                                        static_cast<cudaStream_t>(stream));
}

int fvx_segments_expanded(const double* points, int64_t n_points, const double* br,
                          const double* fr, const double* fl, const double* bl,
                          const double* strengths, const double* r_c0s, const double* ages,
                          double nu, int64_t n_vortices, int leg_set, double* out,
                          int64_t* singularity_counts, void* stream) {
  return fvx::segments_expanded_launch(points, n_points, br, fr, fl, bl, strengths, r_c0s,
                                       ages, nu, n_vortices, leg_set, out, singularity_counts,
                                       static_cast<cudaStream_t>(stream));
}

}  // extern "C"
