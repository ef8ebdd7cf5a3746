// fvx_population.cu -- particle population control on the device, FP64.
//
// The population control of the reference's flapping adapter
// (newton_pc/adapters/flap.py:466-563), which keeps the particle count of a
// long run bounded:
//   drop   the oldest particles beyond a maximum count (flap.py:469-473);
//   merge  one pass of pairwise moment-conserving merging (flap.py:478-563):
//          candidates are the particles outside a protected set (the newest
//          `protect` particles, or those within `protect_dist` of the wing
//          centre); each candidate is hashed to a cell of size
//          0.1 + 0.15 |x - c_wing| (key = floor(x / size) per axis); in the
//          stable lexicographic order of the keys, consecutive candidates of
//          one cell are paired greedily from the left when their strengths
//          are aligned (a1 . a2 > 0); a pair becomes one particle with
//          a = a1 + a2, x = (|a1| x1 + |a2| x2) / (|a1| + |a2| + 1e-30) and
//          sigma = max(sigma1, sigma2), accepted when the velocity it induces
//          at the wing reference points changes by less than eps |V_inf|
//          (low-order algebraic core g = rho^3 / (rho^2 + 1)^1.5).
// Survivors keep their order (a stable compaction), so "oldest first" holds
// for the next drop.  The hash, the merge and the error test use the
// reference's operation order without fused multiply-adds, so that they take
// the same decisions as its NumPy code.
#include "fvx_common.cuh"

namespace fvx {

int scan_ints(const int* in, int n, int* out, int inclusive, int* tmp, cudaStream_t s);
int sort_table_ints(int n);
int sort_pairs_u32(uint32_t* keys, int* idx, uint32_t* keys_tmp, int* idx_tmp, int n, int* table,
                   int* scan_tmp, cudaStream_t s, int passes = 4);

namespace {

constexpr int kT = 256;
constexpr int kMaxRef = 64;
constexpr double kFourPi = 12.566370614359172;  // 4 pi, as the reference forms it

__device__ __forceinline__ double norm3(double x, double y, double z) {
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

// flag[i] = 1 for a merge candidate
__global__ void cand_flag_kernel(int n, const double* __restrict__ pos, double cx, double cy,
                                 double cz, int n_free, double dist, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int f;
  if (dist > 0.0)
    f = norm3(__dsub_rn(pos[3 * i], cx), __dsub_rn(pos[3 * i + 1], cy),
              __dsub_rn(pos[3 * i + 2], cz)) > dist;
  else
    f = i < n_free;
  flag[i] = f;
}

// cand[scan[i]] = i for the flagged particles
__global__ void compact_index_kernel(int n, const int* __restrict__ flag,
                                     const int* __restrict__ scan, int* __restrict__ cand) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) cand[scan[i]] = i;
}

// The cell key of candidate c as one 63-bit number whose order is the
// lexicographic order of (kx, ky, kz): 21 bits per axis after a 2^20 bias
// (|k| < 2^20, i.e. positions within ~10^5 cell sizes of the origin).
__global__ void merge_keys_kernel(int nc, const int* __restrict__ cand,
                                  const double* __restrict__ pos, double cx, double cy, double cz,
                                  uint32_t* __restrict__ lo, uint32_t* __restrict__ hi,
                                  int* __restrict__ idx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int i = cand[c];
  const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
  const double d = norm3(__dsub_rn(x, cx), __dsub_rn(y, cy), __dsub_rn(z, cz));
  const double cell = __dadd_rn(0.1, __dmul_rn(0.15, d));
  uint64_t key = 0;
  const double xs[3] = {x, y, z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double k = floor(__ddiv_rn(xs[a], cell)) + 1048576.0;
    k = fmin(fmax(k, 0.0), 2097151.0);
    key = (key << 21) | static_cast<uint64_t>(k);
  }
  lo[c] = static_cast<uint32_t>(key);
  hi[c] = static_cast<uint32_t>(key >> 32);
  idx[c] = c;
}

__global__ void gather_u32_kernel(int n, const int* __restrict__ idx,
                                  const uint32_t* __restrict__ src, uint32_t* __restrict__ dst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[idx[k]];
}

// Greedy pairing from each run start of equal keys (sorted position k), the
// run's thread writing every slot of the run once: consecutive candidates
// pair when their strengths are aligned; a candidate taken as the second of
// a pair is not the first of the next one (flap.py:514-525).
// pair_i/pair_j[a] = the particles of the pair starting at sorted position a.
__global__ void pair_runs_kernel(int nc, const int* __restrict__ order,
                                 const uint32_t* __restrict__ lo, const uint32_t* __restrict__ hi,
                                 const int* __restrict__ cand, const double* __restrict__ alpha,
                                 int* __restrict__ pair_i, int* __restrict__ pair_j) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  auto same = [&](int a, int b) {
    return lo[order[a]] == lo[order[b]] && hi[order[a]] == hi[order[b]];
  };
  if (k > 0 && same(k - 1, k)) return;  // not a run start: its run start writes the slot
  bool skip = false;
  for (int a = k; a < nc; ++a) {
    const bool next = a + 1 < nc && same(a, a + 1);
    int pi = -1, pj = -1;
    if (skip) {
      skip = false;
    } else if (next) {
      const int ci = cand[order[a]], cj = cand[order[a + 1]];
      const double dot = __dadd_rn(__dadd_rn(__dmul_rn(alpha[3 * ci], alpha[3 * cj]),
                                             __dmul_rn(alpha[3 * ci + 1], alpha[3 * cj + 1])),
                                   __dmul_rn(alpha[3 * ci + 2], alpha[3 * cj + 2]));
      if (dot > 0.0) {
        pi = ci;
        pj = cj;
        skip = true;
      }
    }
    pair_i[a] = pi;
    pair_j[a] = pj;
    if (!next) break;
  }
}

// velocity at R of a particle (X, A, S) with the low-order algebraic core
__device__ void ref_velocity(const double* R, const double* X, const double* A, double S,
                             double* v) {
  const double r0 = __dsub_rn(R[0], X[0]), r1 = __dsub_rn(R[1], X[1]), r2 = __dsub_rn(R[2], X[2]);
  const double d = __dadd_rn(norm3(r0, r1, r2), 1e-30);
  const double rho = __ddiv_rn(d, S);
  const double g = __ddiv_rn(pow(rho, 3.0), pow(__dadd_rn(pow(rho, 2.0), 1.0), 1.5));
  const double f = __ddiv_rn(g, __dmul_rn(kFourPi, pow(d, 3.0)));
  v[0] = __dmul_rn(f, __dsub_rn(__dmul_rn(A[1], r2), __dmul_rn(A[2], r1)));
  v[1] = __dmul_rn(f, __dsub_rn(__dmul_rn(A[2], r0), __dmul_rn(A[0], r2)));
  v[2] = __dmul_rn(f, __dsub_rn(__dmul_rn(A[0], r1), __dmul_rn(A[1], r0)));
}

// Pair at sorted position a: the merged particle and its at-wing velocity
// error; accepted merges overwrite the first particle and remove the second.
__global__ void merge_pairs_kernel(int nc, const int* __restrict__ pair_i,
                                   const int* __restrict__ pair_j, double* __restrict__ pos,
                                   double* __restrict__ alpha, double* __restrict__ sigma,
                                   const double* __restrict__ ref, int n_ref, double tol,
                                   int* __restrict__ removed, int* __restrict__ n_merged) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nc) return;
  const int pi = pair_i[a];
  if (pi < 0) return;
  const int pj = pair_j[a];
  double x1[3], x2[3], a1[3], a2[3], xm[3], am[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    x1[c] = pos[3 * pi + c];
    x2[c] = pos[3 * pj + c];
    a1[c] = alpha[3 * pi + c];
    a2[c] = alpha[3 * pj + c];
  }
  const double s1 = sigma[pi], s2 = sigma[pj];
  const double w1 = norm3(a1[0], a1[1], a1[2]), w2 = norm3(a2[0], a2[1], a2[2]);
  const double wd = __dadd_rn(__dadd_rn(w1, w2), 1e-30);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    am[c] = __dadd_rn(a1[c], a2[c]);
    xm[c] = __ddiv_rn(__dadd_rn(__dmul_rn(w1, x1[c]), __dmul_rn(w2, x2[c])), wd);
  }
  const double sm = fmax(s1, s2);
  double err = 0.0;
  for (int r = 0; r < n_ref; ++r) {
    double v1[3], v2[3], vm[3];
    ref_velocity(ref + 3 * r, x1, a1, s1, v1);
    ref_velocity(ref + 3 * r, x2, a2, s2, v2);
    ref_velocity(ref + 3 * r, xm, am, sm, vm);
#pragma unroll
    for (int c = 0; c < 3; ++c) err = fmax(err, fabs(__dsub_rn(__dadd_rn(v1[c], v2[c]), vm[c])));
  }
  if (!(err < tol)) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    pos[3 * pi + c] = xm[c];
    alpha[3 * pi + c] = am[c];
  }
  sigma[pi] = sm;
  removed[pj] = 1;
  atomicAdd(n_merged, 1);
}

// keep[i] = !removed[i] (merge) or i >= drop (drop)
__global__ void keep_flag_kernel(int n, const int* __restrict__ removed, int drop,
                                 int* __restrict__ keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keep[i] = removed ? !removed[i] : (i >= drop);
}

// stable compaction of the kept particles into the temporary arrays
__global__ void scatter_kept_kernel(int n, const int* __restrict__ keep,
                                    const int* __restrict__ scan, const double* __restrict__ pos,
                                    const double* __restrict__ alpha,
                                    const double* __restrict__ sigma,
                                    const double* __restrict__ age, double* __restrict__ tp,
                                    double* __restrict__ ta, double* __restrict__ ts,
                                    double* __restrict__ tg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  const int o = scan[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    tp[3 * o + c] = pos[3 * i + c];
    ta[3 * o + c] = alpha[3 * i + c];
  }
  ts[o] = sigma[i];
  tg[o] = age[i];
}

unsigned nb(int n) { return static_cast<unsigned>((n + kT - 1) / kT); }

struct Scratch {
  int *flag, *scan, *cand, *ia, *ib, *pair_i, *pair_j, *removed, *table, *scan_tmp, *counter;
  uint32_t *lo, *hi, *ka, *kb;
  double *tp, *ta, *ts, *tg;
};

size_t scratch_layout(int64_t n64, char* base, Scratch* S) {
  const size_t n = static_cast<size_t>(n64 > 0 ? n64 : 1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  Scratch s{};
  s.flag = reinterpret_cast<int*>(take(4 * n));
  s.scan = reinterpret_cast<int*>(take(4 * n));
  s.cand = reinterpret_cast<int*>(take(4 * n));
  s.ia = reinterpret_cast<int*>(take(4 * n));
  s.ib = reinterpret_cast<int*>(take(4 * n));
  s.pair_i = reinterpret_cast<int*>(take(4 * n));
  s.pair_j = reinterpret_cast<int*>(take(4 * n));
  s.removed = reinterpret_cast<int*>(take(4 * n));
  s.table = reinterpret_cast<int*>(take(4 * size_t(sort_table_ints(static_cast<int>(n)))));
  s.scan_tmp = reinterpret_cast<int*>(take(4 * 4096));
  s.counter = reinterpret_cast<int*>(take(16));
  s.lo = reinterpret_cast<uint32_t*>(take(4 * n));
  s.hi = reinterpret_cast<uint32_t*>(take(4 * n));
  s.ka = reinterpret_cast<uint32_t*>(take(4 * n));
  s.kb = reinterpret_cast<uint32_t*>(take(4 * n));
  s.tp = reinterpret_cast<double*>(take(24 * n));
  s.ta = reinterpret_cast<double*>(take(24 * n));
  s.ts = reinterpret_cast<double*>(take(8 * n));
  s.tg = reinterpret_cast<double*>(take(8 * n));
  if (S) *S = s;
  return off;
}

// Keeps the particles flagged by keep_flag_kernel (removed != null: merge;
// else those from index drop on), in order; returns the new count.
int compact(int n, const int* removed, int drop, double* pos, double* alpha, double* sigma,
            double* age, const Scratch& S, cudaStream_t s, int* n_new) {
  keep_flag_kernel<<<nb(n), kT, 0, s>>>(n, removed, drop, S.flag);
  FVX_LAUNCH_CHECK();
  int rc = scan_ints(S.flag, n, S.scan, 0, S.scan_tmp, s);
  if (rc) return rc;
  scatter_kept_kernel<<<nb(n), kT, 0, s>>>(n, S.flag, S.scan, pos, alpha, sigma, age, S.tp, S.ta,
                                           S.ts, S.tg);
  FVX_LAUNCH_CHECK();
  int last_scan = 0, last_flag = 0;
  FVX_CUDA_TRY(cudaMemcpyAsync(&last_scan, S.scan + n - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&last_flag, S.flag + n - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  const int m = last_scan + last_flag;
  if (m > 0) {
    FVX_CUDA_TRY(cudaMemcpyAsync(pos, S.tp, 24 * size_t(m), cudaMemcpyDeviceToDevice, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(alpha, S.ta, 24 * size_t(m), cudaMemcpyDeviceToDevice, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(sigma, S.ts, 8 * size_t(m), cudaMemcpyDeviceToDevice, s));
    FVX_CUDA_TRY(cudaMemcpyAsync(age, S.tg, 8 * size_t(m), cudaMemcpyDeviceToDevice, s));
  }
  *n_new = m;
  return FVX_OK;
}

}  // namespace
}  // namespace fvx

extern "C" {

size_t fvx_vpm_population_scratch_bytes(int64_t n) {
  return fvx::scratch_layout(n, nullptr, nullptr);
}

int fvx_vpm_drop_oldest(int64_t n, int64_t keep, double* pos, double* alpha, double* sigma,
                        double* age, int64_t* n_out, void* scratch, size_t scratch_bytes,
                        void* stream) {
  FVX_ARG_CHECK(n >= 0 && n <= (int64_t(1) << 22) && keep >= 0 && n_out, "bad drop arguments");
  *n_out = n;
  if (n <= keep) return FVX_OK;
  FVX_ARG_CHECK(pos && alpha && sigma && age, "null particle arrays");
  FVX_ARG_CHECK(scratch && scratch_bytes >= fvx::scratch_layout(n, nullptr, nullptr),
                "population control needs %zu scratch bytes", fvx::scratch_layout(n, nullptr, nullptr));
  fvx::Scratch S;
  fvx::scratch_layout(n, static_cast<char*>(scratch), &S);
  int m = 0;
  const int rc = fvx::compact(static_cast<int>(n), nullptr, static_cast<int>(n - keep), pos, alpha,
                              sigma, age, S, static_cast<cudaStream_t>(stream), &m);
  if (rc) return rc;
  *n_out = m;
  return FVX_OK;
}

int fvx_vpm_merge_pass(int64_t n, double* pos, double* alpha, double* sigma, double* age,
                       const double* ref_pts, int n_ref, const double* wing_c, double speed,
                       double eps, int64_t protect_newest, double protect_dist, int64_t* n_out,
                       int64_t* n_merged, void* scratch, size_t scratch_bytes, void* stream) {
  FVX_ARG_CHECK(n >= 0 && n <= (int64_t(1) << 22) && n_out && n_merged && wing_c,
                "bad merge arguments");
  FVX_ARG_CHECK(n_ref >= 1 && n_ref <= fvx::kMaxRef && ref_pts, "1..%d reference points",
                fvx::kMaxRef);
  FVX_ARG_CHECK(protect_newest >= 0, "negative protected count");
  *n_out = n;
  *n_merged = 0;
  // flap.py:486-487: too few particles to merge anything
  if (n < 2 * protect_newest || n < 2) return FVX_OK;
  FVX_ARG_CHECK(pos && alpha && sigma && age, "null particle arrays");
  FVX_ARG_CHECK(scratch && scratch_bytes >= fvx::scratch_layout(n, nullptr, nullptr),
                "population control needs %zu scratch bytes", fvx::scratch_layout(n, nullptr, nullptr));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  fvx::Scratch S;
  fvx::scratch_layout(n, static_cast<char*>(scratch), &S);
  const int ni = static_cast<int>(n);
  using fvx::nb;
  using fvx::kT;
  // candidates
  fvx::cand_flag_kernel<<<nb(ni), kT, 0, s>>>(ni, pos, wing_c[0], wing_c[1], wing_c[2],
                                              static_cast<int>(n - protect_newest),
                                              protect_dist > 0.0 ? protect_dist : 0.0, S.flag);
  FVX_LAUNCH_CHECK();
  int rc = fvx::scan_ints(S.flag, ni, S.scan, 0, S.scan_tmp, s);
  if (rc) return rc;
  fvx::compact_index_kernel<<<nb(ni), kT, 0, s>>>(ni, S.flag, S.scan, S.cand);
  FVX_LAUNCH_CHECK();
  int last_scan = 0, last_flag = 0;
  FVX_CUDA_TRY(cudaMemcpyAsync(&last_scan, S.scan + ni - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaMemcpyAsync(&last_flag, S.flag + ni - 1, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  const int nc = last_scan + last_flag;
  // flap.py:494-495: the distance-protected form needs at least 4 candidates
  if (nc < 2 || (protect_dist > 0.0 && nc < 4)) return FVX_OK;
  // keys, stable lexicographic order: by the low word, then by the high word
  fvx::merge_keys_kernel<<<nb(nc), kT, 0, s>>>(nc, S.cand, pos, wing_c[0], wing_c[1], wing_c[2],
                                               S.lo, S.hi, S.ia);
  FVX_LAUNCH_CHECK();
  FVX_CUDA_TRY(cudaMemcpyAsync(S.ka, S.lo, 4 * size_t(nc), cudaMemcpyDeviceToDevice, s));
  if ((rc = fvx::sort_pairs_u32(S.ka, S.ia, S.kb, S.ib, nc, S.table, S.scan_tmp, s))) return rc;
  fvx::gather_u32_kernel<<<nb(nc), kT, 0, s>>>(nc, S.ia, S.hi, S.ka);
  FVX_LAUNCH_CHECK();
  if ((rc = fvx::sort_pairs_u32(S.ka, S.ia, S.kb, S.ib, nc, S.table, S.scan_tmp, s))) return rc;
  // greedy pairs, merges, compaction
  fvx::pair_runs_kernel<<<nb(nc), kT, 0, s>>>(nc, S.ia, S.lo, S.hi, S.cand, alpha, S.pair_i,
                                              S.pair_j);
  FVX_LAUNCH_CHECK();
  FVX_CUDA_TRY(cudaMemsetAsync(S.removed, 0, 4 * size_t(ni), s));
  FVX_CUDA_TRY(cudaMemsetAsync(S.counter, 0, 4, s));
  fvx::merge_pairs_kernel<<<nb(nc), kT, 0, s>>>(nc, S.pair_i, S.pair_j, pos, alpha, sigma,
                                                ref_pts, n_ref, eps * speed, S.removed,
                                                S.counter);
  FVX_LAUNCH_CHECK();
  int merged = 0;
  FVX_CUDA_TRY(cudaMemcpyAsync(&merged, S.counter, 4, cudaMemcpyDeviceToHost, s));
  FVX_CUDA_TRY(cudaStreamSynchronize(s));
  *n_merged = merged;
  if (merged == 0) return FVX_OK;
  int m = 0;
  if ((rc = fvx::compact(ni, S.removed, 0, pos, alpha, sigma, age, S, s, &m))) return rc;
  *n_out = m;
  return FVX_OK;
}

}  // extern "C"
