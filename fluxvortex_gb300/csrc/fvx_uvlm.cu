// fvx_uvlm.cu -- panel side of the hybrid panel-particle step, FP64.
//
// Kernels for one step of a ring-vortex UVLM with a hybrid ring/particle
// wake, in the order the reference's solver runs it (PteraSoftware's step,
// overridden by tests/experiment_hybrid_panel_particle.py:114-204):
//   kinematics      base vertex grid -> vertices at time t (heave + flapping,
//                   per surface)
//   lattice         quarter-chord ring corners, 3/4-chord collocation points,
//                   normals, areas, bound-leg centres/vectors, TE back edge
//   aic             AIC[i,j] = (unit ring j at collocation i) . n_i, the
//                   expanded ring Biot-Savart fused with the normal product
//   rhs             -((U_inf - v_body) + V_wake) . n
//   lu_solve        batched FP64 Gaussian elimination with partial pivoting
//                   (one CTA per system; the AIC system is tiny and stays in L2)
//   loads           Kutta-Joukowski on the bound legs + unsteady term, reduced
//                   to CL and CDi in fixed order (deterministic)
//   wake_rings      ring-wake vertex lattice -> the five-function ring layout
//   shed            prescribed-wake convection + new trailing-edge row
//   convert         HybridSolver._convert_old_wake_to_particles (:145-204):
//                   rows >= N_keep -> 4 particles per ring, appended on the
//                   device with a block-wide compaction
// Several lifting surfaces share one vertex grid (FvxSurfaces): ring strip j
// spans vertex columns col[j], col[j]+1 and vertex column c moves with
// surface surf[c]; ring k = i ns + j.  All per-step inputs are device arrays;
// the host only sequences launches.
#include <cooperative_groups.h>

#include "fvx_common.cuh"
#include "fvx_segment_math.cuh"

namespace fvx {
namespace {

constexpr int kT = 128;

__device__ __forceinline__ void load3(const double* p, int64_t i, double v[3]) {
  v[0] = p[3 * i];
  v[1] = p[3 * i + 1];
  v[2] = p[3 * i + 2];
}
__device__ __forceinline__ void store3(double* p, int64_t i, const double v[3]) {
  p[3 * i] = v[0];
  p[3 * i + 1] = v[1];
  p[3 * i + 2] = v[2];
}

struct Motion {
  double heave_amp, flap_amp, omega, y0, t;
};

__device__ __forceinline__ int strip_col(const FvxSurfaces& s, int j) {
  return s.col ? s.col[j] : j;
}

// Motion of vertex column c at time t: the surface's row of the table
// (heave_amp, flap_amp, omega, y0).
__device__ __forceinline__ Motion column_motion(const FvxSurfaces& s, int c, double t) {
  const double* m = s.motion + 4 * (s.surf ? s.surf[c] : 0);
  return Motion{m[0], m[1], m[2], m[3], t};
}

// Body-point velocity at current position p: heave rate on z, flapping about
// the x axis through the hinge line y = +-y0 of the point's half wing,
// mirrored per half.
__device__ __forceinline__ void body_velocity(const Motion& m, const double p[3], double v[3]) {
  const double h = m.heave_amp * sin(m.omega * m.t);
  const double hdot = m.heave_amp * m.omega * cos(m.omega * m.t);
  const double thdot = m.flap_amp * m.omega * cos(m.omega * m.t);
  const double s = p[1] >= 0.0 ? 1.0 : -1.0;
  const double dy = p[1] - s * m.y0;
  const double Z = p[2] - h;
  v[0] = 0.0;
  v[1] = -s * thdot * Z;
  v[2] = s * thdot * dy + hdot;
}

__global__ void kinematics_kernel(int64_t nv, const double* __restrict__ base, FvxSurfaces sf,
                                  double t, double* __restrict__ out) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const Motion m = column_motion(sf, static_cast<int>(i % sf.w), t);
  double v[3];
  load3(base, i, v);
  if (m.flap_amp != 0.0) {
    const double th = m.flap_amp * sin(m.omega * m.t);
    const double s = v[1] > 0.0 ? 1.0 : (v[1] < 0.0 ? -1.0 : 0.0);
    const double y = fabs(v[1]) - m.y0, z = v[2];
    const double c = cos(th), sn = sin(th);
    v[1] = s * (m.y0 + (y * c - z * sn));
    v[2] = y * sn + z * c;
  }
  if (m.heave_amp != 0.0) v[2] += m.heave_amp * sin(m.omega * m.t);
  store3(out, i, v);
}

struct LatticeOut {
  double *br, *fr, *fl, *bl, *colloc, *normal, *area, *leg_center, *leg_vec, *te_back;
};

// quarter-chord lattice point of vertex (i, j) of a grid w columns wide
__device__ __forceinline__ void vq(const double* v, int nc, int w, int i, int j, double o[3]) {
  double a[3], b[3];
  if (i < nc) {
    load3(v, static_cast<int64_t>(i) * w + j, a);
    load3(v, static_cast<int64_t>(i + 1) * w + j, b);
    for (int c = 0; c < 3; ++c) o[c] = a[c] + 0.25 * (b[c] - a[c]);
  } else {
    load3(v, static_cast<int64_t>(nc) * w + j, a);
    load3(v, static_cast<int64_t>(nc - 1) * w + j, b);
    for (int c = 0; c < 3; ++c) o[c] = a[c] + 0.25 * (a[c] - b[c]);
  }
}

__global__ void lattice_kernel(const double* __restrict__ v, int nc, FvxSurfaces sf,
                               LatticeOut o) {
  const int ns = sf.ns, w = sf.w;
  const int P = nc * ns;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < w) {  // trailing-edge back edge, every vertex column
    double tb[3];
    vq(v, nc, w, nc, k, tb);
    store3(o.te_back, k, tb);
  }
  if (k >= P) return;
  const int i = k / ns, j = strip_col(sf, k % ns);
  double fl[3], fr[3], br[3], bl[3];
  vq(v, nc, w, i, j, fl);
  vq(v, nc, w, i, j + 1, fr);
  vq(v, nc, w, i + 1, j + 1, br);
  vq(v, nc, w, i + 1, j, bl);
  store3(o.fl, k, fl);
  store3(o.fr, k, fr);
  store3(o.br, k, br);
  store3(o.bl, k, bl);
  double a0[3], a1[3], b0[3], b1[3];  // vertices (i,j), (i,j+1), (i+1,j), (i+1,j+1)
  load3(v, static_cast<int64_t>(i) * w + j, a0);
  load3(v, static_cast<int64_t>(i) * w + j + 1, a1);
  load3(v, static_cast<int64_t>(i + 1) * w + j, b0);
  load3(v, static_cast<int64_t>(i + 1) * w + j + 1, b1);
  double cp[3], d1[3], d2[3], lc[3], lv[3];
  for (int c = 0; c < 3; ++c) {
    const double vc0 = a0[c] + 0.75 * (b0[c] - a0[c]);
    const double vc1 = a1[c] + 0.75 * (b1[c] - a1[c]);
    cp[c] = 0.5 * (vc0 + vc1);
    d1[c] = b1[c] - a0[c];
    d2[c] = a1[c] - b0[c];
    lc[c] = 0.5 * (fr[c] + fl[c]);
    lv[c] = fl[c] - fr[c];
  }
  double cr[3] = {d1[1] * d2[2] - d1[2] * d2[1], d1[2] * d2[0] - d1[0] * d2[2],
                  d1[0] * d2[1] - d1[1] * d2[0]};
  const double nrm = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  double n[3] = {cr[0] / nrm, cr[1] / nrm, cr[2] / nrm};
  store3(o.colloc, k, cp);
  store3(o.normal, k, n);
  o.area[k] = 0.5 * nrm;
  store3(o.leg_center, k, lc);
  store3(o.leg_vec, k, lv);
}

// AIC[i, j] for B independent systems laid out back to back.
__global__ void aic_kernel(int P, const double* __restrict__ colloc,
                           const double* __restrict__ normal, const double* __restrict__ br,
                           const double* __restrict__ fr, const double* __restrict__ fl,
                           const double* __restrict__ bl, double rc0, double nu,
                           double* __restrict__ aic) {
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t PP = static_cast<int64_t>(P) * P;
  const int64_t b = blockIdx.y;
  if (idx >= PP) return;
  const int i = static_cast<int>(idx / P), j = static_cast<int>(idx % P);
  const int64_t ii = b * P + i, jj = b * P + j;
  seg::VortexRec R;
  seg::prep_vortex<FVX_LEGS_RING>(R, br + 3 * jj, fr + 3 * jj, fl + 3 * jj, bl + 3 * jj, 1.0, rc0,
                                  0.0, nu);
  double vx = 0.0, vy = 0.0, vz = 0.0;
  int cnt[4] = {0, 0, 0, 0};
  seg::vortex_velocity<FVX_LEGS_RING>(R, colloc[3 * ii], colloc[3 * ii + 1], colloc[3 * ii + 2],
                                      vx, vy, vz, cnt);
  aic[b * PP + idx] = vx * normal[3 * ii] + vy * normal[3 * ii + 1] + vz * normal[3 * ii + 2];
}

// rhs_i = -((U_inf - v_body) + (v1 + v2)) . n   (v1, v2 may be null)
__global__ void rhs_kernel(int P, FvxSurfaces sf, const double* __restrict__ colloc,
                           const double* __restrict__ normal, const double* __restrict__ v1,
                           const double* __restrict__ v2, double ux, double uy, double uz,
                           double t, double* __restrict__ rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const Motion m = column_motion(sf, strip_col(sf, i % sf.ns), t);
  double p[3], vb[3], n[3];
  load3(colloc, i, p);
  load3(normal, i, n);
  body_velocity(m, p, vb);
  double w[3] = {0.0, 0.0, 0.0};
  if (v1) load3(v1, i, w);
  if (v2) {
    w[0] += v2[3 * i];
    w[1] += v2[3 * i + 1];
    w[2] += v2[3 * i + 2];
  }
  const double a0 = (ux - vb[0]) + w[0], a1 = (uy - vb[1]) + w[1], a2 = (uz - vb[2]) + w[2];
  rhs[i] = -(a0 * n[0] + a1 * n[1] + a2 * n[2]);
}

// In-place solve of A x = b for B systems (A: B x P x P row-major, b: B x P);
// Gaussian elimination with partial pivoting (first maximum wins).  x -> b.
// One CTA of kLuThreads per system.  The right-hand side, the pivot row and
// the multipliers live in shared memory.  The first k0 = P - T elimination
// steps run on the matrix in global memory (L2): warp-shuffle pivot search,
// trailing update over 32 warps of rows with the lanes along the columns.
// The trailing T x T block, once it fits, moves into shared memory (row
// stride T + 1) and the remaining T steps run there.  Back substitution:
// the tail block's columns from shared memory, the head rows' share of them
// as one pass over U12 (each row subtracting in the same column order as the
// column-oriented form), then the head columns from U11.  Every element
// sees the same sequence of operations as the all-global form, so the results
// are the same.
constexpr int kLuThreads = 1024;
constexpr int kLuMaxP = 2048;

// Pivot search over v (the candidates' |a|, index i): max |a|, first row on
// ties; every thread returns the winner.
__device__ __forceinline__ int lu_pivot(double best, int bi, double* s_wv, int* s_wi, int* s_piv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_down_sync(0xffffffffu, best, o);
    const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
    if (v2 > best || (v2 == best && i2 < bi)) {
      best = v2;
      bi = i2;
    }
  }
  if (lane == 0) {
    s_wv[warp] = best;
    s_wi[warp] = bi;
  }
  __syncthreads();
  if (warp == 0) {
    best = s_wv[lane];
    bi = s_wi[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_down_sync(0xffffffffu, best, o);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
      if (v2 > best || (v2 == best && i2 < bi)) {
        best = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      *s_piv = bi;
      if (!(best > 0.0)) flag_status(kStatusNonFinite);
    }
  }
  __syncthreads();
  return *s_piv;
}

// Dynamic shared memory: s_x[P], s_row[P], s_l[P], then the tail block
// (T rows of stride T + 1).
__global__ void __launch_bounds__(kLuThreads) lu_solve_kernel(int P, int T, double* __restrict__ A,
                                                              double* __restrict__ b) {
  extern __shared__ double lu_smem[];
  double* s_x = lu_smem;
  double* s_row = s_x + P;
  double* s_l = s_row + P;
  double* S = s_l + P;
  const int ld = T + 1;
  __shared__ double s_wv[kLuThreads / 32];
  __shared__ int s_wi[kLuThreads / 32];
  __shared__ int s_piv;
  const int64_t PP = static_cast<int64_t>(P) * P;
  double* a = A + blockIdx.x * PP;
  double* x = b + static_cast<int64_t>(blockIdx.x) * P;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k0 = P - T;
  for (int r = tid; r < P; r += kLuThreads) s_x[r] = x[r];
  __syncthreads();
  // ---- head steps on the matrix in global memory
  for (int k = 0; k < k0; ++k) {
    double best = -1.0;
    int bi = P;
    for (int r = k + tid; r < P; r += kLuThreads) {
      const double v = fabs(a[static_cast<int64_t>(r) * P + k]);
      if (v > best) {
        best = v;
        bi = r;
      }
    }
    const int piv = lu_pivot(best, bi, s_wv, s_wi, &s_piv);
    // swap rows k and piv (the whole rows) and cache row k
    for (int c = tid; c < P; c += kLuThreads) {
      double rk = a[static_cast<int64_t>(k) * P + c];
      if (piv != k && piv < P) {
        const double rp = a[static_cast<int64_t>(piv) * P + c];
        a[static_cast<int64_t>(piv) * P + c] = rk;
        a[static_cast<int64_t>(k) * P + c] = rp;
        rk = rp;
      }
      s_row[c] = rk;
    }
    if (tid == 0 && piv != k && piv < P) {
      const double t = s_x[k];
      s_x[k] = s_x[piv];
      s_x[piv] = t;
    }
    __syncthreads();
    const double akk = s_row[k];
    const double xk = s_x[k];
    for (int r = k + 1 + tid; r < P; r += kLuThreads) {
      const double l = a[static_cast<int64_t>(r) * P + k] / akk;
      s_l[r] = l;
      s_x[r] -= l * xk;
    }
    __syncthreads();
    for (int r = k + 1 + warp; r < P; r += kLuThreads / 32) {
      const double l = s_l[r];
      double* ar = a + static_cast<int64_t>(r) * P;
      for (int c = k + 1 + lane; c < P; c += 32) ar[c] -= l * s_row[c];
    }
    __syncthreads();
  }
  // ---- the trailing block into shared memory
  for (int e = tid; e < T * T; e += kLuThreads) {
    const int r = e / T, c = e - r * T;
    S[r * ld + c] = a[static_cast<int64_t>(k0 + r) * P + k0 + c];
  }
  __syncthreads();
  for (int kk = 0; kk < T; ++kk) {
    double best = -1.0;
    int bi = T;
    for (int r = kk + tid; r < T; r += kLuThreads) {
      const double v = fabs(S[r * ld + kk]);
      if (v > best) {
        best = v;
        bi = r;
      }
    }
    const int piv = lu_pivot(best, bi, s_wv, s_wi, &s_piv);
    // swap rows kk and piv of the block (columns kk.. are U's), cache row kk
    for (int c = kk + tid; c < T; c += kLuThreads) {
      double rk = S[kk * ld + c];
      if (piv != kk && piv < T) {
        const double rp = S[piv * ld + c];
        S[piv * ld + c] = rk;
        S[kk * ld + c] = rp;
        rk = rp;
      }
      s_row[c] = rk;
    }
    if (tid == 0 && piv != kk && piv < T) {
      const double t = s_x[k0 + kk];
      s_x[k0 + kk] = s_x[k0 + piv];
      s_x[k0 + piv] = t;
    }
    __syncthreads();
    const double akk = s_row[kk];
    const double xk = s_x[k0 + kk];
    for (int r = kk + 1 + tid; r < T; r += kLuThreads) {
      const double l = S[r * ld + kk] / akk;
      s_l[r] = l;
      s_x[k0 + r] -= l * xk;
    }
    __syncthreads();
    for (int r = kk + 1 + warp; r < T; r += kLuThreads / 32) {
      const double l = s_l[r];
      double* sr = S + r * ld;
      for (int c = kk + 1 + lane; c < T; c += 32) sr[c] -= l * s_row[c];
    }
    __syncthreads();
  }
  // ---- back substitution: the tail columns
  for (int kk = T - 1; kk >= 0; --kk) {
    const double xk = s_x[k0 + kk] / S[kk * ld + kk];
    for (int r = tid; r < kk; r += kLuThreads) s_x[k0 + r] -= S[r * ld + kk] * xk;
    __syncthreads();
    if (tid == 0) s_x[k0 + kk] = xk;
    __syncthreads();
  }
  // the head rows' share of the tail columns (U12), columns in descending order
  for (int r = tid; r < k0; r += kLuThreads) {
    const double* ar = a + static_cast<int64_t>(r) * P + k0;
    double v = s_x[r];
    for (int c = T - 1; c >= 0; --c) v -= ar[c] * s_x[k0 + c];
    s_x[r] = v;
  }
  __syncthreads();
  // the head columns: U11 from shared memory when it fits in the block's room
  const bool u11_smem = k0 <= T;
  if (u11_smem) {
    for (int e = tid; e < k0 * k0; e += kLuThreads) {
      const int r = e / k0, c = e - r * k0;
      S[r * ld + c] = a[static_cast<int64_t>(r) * P + c];
    }
    __syncthreads();
  }
  for (int k = k0 - 1; k >= 0; --k) {
    const double ukk = u11_smem ? S[k * ld + k] : a[static_cast<int64_t>(k) * P + k];
    const double xk = s_x[k] / ukk;
    for (int r = tid; r < k; r += kLuThreads)
      s_x[r] -= (u11_smem ? S[r * ld + k] : a[static_cast<int64_t>(r) * P + k]) * xk;
    __syncthreads();
    if (tid == 0) s_x[k] = xk;
    __syncthreads();
  }
  for (int r = tid; r < P; r += kLuThreads) x[r] = s_x[r];
}

// The same solve on a cluster of kLuCtas CTAs (systems with P <= kLuClusterMaxP):
// one SM's FP64 pipe bounds the single-CTA form, so the columns are dealt out
// cyclically (column j to CTA j mod kLuCtas, kept whole in its shared memory).
// Step k: the owner of column k searches its pivot, swaps and forms the
// multipliers in its own shared memory; after one cluster barrier every CTA
// reads them (distributed shared memory), swaps rows k and piv in its
// columns, updates its copy of the right-hand side and its trailing columns.
// The multipliers alternate between two buffers, so one barrier per step
// suffices (the owner of step k + 2 writes only after every CTA has passed
// step k + 1's barrier, i.e. finished step k).  Every element sees the same
// operations in the same order as the single-CTA form, so the factors and the
// solution are the same.  The upper triangle is then gathered, packed, into
// CTA 0, which back-substitutes.
namespace cg = cooperative_groups;
constexpr int kLuCtas = 8;
constexpr int kLuClusterThreads = 256;
constexpr int kLuClusterMaxP = 192;  // packed U, P (P + 1) / 2 doubles, in CTA 0
static_assert(kLuClusterThreads >= kLuClusterMaxP, "the replayed solve takes one row per thread");

// doubles of one system's factorisation workspace: multipliers P x P, pivots
// P, packed U P (P + 1) / 2
__host__ __device__ constexpr int64_t lu_workspace_doubles(int P) {
  return static_cast<int64_t>(P) * P + P + static_cast<int64_t>(P) * (P + 1) / 2;
}

// Back substitution with the packed upper triangle (column j's rows 0..j at
// j (j + 1) / 2), x in place; every thread of the CTA takes part.
__device__ __forceinline__ void back_substitute(int P, const double* s_u, double* s_x, int tid,
                                                int NT) {
  for (int k = P - 1; k >= 0; --k) {
    const int base = k * (k + 1) / 2;
    const double xk = s_x[k] / s_u[base + k];
    for (int r = tid; r < k; r += NT) s_x[r] -= s_u[base + r] * xk;
    __syncthreads();
    if (tid == 0) s_x[k] = xk;
    __syncthreads();
  }
}

// Dynamic shared memory per CTA: panel[ceil(P/kLuCtas)][P] (column-major),
// s_l[2][P], s_x[P], packed U[P (P + 1) / 2] (used in CTA 0).
// FACTOR: the factorisation alone, no right-hand side: step k's multipliers
// (as formed at step k), its pivot and the packed upper triangle go to the
// workspace W (lu_workspace), from which lu_solve_factored_kernel replays the
// same elimination on a right-hand side later (same operations, same order:
// the same solution bit for bit), so the factorisation can run while the
// right-hand side is still being formed.
template <bool FACTOR>
__global__ void __cluster_dims__(kLuCtas, 1, 1) __launch_bounds__(kLuClusterThreads)
    lu_cluster_kernel(int P, double* __restrict__ A, double* __restrict__ b,
                      double* __restrict__ W) {
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double lc_smem[];
  const int rank = static_cast<int>(cl.block_rank());
  const int sys = blockIdx.x / kLuCtas;
  double* a = A + static_cast<int64_t>(sys) * P * P;
  double* xg = FACTOR ? nullptr : b + static_cast<int64_t>(sys) * P;
  // workspace of this system: multipliers L[k][r] (row k: step k's, r > k),
  // pivots (as doubles), packed U
  double* wl = FACTOR ? W + static_cast<int64_t>(sys) * lu_workspace_doubles(P) : nullptr;
  double* wp = FACTOR ? wl + static_cast<int64_t>(P) * P : nullptr;
  double* wu = FACTOR ? wp + P : nullptr;
  const int ncmax = (P + kLuCtas - 1) / kLuCtas;
  const int ncol = rank < P ? (P - rank + kLuCtas - 1) / kLuCtas : 0;
  double* panel = lc_smem;
  double* s_l = panel + static_cast<size_t>(ncmax) * P;
  double* s_x = s_l + 2 * P;
  double* s_u = s_x + P;
  __shared__ double s_wv[kLuClusterThreads / 32];
  __shared__ int s_wi[kLuClusterThreads / 32];
  __shared__ int s_piv[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NT = kLuClusterThreads;
  for (int e = tid; e < ncol * P; e += NT) {
    const int q = e / P, r = e - q * P;
    panel[q * P + r] = a[static_cast<int64_t>(r) * P + rank + kLuCtas * q];
  }
  if (!FACTOR)
    for (int r = tid; r < P; r += NT) s_x[r] = xg[r];
  __syncthreads();
  for (int k = 0; k < P; ++k) {
    const int o = k % kLuCtas, par = k & 1;
    double* l_own = s_l + par * P;
    if (rank == o) {
      double* col = panel + (k / kLuCtas) * P;
      double best = -1.0;
      int bi = P;
      for (int r = k + tid; r < P; r += NT) {
        const double v = fabs(col[r]);
        if (v > best) {
          best = v;
          bi = r;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const double v2 = __shfl_down_sync(0xffffffffu, best, off);
        const int i2 = __shfl_down_sync(0xffffffffu, bi, off);
        if (v2 > best || (v2 == best && i2 < bi)) {
          best = v2;
          bi = i2;
        }
      }
      if (lane == 0) {
        s_wv[warp] = best;
        s_wi[warp] = bi;
      }
      __syncthreads();
      if (tid == 0) {
        best = s_wv[0];
        bi = s_wi[0];
        for (int w = 1; w < NT / 32; ++w)
          if (s_wv[w] > best || (s_wv[w] == best && s_wi[w] < bi)) {
            best = s_wv[w];
            bi = s_wi[w];
          }
        if (!(best > 0.0)) flag_status(kStatusNonFinite);
        s_piv[par] = bi;
        if (bi != k && bi < P) {
          const double t = col[k];
          col[k] = col[bi];
          col[bi] = t;
        }
      }
      __syncthreads();
      const double akk = col[k];
      for (int r = k + 1 + tid; r < P; r += NT) l_own[r] = col[r] / akk;
      if (FACTOR) {
        for (int r = k + 1 + tid; r < P; r += NT) wl[static_cast<int64_t>(k) * P + r] = l_own[r];
        if (tid == 0) wp[k] = static_cast<double>(s_piv[par]);
      }
    }
    cl.sync();
    const double* l_src = cl.map_shared_rank(l_own, o);
    const int piv = *cl.map_shared_rank(s_piv + par, o);
    if (rank != o)
      for (int r = k + 1 + tid; r < P; r += NT) l_own[r] = l_src[r];
    // rows k and piv in this CTA's columns j > k (the owner's column k is done)
    const int q0 = (k + 1 - rank + kLuCtas - 1) / kLuCtas > 0 ? (k + 1 - rank + kLuCtas - 1) / kLuCtas
                                                             : 0;  // first q with j > k
    if (piv != k && piv < P)
      for (int q = q0 + tid; q < ncol; q += NT) {
        double* c = panel + q * P;
        const double t = c[k];
        c[k] = c[piv];
        c[piv] = t;
      }
    if (!FACTOR && tid == 0 && piv != k && piv < P) {
      const double t = s_x[k];
      s_x[k] = s_x[piv];
      s_x[piv] = t;
    }
    __syncthreads();
    if (!FACTOR) {
      const double xk = s_x[k];
      for (int r = k + 1 + tid; r < P; r += NT) s_x[r] -= l_own[r] * xk;
    }
    // trailing update of this CTA's columns j > k, rows r > k
    const int nq = ncol - q0, nr = P - k - 1;
    for (int e = tid; e < nq * nr; e += NT) {
      const int qq = e / nr, r = k + 1 + (e - qq * nr);
      double* c = panel + (q0 + qq) * P;
      c[r] -= l_own[r] * c[k];
    }
    __syncthreads();
  }
  // gather the upper triangle, packed by columns, into CTA 0
  double* u0 = cl.map_shared_rank(s_u, 0);
  for (int q = 0; q < ncol; ++q) {
    const int j = rank + kLuCtas * q;
    const int base = j * (j + 1) / 2;
    for (int r = tid; r <= j; r += NT) u0[base + r] = panel[q * P + r];
  }
  cl.sync();
  if (rank == 0) {
    if (FACTOR) {
      for (int e = tid; e < P * (P + 1) / 2; e += NT) wu[e] = s_u[e];
      return;
    }
    back_substitute(P, s_u, s_x, tid, NT);
    for (int r = tid; r < P; r += NT) xg[r] = s_x[r];
  }
}

// The solve of a factorisation left by lu_cluster_kernel<true> in W: the
// fused kernel's right-hand-side operations replayed in its order (the pivot
// swap and the multipliers of step k, k = 0..P-1, then the back
// substitution), one CTA per system.  Dynamic shared memory: s_x[P], packed
// U[P (P + 1) / 2], the pivots[P].
__global__ void __launch_bounds__(kLuClusterThreads)
    lu_solve_factored_kernel(int P, const double* __restrict__ W, double* __restrict__ b) {
  extern __shared__ double sf_smem[];
  const int sys = blockIdx.x;
  const double* wl = W + static_cast<int64_t>(sys) * lu_workspace_doubles(P);
  const double* wp = wl + static_cast<int64_t>(P) * P;
  const double* wu = wp + P;
  double* xg = b + static_cast<int64_t>(sys) * P;
  double* s_x = sf_smem;
  double* s_u = s_x + P;
  double* s_p = s_u + P * (P + 1) / 2;  // pivots
  const int tid = threadIdx.x;
  constexpr int NT = kLuClusterThreads;  // >= P: one row per thread and step
  for (int r = tid; r < P; r += NT) {
    s_x[r] = xg[r];
    s_p[r] = wp[r];
  }
  for (int e = tid; e < P * (P + 1) / 2; e += NT) s_u[e] = wu[e];
  __syncthreads();
  // step k updates row k + 1 + tid with step k's multiplier for that row; the
  // next step's multiplier is loaded while this step's barrier waits
  double lcur = 1 + tid < P ? wl[1 + tid] : 0.0;
  for (int k = 0; k < P; ++k) {
    const int piv = static_cast<int>(s_p[k]);
    if (tid == 0 && piv != k && piv < P) {
      const double t = s_x[k];
      s_x[k] = s_x[piv];
      s_x[piv] = t;
    }
    __syncthreads();
    const double xk = s_x[k];
    const int rn = k + 2 + tid;
    const double lnext = rn < P ? wl[static_cast<int64_t>(k + 1) * P + rn] : 0.0;
    const int r = k + 1 + tid;
    if (r < P) s_x[r] -= lcur * xk;
    lcur = lnext;
    __syncthreads();
  }
  back_substitute(P, s_u, s_x, tid, NT);
  for (int r = tid; r < P; r += NT) xg[r] = s_x[r];
}

struct LoadsArgs {
  int nc;
  FvxSurfaces sf;
  const double* gamma;
  const double* gamma_prev;  // null: no unsteady term (first step)
  const double* leg_center;
  const double* leg_vec;
  const double* area;
  const double* normal;
  const double* v1;  // induced velocities at the leg centres (summed, any may be null)
  const double* v2;
  const double* v3;
  double ux, uy, uz, rho, dt, t;
  double s_ref;     // <= 0: the sum of the panel areas
  double* cl_out;   // cl_out[0], cdi_out[0] written
  double* cdi_out;
  double* force;    // optional (P,3) per-panel force
};

__global__ void __launch_bounds__(256) loads_kernel(LoadsArgs a) {
  const int ns = a.sf.ns;
  const int P = a.nc * ns;
  double F[3] = {0.0, 0.0, 0.0}, S = 0.0;
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const int i = k / ns;
    const double g = a.gamma[k];
    const double geff = i > 0 ? g - a.gamma[k - ns] : g;
    double p[3], vb[3], l[3], n[3];
    load3(a.leg_center, k, p);
    load3(a.leg_vec, k, l);
    load3(a.normal, k, n);
    body_velocity(column_motion(a.sf, strip_col(a.sf, k % ns), a.t), p, vb);
    double w[3] = {0.0, 0.0, 0.0};
    if (a.v1) load3(a.v1, k, w);
    if (a.v2) {
      w[0] += a.v2[3 * k];
      w[1] += a.v2[3 * k + 1];
      w[2] += a.v2[3 * k + 2];
    }
    if (a.v3) {
      w[0] += a.v3[3 * k];
      w[1] += a.v3[3 * k + 1];
      w[2] += a.v3[3 * k + 2];
    }
    const double V0 = (a.ux - vb[0]) + w[0], V1 = (a.uy - vb[1]) + w[1],
                 V2 = (a.uz - vb[2]) + w[2];
    const double cx = V1 * l[2] - V2 * l[1], cy = V2 * l[0] - V0 * l[2],
                 cz = V0 * l[1] - V1 * l[0];
    const double dg = a.gamma_prev ? (g - a.gamma_prev[k]) / a.dt : 0.0;
    const double ua = a.rho * dg * a.area[k];
    const double f0 = a.rho * geff * cx - ua * n[0];
    const double f1 = a.rho * geff * cy - ua * n[1];
    const double f2 = a.rho * geff * cz - ua * n[2];
    if (a.force) {
      a.force[3 * k] = f0;
      a.force[3 * k + 1] = f1;
      a.force[3 * k + 2] = f2;
    }
    F[0] += f0;
    F[1] += f1;
    F[2] += f2;
    S += a.area[k];
  }
  __shared__ double red[4][256];
  red[0][threadIdx.x] = F[0];
  red[1][threadIdx.x] = F[1];
  red[2][threadIdx.x] = F[2];
  red[3][threadIdx.x] = S;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double V = sqrt(a.ux * a.ux + a.uy * a.uy + a.uz * a.uz);
    const double eD[3] = {a.ux / V, a.uy / V, a.uz / V};
    const double eL[3] = {-eD[2], 0.0, eD[0]};
    const double qS = 0.5 * a.rho * V * V * (a.s_ref > 0.0 ? a.s_ref : red[3][0]);
    a.cl_out[0] = (red[0][0] * eL[0] + red[1][0] * eL[1] + red[2][0] * eL[2]) / qS;
    a.cdi_out[0] = (red[0][0] * eD[0] + red[1][0] * eD[1] + red[2][0] * eD[2]) / qS;
  }
}

// Unsteady Bernoulli loads (newton_pc/adapters/flap.py:357-377): per panel
// the chordwise and spanwise tangents between the midpoints of its vertex
// edges, the circulation gradients along them (first row / first strip of a
// surface: the panel's own strength), and the pressure jump
// dp = rho (V . t_c dG/dc + V . t_s dG/ds + dG/dt) acting along the normal
// over the panel area, V = u_inf - v_body + v1 + v2 at the collocation point
// (the wake rings and particles; no bound self-induction).
struct BernoulliArgs {
  int nc;
  FvxSurfaces sf;
  const double* verts;
  const double* gamma;
  const double* gamma_prev;  // null: no unsteady term
  const double* colloc;
  const double* area;
  const double* normal;
  const double* v1;
  const double* v2;
  double ux, uy, uz, rho, dt, t, s_ref;
  double* cl_out;
  double* cdi_out;
  double* force;
};

__global__ void __launch_bounds__(256) bernoulli_loads_kernel(BernoulliArgs a) {
  const int ns = a.sf.ns, w = a.sf.w;
  const int P = a.nc * ns;
  double F[3] = {0.0, 0.0, 0.0}, S = 0.0;
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const int i = k / ns, jj = k % ns, c = strip_col(a.sf, jj);
    double a0[3], a1[3], b0[3], b1[3];
    load3(a.verts, static_cast<int64_t>(i) * w + c, a0);
    load3(a.verts, static_cast<int64_t>(i) * w + c + 1, a1);
    load3(a.verts, static_cast<int64_t>(i + 1) * w + c, b0);
    load3(a.verts, static_cast<int64_t>(i + 1) * w + c + 1, b1);
    double tc[3], ts[3];
    for (int q = 0; q < 3; ++q) {
      tc[q] = 0.5 * (b1[q] + b0[q]) - 0.5 * (a1[q] + a0[q]);
      ts[q] = 0.5 * (b1[q] + a1[q]) - 0.5 * (b0[q] + a0[q]);
    }
    const double dc = sqrt(tc[0] * tc[0] + tc[1] * tc[1] + tc[2] * tc[2]);
    const double ds = sqrt(ts[0] * ts[0] + ts[1] * ts[1] + ts[2] * ts[2]);
    const double g = a.gamma[k];
    const bool first_strip = jj == 0 || strip_col(a.sf, jj - 1) + 1 != c;
    const double dgc = (i > 0 ? g - a.gamma[k - ns] : g) / dc;
    const double dgs = (first_strip ? g : g - a.gamma[k - 1]) / ds;
    double p[3], vb[3], n[3];
    load3(a.colloc, k, p);
    load3(a.normal, k, n);
    body_velocity(column_motion(a.sf, c, a.t), p, vb);
    double wv[3] = {0.0, 0.0, 0.0};
    if (a.v1) load3(a.v1, k, wv);
    if (a.v2)
      for (int q = 0; q < 3; ++q) wv[q] += a.v2[3 * k + q];
    const double V0 = (a.ux - vb[0]) + wv[0], V1 = (a.uy - vb[1]) + wv[1],
                 V2 = (a.uz - vb[2]) + wv[2];
    const double vtc = (V0 * tc[0] + V1 * tc[1] + V2 * tc[2]) / dc;
    const double vts = (V0 * ts[0] + V1 * ts[1] + V2 * ts[2]) / ds;
    const double dgdt = a.gamma_prev ? (g - a.gamma_prev[k]) / a.dt : 0.0;
    // the reference's rings circulate front-left -> front-right -> back-right
    // -> back-left (flap.py:330-332), against PteraSoftware's (these
    // strengths): the same flow has the opposite strengths, so dp changes sign
    const double dp = -a.rho * (vtc * dgc + vts * dgs + dgdt);
    const double f0 = dp * a.area[k] * n[0], f1 = dp * a.area[k] * n[1],
                 f2 = dp * a.area[k] * n[2];
    if (a.force) {
      a.force[3 * k] = f0;
      a.force[3 * k + 1] = f1;
      a.force[3 * k + 2] = f2;
    }
    F[0] += f0;
    F[1] += f1;
    F[2] += f2;
    S += a.area[k];
  }
  __shared__ double red[4][256];
  red[0][threadIdx.x] = F[0];
  red[1][threadIdx.x] = F[1];
  red[2][threadIdx.x] = F[2];
  red[3][threadIdx.x] = S;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double V = sqrt(a.ux * a.ux + a.uy * a.uy + a.uz * a.uz);
    const double eD[3] = {a.ux / V, a.uy / V, a.uz / V};
    const double eL[3] = {-eD[2], 0.0, eD[0]};
    const double qS = 0.5 * a.rho * V * V * (a.s_ref > 0.0 ? a.s_ref : red[3][0]);
    a.cl_out[0] = (red[0][0] * eL[0] + red[1][0] * eL[1] + red[2][0] * eL[2]) / qS;
    a.cdi_out[0] = (red[0][0] * eD[0] + red[1][0] * eD[1] + red[2][0] * eD[2]) / qS;
  }
}

// Ring wake (R rows x ns rings) from the vertex lattice W ((R+1) x w).
__global__ void wake_rings_kernel(int R, FvxSurfaces sf, const double* __restrict__ W,
                                  const double* __restrict__ gam, const double* __restrict__ age,
                                  double rc0, double* br, double* fr, double* fl, double* bl,
                                  double* strength, double* rc0s, double* ages) {
  const int ns = sf.ns, w = sf.w;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= R * ns) return;
  const int r = k / ns, j = strip_col(sf, k % ns);
  double p[3];
  load3(W, static_cast<int64_t>(r) * w + j, p);
  store3(fl, k, p);
  load3(W, static_cast<int64_t>(r) * w + j + 1, p);
  store3(fr, k, p);
  load3(W, static_cast<int64_t>(r + 1) * w + j + 1, p);
  store3(br, k, p);
  load3(W, static_cast<int64_t>(r + 1) * w + j, p);
  store3(bl, k, p);
  strength[k] = gam[k];
  rc0s[k] = rc0;
  ages[k] = age[r];
}

// New wake from the old one: row 0 = trailing edge of the next step, rows
// m >= 1 = old rows convected by U_inf dt; strengths shift by one row and take
// the trailing-edge ring strengths; ages shift and grow by dt.
// Free ring wake: v1..v3 (any null) are velocities induced at the old
// vertices, which then move by (u_inf + v1 + v2 + v3) dt; all null: the
// prescribed wake (u_inf dt).
__global__ void shed_kernel(int R_old, int nc, int ns, int w, const double* __restrict__ W_old,
                            const double* __restrict__ gam_old,
                            const double* __restrict__ age_old,
                            const double* __restrict__ te_next, const double* __restrict__ gamma,
                            double ux, double uy, double uz, double dt,
                            const double* __restrict__ v1, const double* __restrict__ v2,
                            const double* __restrict__ v3, double* __restrict__ W_new,
                            double* __restrict__ gam_new, double* __restrict__ age_new) {
  const int nverts = (R_old + 2) * w;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nverts) {
    const int r = k / w, j = k % w;
    double p[3];
    if (r == 0) {
      load3(te_next, j, p);
    } else {
      const int64_t o = static_cast<int64_t>(r - 1) * w + j;
      load3(W_old, o, p);
      if (v1 || v2 || v3) {
        double v[3] = {ux, uy, uz};
        const double* vs[3] = {v1, v2, v3};
        for (int q = 0; q < 3; ++q)
          if (vs[q])
            for (int c = 0; c < 3; ++c) v[c] += vs[q][3 * o + c];
        for (int c = 0; c < 3; ++c) p[c] = __dadd_rn(p[c], __dmul_rn(v[c], dt));
      } else {
        // u dt rounded, then added (no fused multiply-add)
        p[0] = __dadd_rn(p[0], __dmul_rn(ux, dt));
        p[1] = __dadd_rn(p[1], __dmul_rn(uy, dt));
        p[2] = __dadd_rn(p[2], __dmul_rn(uz, dt));
      }
    }
    store3(W_new, k, p);
  }
  if (k < (R_old + 1) * ns) {
    const int r = k / ns, j = k % ns;
    gam_new[k] = r == 0 ? gamma[(nc - 1) * ns + j] : gam_old[(r - 1) * ns + j];
  }
  if (k < R_old + 1) age_new[k] = k == 0 ? 0.0 : age_old[k - 1] + dt;
}

// Rows r >= n_keep of the wake lattice -> particles appended at *count.
__global__ void __launch_bounds__(256) convert_kernel(int R, int n_keep, FvxSurfaces sf,
                                                      const double* __restrict__ W,
                                                      const double* __restrict__ gam,
                                                      int sigma_rule, double sigma_vdt,
                                                      int64_t capacity, int64_t* count,
                                                      double* pos, double* alpha, double* sigma,
                                                      double* age) {
  __shared__ int s_scan[256];
  __shared__ int64_t s_base;
  if (threadIdx.x == 0) s_base = *count;
  __syncthreads();
  const int ns = sf.ns, w = sf.w;
  const int nrings = (R - n_keep) * ns;
  for (int c0 = 0; c0 < nrings; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    double q[4][3], al[4][3];
    int emit = 0, mask = 0;
    double sg = sigma_vdt;
    if (k < nrings) {
      const int r = n_keep + k / ns, j = strip_col(sf, k % ns);
      const double g = gam[r * ns + k % ns];
      double fl[3], fr[3], bl[3], br[3];
      load3(W, static_cast<int64_t>(r) * w + j, fl);
      load3(W, static_cast<int64_t>(r) * w + j + 1, fr);
      load3(W, static_cast<int64_t>(r + 1) * w + j, bl);
      load3(W, static_cast<int64_t>(r + 1) * w + j + 1, br);
      const double* A[4] = {fr, fl, bl, br};  // legs front, left, back, right
      const double* B[4] = {fl, bl, br, fr};
      if (sigma_rule == 1) {
        double e = 0.0;
        for (int l = 0; l < 4; ++l) {
          const double d0 = A[l][0] - B[l][0], d1 = A[l][1] - B[l][1], d2 = A[l][2] - B[l][2];
          e += sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        }
        sg = 1.3 * 0.25 * e;
      }
      if (!(fabs(g) < 1e-15)) {
        for (int l = 0; l < 4; ++l) {
          double s2 = 0.0;
          for (int c = 0; c < 3; ++c) {
            al[l][c] = g * (B[l][c] - A[l][c]);
            q[l][c] = 0.5 * (A[l][c] + B[l][c]);
            s2 += al[l][c] * al[l][c];
          }
          if (s2 > 1e-30) {
            mask |= 1 << l;
            ++emit;
          }
        }
      }
    }
    // block-wide exclusive scan of emit (ring-major order)
    s_scan[threadIdx.x] = emit;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
      int v = threadIdx.x >= off ? s_scan[threadIdx.x - off] : 0;
      __syncthreads();
      s_scan[threadIdx.x] += v;
      __syncthreads();
    }
    const int incl = s_scan[threadIdx.x];
    const int total = s_scan[blockDim.x - 1];
    int64_t o = s_base + incl - emit;
    for (int l = 0; l < 4; ++l) {
      if (!((mask >> l) & 1)) continue;
      if (o < capacity) {
        store3(pos, o, q[l]);
        store3(alpha, o, al[l]);
        sigma[o] = sg;
        age[o] = 0.0;
      } else {
        flag_status(kStatusCapacity);
      }
      ++o;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = s_base < capacity ? s_base : capacity;
}

unsigned nblk(int64_t n, int t = kT) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace
}  // namespace fvx


// A layout is usable when its sizes are positive, the motion table is given
// and, without a strip map, the grid is one surface (w = ns + 1).
static bool layout_ok(const FvxSurfaces* s) {
  return s && s->ns >= 1 && s->w >= 2 && s->motion && (s->col || s->w == s->ns + 1);
}

extern "C" {

int fvx_uvlm_kinematics(int nc, const FvxSurfaces* s, const double* base, double t, double* out,
                        void* stream) {
  FVX_ARG_CHECK(nc >= 1 && layout_ok(s) && base && out, "bad kinematics arguments");
  const int64_t nv = static_cast<int64_t>(nc + 1) * s->w;
  fvx::kinematics_kernel<<<fvx::nblk(nv), fvx::kT, 0, static_cast<cudaStream_t>(stream)>>>(
      nv, base, *s, t, out);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_lattice(const double* verts, int nc, const FvxSurfaces* s, double* br, double* fr,
                     double* fl, double* bl, double* colloc, double* normal, double* area,
                     double* leg_center, double* leg_vec, double* te_back, void* stream) {
  FVX_ARG_CHECK(nc >= 2 && layout_ok(s) && verts, "lattice needs nc >= 2 and a layout");
  fvx::LatticeOut o{br, fr, fl, bl, colloc, normal, area, leg_center, leg_vec, te_back};
  const int n = nc * s->ns > s->w ? nc * s->ns : s->w;
  fvx::lattice_kernel<<<fvx::nblk(n), fvx::kT, 0, static_cast<cudaStream_t>(stream)>>>(verts, nc,
                                                                                      *s, o);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_aic(int n_systems, int P, const double* colloc, const double* normal,
                 const double* br, const double* fr, const double* fl, const double* bl,
                 double rc0, double nu, double* aic, void* stream) {
  FVX_ARG_CHECK(n_systems >= 1 && P >= 1 && n_systems <= 65535, "bad AIC sizes");
  const int64_t PP = static_cast<int64_t>(P) * P;
  dim3 grid(fvx::nblk(PP), n_systems);
  fvx::aic_kernel<<<grid, fvx::kT, 0, static_cast<cudaStream_t>(stream)>>>(
      P, colloc, normal, br, fr, fl, bl, rc0, nu, aic);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_rhs(int nc, const FvxSurfaces* s, const double* colloc, const double* normal,
                 const double* v1, const double* v2, const double* u_inf, double t, double* rhs,
                 void* stream) {
  FVX_ARG_CHECK(nc >= 1 && layout_ok(s) && colloc && normal && u_inf && rhs,
                "bad rhs arguments");
  const int P = nc * s->ns;
  fvx::rhs_kernel<<<fvx::nblk(P), fvx::kT, 0, static_cast<cudaStream_t>(stream)>>>(
      P, *s, colloc, normal, v1, v2, u_inf[0], u_inf[1], u_inf[2], t, rhs);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_lu_solve_batched(int n_systems, int P, double* A, double* b, void* stream) {
  FVX_ARG_CHECK(n_systems >= 1 && P >= 1 && P <= fvx::kLuMaxP && A && b,
                "bad solve arguments (P must be 1..%d)", fvx::kLuMaxP);
  if (P <= fvx::kLuClusterMaxP) {
    const int ncmax = (P + fvx::kLuCtas - 1) / fvx::kLuCtas;
    const size_t smem =
        8 * (static_cast<size_t>(ncmax) * P + 3 * static_cast<size_t>(P) + P * (P + 1) / 2);
    FVX_CUDA_TRY(cudaFuncSetAttribute(fvx::lu_cluster_kernel<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
    fvx::lu_cluster_kernel<false><<<n_systems * fvx::kLuCtas, fvx::kLuClusterThreads, smem,
                                    static_cast<cudaStream_t>(stream)>>>(P, A, b, nullptr);
    FVX_LAUNCH_CHECK();
    return FVX_OK;
  }
  // tail size T: the largest block (row stride T + 1) that fits next to the
  // three P-vectors in the opt-in shared memory
  const int budget = fvx::device_smem_optin() - 1024;  // static arrays of the kernel
  int T = 0;
  while (T < P && 8L * (3L * P + static_cast<long>(T + 1) * (T + 2)) <= budget) ++T;
  const size_t smem = 8 * (3 * static_cast<size_t>(P) + static_cast<size_t>(T) * (T + 1));
  FVX_CUDA_TRY(cudaFuncSetAttribute(fvx::lu_solve_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
  fvx::lu_solve_kernel<<<n_systems, fvx::kLuThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      P, T, A, b);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int64_t fvx_lu_workspace_bytes(int P) {
  return P >= 1 && P <= fvx::kLuClusterMaxP ? 8 * fvx::lu_workspace_doubles(P) : 0;
}

int fvx_lu_factor_batched(int n_systems, int P, double* A, double* work, void* stream) {
  FVX_ARG_CHECK(n_systems >= 1 && P >= 1 && P <= fvx::kLuClusterMaxP && A && work,
                "bad factor arguments (P must be 1..%d)", fvx::kLuClusterMaxP);
  const int ncmax = (P + fvx::kLuCtas - 1) / fvx::kLuCtas;
  const size_t smem =
      8 * (static_cast<size_t>(ncmax) * P + 3 * static_cast<size_t>(P) + P * (P + 1) / 2);
  FVX_CUDA_TRY(cudaFuncSetAttribute(fvx::lu_cluster_kernel<true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
  fvx::lu_cluster_kernel<true><<<n_systems * fvx::kLuCtas, fvx::kLuClusterThreads, smem,
                                 static_cast<cudaStream_t>(stream)>>>(P, A, nullptr, work);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_lu_solve_factored_batched(int n_systems, int P, const double* work, double* b,
                                  void* stream) {
  FVX_ARG_CHECK(n_systems >= 1 && P >= 1 && P <= fvx::kLuClusterMaxP && work && b,
                "bad solve arguments (P must be 1..%d)", fvx::kLuClusterMaxP);
  const size_t smem = 8 * (2 * static_cast<size_t>(P) + static_cast<size_t>(P) * (P + 1) / 2);
  FVX_CUDA_TRY(cudaFuncSetAttribute(fvx::lu_solve_factored_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
  fvx::lu_solve_factored_kernel<<<n_systems, fvx::kLuClusterThreads, smem,
                                  static_cast<cudaStream_t>(stream)>>>(P, work, b);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_loads(int nc, const FvxSurfaces* s, const double* gamma, const double* gamma_prev,
                   const double* leg_center, const double* leg_vec, const double* area,
                   const double* normal, const double* v1, const double* v2, const double* v3,
                   const double* u_inf, double rho, double dt, double t, double s_ref,
                   double* cl, double* cdi, double* force, void* stream) {
  FVX_ARG_CHECK(nc >= 1 && layout_ok(s) && gamma && u_inf && cl && cdi, "bad loads arguments");
  fvx::LoadsArgs a{nc,       *s,       gamma,    gamma_prev, leg_center, leg_vec, area,
                   normal,   v1,       v2,       v3,         u_inf[0],   u_inf[1], u_inf[2],
                   rho,      dt,       t,        s_ref,      cl,         cdi,     force};
  fvx::loads_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_loads_bernoulli(int nc, const FvxSurfaces* s, const double* verts,
                             const double* gamma, const double* gamma_prev, const double* colloc,
                             const double* area, const double* normal, const double* v1,
                             const double* v2, const double* u_inf, double rho, double dt,
                             double t, double s_ref, double* cl, double* cdi, double* force,
                             void* stream) {
  FVX_ARG_CHECK(nc >= 1 && layout_ok(s) && verts && gamma && colloc && area && normal && u_inf &&
                    cl && cdi,
                "bad loads arguments");
  fvx::BernoulliArgs a{nc,    *s,     verts,    gamma,    gamma_prev, colloc, area,
                       normal, v1,    v2,       u_inf[0], u_inf[1],   u_inf[2], rho,
                       dt,     t,     s_ref,    cl,       cdi,        force};
  fvx::bernoulli_loads_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_wake_rings(int R, const FvxSurfaces* s, const double* W, const double* gam,
                        const double* age, double rc0, double* br, double* fr, double* fl,
                        double* bl, double* strength, double* rc0s, double* ages, void* stream) {
  FVX_ARG_CHECK(R >= 0 && layout_ok(s), "bad wake sizes");
  if (R == 0) return FVX_OK;
  fvx::wake_rings_kernel<<<fvx::nblk(R * s->ns), fvx::kT, 0,
                           static_cast<cudaStream_t>(stream)>>>(R, *s, W, gam, age, rc0, br, fr,
                                                                fl, bl, strength, rc0s, ages);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_shed(int R_old, int nc, const FvxSurfaces* s, const double* W_old,
                  const double* gam_old, const double* age_old, const double* te_next,
                  const double* gamma, const double* u_inf, double dt, const double* v1,
                  const double* v2, const double* v3, double* W_new, double* gam_new,
                  double* age_new, void* stream) {
  FVX_ARG_CHECK(R_old >= 0 && nc >= 1 && layout_ok(s) && u_inf, "bad shed arguments");
  const int n = (R_old + 2) * s->w;
  fvx::shed_kernel<<<fvx::nblk(n), fvx::kT, 0, static_cast<cudaStream_t>(stream)>>>(
      R_old, nc, s->ns, s->w, W_old, gam_old, age_old, te_next, gamma, u_inf[0], u_inf[1],
      u_inf[2], dt, v1, v2, v3, W_new, gam_new, age_new);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_uvlm_convert(int R, int n_keep, const FvxSurfaces* s, const double* W,
                     const double* gam, int sigma_rule, double sigma_vdt, int64_t capacity,
                     int64_t* count, double* pos, double* alpha, double* sigma, double* age,
                     void* stream) {
  FVX_ARG_CHECK(R >= 0 && n_keep >= 0 && layout_ok(s) && count, "bad convert arguments");
  if (R <= n_keep) return FVX_OK;
  fvx::convert_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      R, n_keep, *s, W, gam, sigma_rule, sigma_vdt, capacity, count, pos, alpha, sigma, age);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

}  // extern "C"
