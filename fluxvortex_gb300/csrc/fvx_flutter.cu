// fvx_flutter.cu -- batched aeroelastic flutter sweep: one persistent CTA per
// environment (airspeed) runs the coupled UVLM + beam time history.
//
// Per step, all in the CTA (FP64 unless noted):
//   deform the base vertex grid by the beam's heave/twist (linear span
//   interpolation, rotation about the elastic axis) and take the vertex
//   velocities from the beam velocities; build the ring lattice (quarter-
//   chord rings, 3/4-chord collocation points, normals, areas, bound legs);
//   AIC[i][j] = (unit ring j at collocation i) . n_i; wake ring rows and the
//   particle wake induced at the 2P points (collocation + bound-leg centres),
//   in FP64 or -- mixed precision -- in FP32 on FP64 offsets with compensated
//   particle sums (particles staged through shared memory, split over thread
//   slices, slices reduced in fixed order); the
//   right-hand side; an in-place LU solve with partial pivoting (first
//   largest pivot, as LAPACK's getrf); Kutta-Joukowski forces on the bound
//   legs with the full induced velocity and the unsteady term; station lift
//   and torque about the elastic axis distributed to the beam nodes; the
//   Newmark average-acceleration step with the precomputed inverse of the
//   effective stiffness; the tip history; the wake update (convect with the
//   freestream, shed the trailing-edge row at the new geometry, convert the
//   row past n_keep into 4 particles per ring, FIFO-capped particle store).
// Reference: src/fluxvortex/aeroelastic_solver.py:68-221 and beam_fe.py:231-351
// around PteraSoftware's ring-vortex UVLM; the PteraSoftware-free model is
// described in fluxvortex_gb300/flutter.py.
#include <cooperative_groups.h>

#include "fvx_common.cuh"
#include "fvx_pair_math.cuh"
#include "fvx_segment_math.cuh"

namespace fvx {
namespace flutter {

constexpr int kMaxP = 64;       // panels per environment
constexpr int kMaxNV = 128;     // vertices
constexpr int kMaxRows = 16;    // n_keep + 1 wake ring rows
constexpr int kMaxNS = 16;      // spanwise panels
constexpr int kMaxDof = 48;     // beam DOF (all nodes)
constexpr int kTile = 128;      // particles staged per tile
constexpr double kC = -0.07957747154594767;  // -1/(4 pi): particle strength scaling

struct Smem {
  double verts[kMaxNV][3], vvel[kMaxNV][3];
  double colloc[kMaxP][3], normal[kMaxP][3], legc[kMaxP][3], legv[kMaxP][3];
  double vcol[kMaxP][3], vleg[kMaxP][3], area[kMaxP];
  seg::VortexRec bound[kMaxP];
  seg::VortexRec wake[kMaxRows * kMaxNS];
  double A[kMaxP][kMaxP + 1];
  double rhs[kMaxP], gam[kMaxP], gprev[kMaxP];
  double Vind[2 * kMaxP][3];
  double Vsum[2 * kMaxP][3];  // cluster form: both CTAs' partial inductions summed
  double W[kMaxRows + 1][kMaxNS + 1][3];
  double wgam[kMaxRows][kMaxNS], wage[kMaxRows];
  double d[kMaxDof], v[kMaxDof], a[kMaxDof], F[kMaxDof], feff[kMaxDof], gd[kMaxDof];
  double tile[kTile][8];  // staged particles: x y z | a' (C-scaled) | sigma^2, 2.5 sigma^2
  double red[8];
  int piv;
};

__device__ __forceinline__ void vadd(double* o, double x, double y, double z) {
  o[0] += x;
  o[1] += y;
  o[2] += z;
}

// Deformed vertices and their velocities from the beam state in S.d / S.v.
__device__ void deform(Smem& S, const FlutterParams& p) {
  const int nv = (p.nc + 1) * (p.ns + 1);
  for (int k = threadIdx.x; k < nv; k += blockDim.x) {
    const int n = p.vert_node[k];
    const double xi = p.vert_xi[k];
    const double w = S.d[3 * n] * (1.0 - xi) + S.d[3 * (n + 1)] * xi;
    const double th = S.d[3 * n + 2] * (1.0 - xi) + S.d[3 * (n + 1) + 2] * xi;
    const double wd = S.v[3 * n] * (1.0 - xi) + S.v[3 * (n + 1)] * xi;
    const double thd = S.v[3 * n + 2] * (1.0 - xi) + S.v[3 * (n + 1) + 2] * xi;
    const double* b = p.base_verts + 3 * k;
    const double xr = b[0] - p.x_ea;
    const double s = sin(th), c = cos(th);
    S.verts[k][0] = p.x_ea + xr * c;
    S.verts[k][1] = b[1];
    S.verts[k][2] = b[2] + w - xr * s;
    S.vvel[k][0] = -xr * s * thd;
    S.vvel[k][1] = 0.0;
    S.vvel[k][2] = wd - xr * c * thd;
  }
}

// quarter-chord point of vertex column j at chordwise station i (0..nc)
__device__ __forceinline__ void quarter(const double (*V)[3], int nc, int ns, int i, int j,
                                        double* q) {
  const int s1 = ns + 1;
  const double* a = V[i * s1 + j];
  if (i < nc) {
    const double* b = V[(i + 1) * s1 + j];
    for (int c = 0; c < 3; ++c) q[c] = a[c] + 0.25 * (b[c] - a[c]);
  } else {
    const double* b = V[(i - 1) * s1 + j];
    for (int c = 0; c < 3; ++c) q[c] = a[c] + 0.25 * (a[c] - b[c]);
  }
}

__device__ void build_lattice(Smem& S, const FlutterParams& p) {
  const int P = p.nc * p.ns, s1 = p.ns + 1;
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const int i = k / p.ns, j = k % p.ns;
    double fl[3], fr[3], br[3], bl[3], vfl[3], vfr[3];
    quarter(S.verts, p.nc, p.ns, i, j, fl);
    quarter(S.verts, p.nc, p.ns, i, j + 1, fr);
    quarter(S.verts, p.nc, p.ns, i + 1, j + 1, br);
    quarter(S.verts, p.nc, p.ns, i + 1, j, bl);
    quarter(S.vvel, p.nc, p.ns, i, j, vfl);
    quarter(S.vvel, p.nc, p.ns, i, j + 1, vfr);
    const double* v00 = S.verts[i * s1 + j];
    const double* v01 = S.verts[i * s1 + j + 1];
    const double* v10 = S.verts[(i + 1) * s1 + j];
    const double* v11 = S.verts[(i + 1) * s1 + j + 1];
    const double* u00 = S.vvel[i * s1 + j];
    const double* u01 = S.vvel[i * s1 + j + 1];
    const double* u10 = S.vvel[(i + 1) * s1 + j];
    const double* u11 = S.vvel[(i + 1) * s1 + j + 1];
    double d1[3], d2[3];
    for (int c = 0; c < 3; ++c) {
      const double c0 = v00[c] + 0.75 * (v10[c] - v00[c]);
      const double c1 = v01[c] + 0.75 * (v11[c] - v01[c]);
      S.colloc[k][c] = 0.5 * (c0 + c1);
      const double e0 = u00[c] + 0.75 * (u10[c] - u00[c]);
      const double e1 = u01[c] + 0.75 * (u11[c] - u01[c]);
      S.vcol[k][c] = 0.5 * (e0 + e1);
      S.legc[k][c] = 0.5 * (fr[c] + fl[c]);
      S.legv[k][c] = fl[c] - fr[c];
      S.vleg[k][c] = 0.5 * (vfr[c] + vfl[c]);
      d1[c] = v11[c] - v00[c];
      d2[c] = v01[c] - v10[c];
    }
    const double cx = d1[1] * d2[2] - d1[2] * d2[1];
    const double cy = d1[2] * d2[0] - d1[0] * d2[2];
    const double cz = d1[0] * d2[1] - d1[1] * d2[0];
    const double nrm = sqrt(cx * cx + cy * cy + cz * cz);
    S.normal[k][0] = cx / nrm;
    S.normal[k][1] = cy / nrm;
    S.normal[k][2] = cz / nrm;
    S.area[k] = 0.5 * nrm;
    seg::prep_vortex<FVX_LEGS_RING>(S.bound[k], br, fr, fl, bl, 1.0, p.rc0, 0.0, p.nu);
  }
}

// The reference's panel deformation (coupling 1; aeroelastic_solver.py:150-221):
// panel k of strip j moves with the heave w and twist th (nose-up) of the
// displacements S.gd interpolated at the strip's collocation span station; its
// corners and ring vertices by dz = w - (x - x_ea) sin th, dx = (x - x_ea)
// (cos th - 1), its collocation point by dz only.  Normal and area from the
// moved corners; no motion velocity.
__device__ __forceinline__ void ref_motion(const FlutterParams& p, const Smem& S, int j,
                                           double& w, double& s, double& c1) {
  const int n = p.station_node[j];
  const double xi = p.station_xi[j];
  w = S.gd[3 * n] * (1.0 - xi) + S.gd[3 * (n + 1)] * xi;
  const double th = S.gd[3 * n + 2] * (1.0 - xi) + S.gd[3 * (n + 1) + 2] * xi;
  s = sin(th);
  c1 = cos(th) - 1.0;
}
__device__ __forceinline__ void ref_move(const FlutterParams& p, double w, double s, double c1,
                                         double* q) {
  const double xr = q[0] - p.x_ea;
  q[0] += xr * c1;
  q[2] += w - xr * s;
}
__device__ void build_lattice_reference(Smem& S, const FlutterParams& p) {
  const int P = p.nc * p.ns, s1 = p.ns + 1;
  const double(*B)[3] = reinterpret_cast<const double(*)[3]>(p.base_verts);
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const int i = k / p.ns, j = k % p.ns;
    double w, sn, c1;
    ref_motion(p, S, j, w, sn, c1);
    double fl[3], fr[3], br[3], bl[3], v00[3], v01[3], v10[3], v11[3];
    quarter(B, p.nc, p.ns, i, j, fl);
    quarter(B, p.nc, p.ns, i, j + 1, fr);
    quarter(B, p.nc, p.ns, i + 1, j + 1, br);
    quarter(B, p.nc, p.ns, i + 1, j, bl);
    for (int c = 0; c < 3; ++c) {
      v00[c] = B[i * s1 + j][c];
      v01[c] = B[i * s1 + j + 1][c];
      v10[c] = B[(i + 1) * s1 + j][c];
      v11[c] = B[(i + 1) * s1 + j + 1][c];
      const double c0 = v00[c] + 0.75 * (v10[c] - v00[c]);
      const double c1b = v01[c] + 0.75 * (v11[c] - v01[c]);
      S.colloc[k][c] = 0.5 * (c0 + c1b);
    }
    S.colloc[k][2] += w - (S.colloc[k][0] - p.x_ea) * sn;
    ref_move(p, w, sn, c1, fl);
    ref_move(p, w, sn, c1, fr);
    ref_move(p, w, sn, c1, br);
    ref_move(p, w, sn, c1, bl);
    ref_move(p, w, sn, c1, v00);
    ref_move(p, w, sn, c1, v01);
    ref_move(p, w, sn, c1, v10);
    ref_move(p, w, sn, c1, v11);
    double d1[3], d2[3];
    for (int c = 0; c < 3; ++c) {
      S.vcol[k][c] = 0.0;
      S.vleg[k][c] = 0.0;
      S.legc[k][c] = 0.5 * (fr[c] + fl[c]);
      S.legv[k][c] = fl[c] - fr[c];
      d1[c] = v11[c] - v00[c];
      d2[c] = v01[c] - v10[c];
    }
    const double cx = d1[1] * d2[2] - d1[2] * d2[1];
    const double cy = d1[2] * d2[0] - d1[0] * d2[2];
    const double cz = d1[0] * d2[1] - d1[1] * d2[0];
    const double nrm = sqrt(cx * cx + cy * cy + cz * cz);
    S.normal[k][0] = cx / nrm;
    S.normal[k][1] = cy / nrm;
    S.normal[k][2] = cz / nrm;
    S.area[k] = 0.5 * nrm;
    seg::prep_vortex<FVX_LEGS_RING>(S.bound[k], br, fr, fl, bl, 1.0, p.rc0, 0.0, p.nu);
  }
}

// The reference's trailing edge for the wake's new row (coupling 1): the back
// vertices of the last chordwise rings, strip k's back-left one and the last
// strip's back-right one, each moved with its strip's deformation.
__device__ void trailing_edge_reference(const Smem& S, const FlutterParams& p, double* out,
                                        int k) {
  const double(*B)[3] = reinterpret_cast<const double(*)[3]>(p.base_verts);
  const int j = k < p.ns ? k : p.ns - 1;
  double w, sn, c1;
  ref_motion(p, S, j, w, sn, c1);
  quarter(B, p.nc, p.ns, p.nc, k, out);
  ref_move(p, w, sn, c1, out);
}

// One wake ring at point p in FP32 on offsets taken in FP64 (the ring-vortex
// formula and skip tests of seg::vortex_velocity, ring leg set).
__device__ __forceinline__ void ring_velocity_f32(const seg::VortexRec& R, double px, double py,
                                                  double pz, float& vx, float& vy, float& vz) {
  float dx[4], dy[4], dz[4], len[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    dx[c] = static_cast<float>(R.c[c][0] - px);
    dy[c] = static_cast<float>(R.c[c][1] - py);
    dz[c] = static_cast<float>(R.c[c][2] - pz);
    len[c] = sqrtf(dx[c] * dx[c] + dy[c] * dy[c] + dz[c] * dz[c]);
  }
  const float c1 = static_cast<float>(R.c1);
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const int a = l, b = (l + 1) & 3;
    if (!((R.valid >> l) & 1)) continue;
    const float tol = static_cast<float>(R.tol[l]);
    if (len[a] < tol || len[b] < tol) continue;
    const float r3x = dy[a] * dz[b] - dz[a] * dy[b];
    const float r3y = dz[a] * dx[b] - dx[a] * dz[b];
    const float r3z = dx[a] * dy[b] - dy[a] * dx[b];
    const float r3_sq = r3x * r3x + r3y * r3y + r3z * r3z;
    const float r1r2 = len[a] * len[b];
    const float thr = 1.0e-10f * r1r2;
    if (r3_sq < 2.f * thr * thr && sqrtf(r3_sq) < thr) continue;
    const float c3 = dx[a] * dx[b] + dy[a] * dy[b] + dz[a] * dz[b];
    const float c4 = c1 * (len[a] + len[b]) * (r1r2 - c3) /
                     (r1r2 * (r3_sq + static_cast<float>(R.c2[l])));
    vx += c4 * r3x;
    vy += c4 * r3y;
    vz += c4 * r3z;
  }
}

// Induced velocity of the wake rings and particles at the 2P points
// (collocation points, then bound-leg centres) into S.Vind.
// CL > 1: the environment runs on a cluster of CL CTAs; CTA `crank` takes
// every CL-th ring (by slice) and every CL-th particle tile, and the partial
// inductions are summed in rank order through distributed shared memory, so
// both CTAs hold the same total.
template <bool F32, int CL>
__device__ void wake_induction(Smem& S, const FlutterParams& p, const FlutterState& st, int env,
                               int R, int head, int count, int crank) {
  const int P = p.nc * p.ns, T2 = 2 * P;
  const int slices = blockDim.x / T2;
  const int tgt = threadIdx.x % T2, sl = threadIdx.x / T2;
  const bool active = sl < slices;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (active) {
    const double* q = tgt < P ? S.colloc[tgt] : S.legc[tgt - P];
    px = q[0];
    py = q[1];
    pz = q[2];
  }
  // wake rings: slice sl takes rings sl, sl + slices, ...
  double vx = 0.0, vy = 0.0, vz = 0.0;
  int cnt[4] = {0, 0, 0, 0};
  if (active) {
    if constexpr (F32) {
      float fx = 0.f, fy = 0.f, fz = 0.f;
      for (int r = sl + crank * slices; r < R * p.ns; r += slices * CL)
        ring_velocity_f32(S.wake[r], px, py, pz, fx, fy, fz);
      vx = fx;
      vy = fy;
      vz = fz;
    } else {
      for (int r = sl + crank * slices; r < R * p.ns; r += slices * CL)
        seg::vortex_velocity<FVX_LEGS_RING>(S.wake[r], px, py, pz, vx, vy, vz, cnt);
    }
  }
  // particles, staged in tiles, oldest first
  const int Pm = p.max_particles;
  const double* pp = st.ppos + static_cast<int64_t>(env) * Pm * 3;
  const double* pa = st.palp + static_cast<int64_t>(env) * Pm * 3;
  const double* ps = st.psig + static_cast<int64_t>(env) * Pm;
  float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
  for (int t0 = crank * kTile; t0 < count; t0 += kTile * CL) {
    const int nt = min(kTile, count - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt; e += blockDim.x) {
      const int q = (head + t0 + e) % Pm;
      const double s = ps[q];
      S.tile[e][0] = pp[3 * q];
      S.tile[e][1] = pp[3 * q + 1];
      S.tile[e][2] = pp[3 * q + 2];
      S.tile[e][3] = kC * pa[3 * q];
      S.tile[e][4] = kC * pa[3 * q + 1];
      S.tile[e][5] = kC * pa[3 * q + 2];
      S.tile[e][6] = s * s;
      S.tile[e][7] = 2.5 * s * s;
    }
    __syncthreads();
    if (!active) continue;
    for (int e = sl; e < nt; e += slices) {
      const double* s = S.tile[e];
      if constexpr (F32) {
        // FP32 pair arithmetic on the exact FP64 offset, compensated sums
        const float dx = static_cast<float>(px - s[0]), dy = static_cast<float>(py - s[1]),
                    dz = static_cast<float>(pz - s[2]);
        const float r2 = dx * dx + dy * dy + dz * dz;
        float f, fpr;
        pair::core_f32<FVX_KERNEL_WINCKELMANS, false>(r2, static_cast<float>(s[6]),
                                                      static_cast<float>(s[7]), f, fpr);
        const float ax = static_cast<float>(s[3]), ay = static_cast<float>(s[4]),
                    az = static_cast<float>(s[5]);
        const float ex = f * dx, ey = f * dy, ez = f * dz;
        const float ux = ey * az - ez * ay, uy = ez * ax - ex * az, uz = ex * ay - ey * ax;
        float t = hx + ux;
        lx += (hx - t) + ux;
        hx = t;
        t = hy + uy;
        ly += (hy - t) + uy;
        hy = t;
        t = hz + uz;
        lz += (hz - t) + uz;
        hz = t;
      } else {
        const double dx = px - s[0], dy = py - s[1], dz = pz - s[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        double f, fpr;
        pair::core_f64<FVX_KERNEL_WINCKELMANS, false>(r2, s[6], s[7], f, fpr);
        const double ex = f * dx, ey = f * dy, ez = f * dz;
        vx += ey * s[5] - ez * s[4];
        vy += ez * s[3] - ex * s[5];
        vz += ex * s[4] - ey * s[3];
      }
    }
  }
  if constexpr (F32) {
    vx += static_cast<double>(hx) + static_cast<double>(lx);
    vy += static_cast<double>(hy) + static_cast<double>(ly);
    vz += static_cast<double>(hz) + static_cast<double>(lz);
  }
  // slice partials -> fixed-order sum: reuse A's storage as scratch
  __syncthreads();
  double* part = &S.A[0][0];  // needs slices * 2P * 3 <= kMaxP * (kMaxP + 1)
  if (active) {
    part[(sl * T2 + tgt) * 3 + 0] = vx;
    part[(sl * T2 + tgt) * 3 + 1] = vy;
    part[(sl * T2 + tgt) * 3 + 2] = vz;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < T2; k += blockDim.x) {
    double x = 0.0, y = 0.0, z = 0.0;
    for (int s2 = 0; s2 < slices; ++s2) {
      x += part[(s2 * T2 + k) * 3 + 0];
      y += part[(s2 * T2 + k) * 3 + 1];
      z += part[(s2 * T2 + k) * 3 + 2];
    }
    S.Vind[k][0] = x;
    S.Vind[k][1] = y;
    S.Vind[k][2] = z;
  }
  __syncthreads();
  if constexpr (CL > 1) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();  // every CTA's partial is complete
    for (int k = threadIdx.x; k < T2; k += blockDim.x) {
      double x = 0.0, y = 0.0, z = 0.0;
      for (int r = 0; r < CL; ++r) {
        const double(*V)[3] = r == crank ? S.Vind : cl.map_shared_rank(S.Vind, r);
        x += V[k][0];
        y += V[k][1];
        z += V[k][2];
      }
      S.Vsum[k][0] = x;
      S.Vsum[k][1] = y;
      S.Vsum[k][2] = z;
    }
    cl.sync();  // every CTA has read the others' partials
    for (int k = threadIdx.x; k < T2; k += blockDim.x)
      for (int c = 0; c < 3; ++c) S.Vind[k][c] = S.Vsum[k][c];
    __syncthreads();
  }
}

// In-place LU solve of S.A x = S.rhs (partial pivoting, first largest |pivot|).
__device__ bool lu_solve(Smem& S, int P) {
  bool ok = true;
  for (int k = 0; k < P; ++k) {
    if (threadIdx.x == 0) {
      int piv = k;
      double best = fabs(S.A[k][k]);
      for (int i = k + 1; i < P; ++i) {
        const double v = fabs(S.A[i][k]);
        if (v > best) {
          best = v;
          piv = i;
        }
      }
      S.piv = best > 0.0 ? piv : -1;
    }
    __syncthreads();
    const int piv = S.piv;
    if (piv < 0) {
      ok = false;
      break;
    }
    if (piv != k) {
      for (int j = threadIdx.x; j < P; j += blockDim.x) {
        const double t = S.A[k][j];
        S.A[k][j] = S.A[piv][j];
        S.A[piv][j] = t;
      }
      if (threadIdx.x == 0) {
        const double t = S.rhs[k];
        S.rhs[k] = S.rhs[piv];
        S.rhs[piv] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / S.A[k][k];
    const int rows = P - k - 1;
    for (int e = threadIdx.x; e < rows * (P - k); e += blockDim.x) {
      const int i = k + 1 + e / (P - k), j = k + e % (P - k);
      const double l = S.A[i][k] * inv;
      if (j > k) S.A[i][j] -= l * S.A[k][j];
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < P; i += blockDim.x) {
      const double l = S.A[i][k] * inv;
      S.rhs[i] -= l * S.rhs[k];
      S.A[i][k] = l;
    }
    __syncthreads();
  }
  if (!ok) return false;
  if (threadIdx.x == 0) {
    for (int i = P - 1; i >= 0; --i) {
      double s = S.rhs[i];
      for (int j = i + 1; j < P; ++j) s -= S.A[i][j] * S.gam[j];
      S.gam[i] = s / S.A[i][i];
    }
  }
  __syncthreads();
  return true;
}

// CL CTAs per environment (a cluster, launched with that cluster size): they
// run the same step redundantly, except the wake induction, which they share
// (wake_induction); rank 0 alone writes the environment's global state, and a
// cluster barrier at the start of every step makes its particle writes of
// the last step visible to the others.
template <bool F32, int CL>
__global__ void __launch_bounds__(512) sweep_kernel(FlutterParams p, FlutterState st, int step_end) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  int crank = 0;
  if constexpr (CL > 1) crank = static_cast<int>(cooperative_groups::this_cluster().block_rank());
  const bool writer = crank == 0;
  const int env = blockIdx.x / CL;
  const int P = p.nc * p.ns, s1 = p.ns + 1, ndof = 3 * p.nnodes, nf = ndof - 3;
  const int last = min(step_end, p.n_steps[env]);
  int step = st.step[env];
  if (step >= last) return;
  const double ux = p.u_inf[3 * env], uy = p.u_inf[3 * env + 1], uz = p.u_inf[3 * env + 2];
  const double dt = p.dt;
  // load state
  const bool ref = p.coupling == 1;
  for (int k = threadIdx.x; k < ndof; k += blockDim.x) {
    S.d[k] = st.d[env * ndof + k];
    S.v[k] = st.v[env * ndof + k];
    S.a[k] = st.a[env * ndof + k];
    S.gd[k] = ref ? st.gd[env * ndof + k] : 0.0;
  }
  int R = st.nrows[env];
  for (int k = threadIdx.x; k < (R + 1) * s1 * 3; k += blockDim.x)
    (&S.W[0][0][0])[(k / (s1 * 3)) * (kMaxNS + 1) * 3 + k % (s1 * 3)] =
        st.W[(static_cast<int64_t>(env) * (p.n_keep + 2)) * s1 * 3 + k];
  for (int k = threadIdx.x; k < R * p.ns; k += blockDim.x)
    S.wgam[k / p.ns][k % p.ns] = st.wgam[env * (p.n_keep + 1) * p.ns + k];
  for (int k = threadIdx.x; k < R; k += blockDim.x) S.wage[k] = st.wage[env * (p.n_keep + 1) + k];
  for (int k = threadIdx.x; k < P; k += blockDim.x) S.gprev[k] = st.gprev[env * P + k];
  int has_prev = st.has_prev[env];
  int head = st.phead[env], count = st.pcount[env];
  __syncthreads();
  bool ok = true;
  for (; step < last && ok; ++step) {
    if constexpr (CL > 1) {
      __threadfence();
      cooperative_groups::this_cluster().sync();  // rank 0's particle writes visible
    }
    // 1. geometry and lattice
    if (ref) {
      build_lattice_reference(S, p);
    } else {
      deform(S, p);
      __syncthreads();
      build_lattice(S, p);
    }
    for (int k = threadIdx.x; k < R * p.ns; k += blockDim.x) {
      const int r = k / p.ns, j = k % p.ns;
      seg::prep_vortex<FVX_LEGS_RING>(S.wake[k], S.W[r + 1][j + 1], S.W[r][j + 1], S.W[r][j],
                                      S.W[r + 1][j], S.wgam[r][j], p.rc0, S.wage[r], p.nu);
    }
    __syncthreads();
    // 2. wake + particles at collocation points and bound-leg centres
    wake_induction<F32, CL>(S, p, st, env, R, head, count, crank);
    // 3. AIC (written after the induction, whose scratch overlaps it) and rhs
    for (int e = threadIdx.x; e < P * P; e += blockDim.x) {
      const int i = e / P, j = e % P;
      double vx = 0.0, vy = 0.0, vz = 0.0;
      int cnt[4] = {0, 0, 0, 0};
      seg::vortex_velocity<FVX_LEGS_RING>(S.bound[j], S.colloc[i][0], S.colloc[i][1],
                                          S.colloc[i][2], vx, vy, vz, cnt);
      S.A[i][j] = vx * S.normal[i][0] + vy * S.normal[i][1] + vz * S.normal[i][2];
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const double wx = (ux - S.vcol[i][0]) + S.Vind[i][0];
      const double wy = (uy - S.vcol[i][1]) + S.Vind[i][1];
      const double wz = (uz - S.vcol[i][2]) + S.Vind[i][2];
      S.rhs[i] = -(wx * S.normal[i][0] + wy * S.normal[i][1] + wz * S.normal[i][2]);
    }
    __syncthreads();
    // 4. strengths
    if (!lu_solve(S, P)) {
      ok = false;
      break;
    }
    // 5. loads: bound rings with strengths gamma at the bound-leg centres
    for (int k = threadIdx.x; k < P; k += blockDim.x) S.bound[k].c1 = S.gam[k] * seg::kInv4Pi;
    __syncthreads();
    double* Fz = &S.A[0][0];     // P station-force z components (A is free now)
    double* arm = Fz + kMaxP;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
      double vx = 0.0, vy = 0.0, vz = 0.0;
      int cnt[4] = {0, 0, 0, 0};
      for (int j = 0; j < P; ++j)
        seg::vortex_velocity<FVX_LEGS_RING>(S.bound[j], S.legc[k][0], S.legc[k][1], S.legc[k][2],
                                            vx, vy, vz, cnt);
      const double Vx = (ux - S.vleg[k][0]) + (S.Vind[P + k][0] + vx);
      const double Vy = (uy - S.vleg[k][1]) + (S.Vind[P + k][1] + vy);
      const double Vz = (uz - S.vleg[k][2]) + (S.Vind[P + k][2] + vz);
      const int i = k / p.ns;
      const double geff = i > 0 ? S.gam[k] - S.gam[k - p.ns] : S.gam[k];
      const double dg = has_prev ? (S.gam[k] - S.gprev[k]) / dt : 0.0;
      const double* l = S.legv[k];
      const double cz = Vx * l[1] - Vy * l[0];
      const double fz = p.rho * geff * cz - p.rho * dg * S.area[k] * S.normal[k][2];
      // physical: torque about the elastic axis with the bound leg's arm;
      // reference: the lift's moment about x = 0 with the collocation
      // point's arm (nose-up: -x_c F_z)
      Fz[k] = fz;
      arm[k] = ref ? -S.colloc[k][0] : p.x_ea - S.legc[k][0];
    }
    __syncthreads();
    // the reference couples from step 1 to the step before the last
    const bool couple = !ref || (step >= 1 && step < p.n_steps[env] - 1);
    // 6. station loads -> nodal forces (one thread, fixed order)
    if (couple && threadIdx.x == 0) {
      for (int k = 0; k < ndof; ++k) S.F[k] = 0.0;
      for (int j = 0; j < p.ns; ++j) {
        double lift = 0.0, torque = 0.0;
        for (int i = 0; i < p.nc; ++i) lift += Fz[i * p.ns + j];
        for (int i = 0; i < p.nc; ++i) torque += Fz[i * p.ns + j] * arm[i * p.ns + j];
        const int n = p.station_node[j];
        const double xi = p.station_xi[j];
        S.F[3 * n] += lift * (1.0 - xi);
        S.F[3 * (n + 1)] += lift * xi;
        S.F[3 * n + 2] += torque * (1.0 - xi);
        S.F[3 * (n + 1) + 2] += torque * xi;
      }
    }
    __syncthreads();
    // 7. Newmark: F_eff = F + M (a0 d + a1 v + a2 a) + C (a3 d + a4 v + a5 a)
    const double b = p.beta, g = p.gamma;
    const double a0 = 1.0 / (b * dt * dt), a1 = 1.0 / (b * dt), a2 = 1.0 / (2.0 * b) - 1.0;
    const double a3 = g / (b * dt), a4 = g / b - 1.0, a5 = dt * (g / (2.0 * b) - 1.0);
    for (int r = threadIdx.x; r < nf && couple; r += blockDim.x) {
      double fm = 0.0, fc = 0.0;
      for (int c = 0; c < nf; ++c) {
        const double dc = S.d[3 + c], vc = S.v[3 + c], ac = S.a[3 + c];
        fm += p.mr[r * nf + c] * (a0 * dc + a1 * vc + a2 * ac);
        fc += p.cr[r * nf + c] * (a3 * dc + a4 * vc + a5 * ac);
      }
      S.feff[r] = S.F[3 + r] + fm + fc;
    }
    __syncthreads();
    double dn = 0.0, an = 0.0, vn = 0.0;
    for (int r = threadIdx.x; r < nf && couple; r += blockDim.x) {
      for (int c = 0; c < nf; ++c) dn += p.kinv[r * nf + c] * S.feff[c];
      const double d0 = S.d[3 + r], v0 = S.v[3 + r], acc0 = S.a[3 + r];
      an = a0 * (dn - d0) - a1 * v0 - a2 * acc0;
      vn = v0 + dt * ((1.0 - g) * acc0 + g * an);
    }
    __syncthreads();
    if (couple && threadIdx.x < nf) {
      S.d[3 + threadIdx.x] = dn;
      S.v[3 + threadIdx.x] = vn;
      S.a[3 + threadIdx.x] = an;
    }
    __syncthreads();
    if (couple && writer && threadIdx.x == 0) {
      const int h = ref ? step - 1 : step;
      st.hist_w[static_cast<int64_t>(env) * p.max_steps + h] = S.d[ndof - 3];
      st.hist_th[static_cast<int64_t>(env) * p.max_steps + h] = S.d[ndof - 1];
    }
    if (couple && writer && st.hist_nodes != nullptr) {
      const int h = ref ? step - 1 : step;
      double* hn = st.hist_nodes + (static_cast<int64_t>(env) * p.max_steps + h) * p.nnodes * 2;
      for (int n = threadIdx.x; n < p.nnodes; n += blockDim.x) {
        hn[2 * n] = S.d[3 * n];
        hn[2 * n + 1] = S.d[3 * n + 2];
      }
    }
    // the coupling's displacements shape the next step (reference)
    if (ref && couple)
      for (int k = threadIdx.x; k < ndof; k += blockDim.x) S.gd[k] = S.d[k];
    // 8. wake: next geometry's trailing edge, convect rows and particles
    if (!ref) deform(S, p);
    __syncthreads();
    const int Pm = p.max_particles;
    double* pp = st.ppos + static_cast<int64_t>(env) * Pm * 3;
    double* pa = st.palp + static_cast<int64_t>(env) * Pm * 3;
    double* ps = st.psig + static_cast<int64_t>(env) * Pm;
    for (int e = threadIdx.x; e < (writer ? count : 0); e += blockDim.x) {
      const int q = (head + e) % Pm;
      pp[3 * q] += ux * dt;
      pp[3 * q + 1] += uy * dt;
      pp[3 * q + 2] += uz * dt;
    }
    // shift rows down by one (new row 0), from the back so nothing is overwritten early
    for (int r = R; r >= 0; --r) {
      for (int k = threadIdx.x; k < s1; k += blockDim.x) {
        S.W[r + 1][k][0] = S.W[r][k][0] + ux * dt;
        S.W[r + 1][k][1] = S.W[r][k][1] + uy * dt;
        S.W[r + 1][k][2] = S.W[r][k][2] + uz * dt;
      }
      __syncthreads();
    }
    for (int r = R - 1; r >= 0; --r) {
      for (int k = threadIdx.x; k < p.ns; k += blockDim.x) S.wgam[r + 1][k] = S.wgam[r][k];
      if (threadIdx.x == 0) S.wage[r + 1] = S.wage[r] + dt;
      __syncthreads();
    }
    for (int k = threadIdx.x; k < s1; k += blockDim.x) {
      if (ref)
        trailing_edge_reference(S, p, S.W[0][k], k);
      else
        quarter(S.verts, p.nc, p.ns, p.nc, k, S.W[0][k]);
    }
    for (int k = threadIdx.x; k < p.ns; k += blockDim.x) S.wgam[0][k] = S.gam[(p.nc - 1) * p.ns + k];
    if (threadIdx.x == 0) S.wage[0] = 0.0;
    ++R;
    __syncthreads();
    // 9. rows >= n_keep -> particles (one thread appends in the reference order)
    if (R > p.n_keep) {
      if (threadIdx.x == 0) {
        for (int r = p.n_keep; r < R; ++r) {
          for (int j = 0; j < p.ns; ++j) {
            const double gr = S.wgam[r][j];
            if (fabs(gr) < 1e-15) continue;
            const double* fl = S.W[r][j];
            const double* fr = S.W[r][j + 1];
            const double* bl = S.W[r + 1][j];
            const double* br = S.W[r + 1][j + 1];
            auto dist = [](const double* x, const double* y) {
              const double a = x[0] - y[0], b2 = x[1] - y[1], c = x[2] - y[2];
              return sqrt(a * a + b2 * b2 + c * c);
            };
            const double sg =
                1.3 * 0.25 * (dist(fl, fr) + dist(bl, fl) + dist(br, bl) + dist(fr, br));
            const double* ends[4][2] = {{fr, fl}, {fl, bl}, {bl, br}, {br, fr}};
            for (int e = 0; e < 4; ++e) {
              const double* a = ends[e][0];
              const double* bb = ends[e][1];
              const double alx = gr * (bb[0] - a[0]), aly = gr * (bb[1] - a[1]),
                           alz = gr * (bb[2] - a[2]);
              if (!(alx * alx + aly * aly + alz * alz > 1e-30)) continue;
              int q;
              if (count < Pm) {
                q = (head + count) % Pm;
                ++count;
              } else {
                q = head;  // drop the oldest
                head = (head + 1) % Pm;
              }
              if (writer) {
                pp[3 * q] = 0.5 * (a[0] + bb[0]);
                pp[3 * q + 1] = 0.5 * (a[1] + bb[1]);
                pp[3 * q + 2] = 0.5 * (a[2] + bb[2]);
                pa[3 * q] = alx;
                pa[3 * q + 1] = aly;
                pa[3 * q + 2] = alz;
                ps[q] = sg;
              }
            }
          }
        }
        S.red[0] = static_cast<double>(head);
        S.red[1] = static_cast<double>(count);
      }
      R = p.n_keep;
      __syncthreads();
      head = static_cast<int>(S.red[0]);
      count = static_cast<int>(S.red[1]);
    }
    for (int k = threadIdx.x; k < P; k += blockDim.x) S.gprev[k] = S.gam[k];
    has_prev = 1;
    __syncthreads();
  }
  if (!ok) {
    if (threadIdx.x == 0) flag_status(kStatusNonFinite);
  }
  // store state (rank 0)
  if (!writer) return;
  for (int k = threadIdx.x; k < ndof; k += blockDim.x) {
    st.d[env * ndof + k] = S.d[k];
    st.v[env * ndof + k] = S.v[k];
    st.a[env * ndof + k] = S.a[k];
    if (ref) st.gd[env * ndof + k] = S.gd[k];
  }
  for (int k = threadIdx.x; k < (R + 1) * s1 * 3; k += blockDim.x)
    st.W[(static_cast<int64_t>(env) * (p.n_keep + 2)) * s1 * 3 + k] =
        (&S.W[0][0][0])[(k / (s1 * 3)) * (kMaxNS + 1) * 3 + k % (s1 * 3)];
  for (int k = threadIdx.x; k < R * p.ns; k += blockDim.x)
    st.wgam[env * (p.n_keep + 1) * p.ns + k] = S.wgam[k / p.ns][k % p.ns];
  for (int k = threadIdx.x; k < R; k += blockDim.x) st.wage[env * (p.n_keep + 1) + k] = S.wage[k];
  for (int k = threadIdx.x; k < P; k += blockDim.x) st.gprev[env * P + k] = S.gprev[k];
  if (threadIdx.x == 0) {
    st.nrows[env] = R;
    st.has_prev[env] = has_prev;
    st.phead[env] = head;
    st.pcount[env] = count;
    st.step[env] = step;
  }
}

}  // namespace flutter
}  // namespace fvx

extern "C" int fvx_flutter_sweep(const FlutterParams* params, const FlutterState* state,
                                 int step_end, int precision, int threads, void* stream) {
  using namespace fvx::flutter;
  FVX_ARG_CHECK(params && state, "null argument");
  const FlutterParams& p = *params;
  const int P = p.nc * p.ns;
  FVX_ARG_CHECK(p.n_env > 0 && p.nc >= 2 && p.ns >= 1 && P <= kMaxP && p.ns <= kMaxNS &&
                    (p.nc + 1) * (p.ns + 1) <= kMaxNV,
                "lattice %d x %d outside the kernel's limits", p.nc, p.ns);
  FVX_ARG_CHECK(p.n_keep >= 1 && p.n_keep + 1 <= kMaxRows, "n_keep %d out of range", p.n_keep);
  FVX_ARG_CHECK(3 * p.nnodes <= kMaxDof && p.nnodes >= 2, "beam too large");
  FVX_ARG_CHECK(p.max_particles >= 1 && p.max_steps >= 1, "bad capacities");
  FVX_ARG_CHECK(precision == FVX_PREC_F64 || precision == FVX_PREC_F32C, "bad precision");
  FVX_ARG_CHECK(p.coupling == 0 || (p.coupling == 1 && state->gd != nullptr),
                "coupling %d unknown (or its displacement array missing)", p.coupling);
  FVX_ARG_CHECK(threads >= 2 * P && threads <= 512 && threads % (2 * P) == 0 && threads % 32 == 0,
                "threads must be a multiple of 2 x panels (and of 32), at most 512");
  FVX_ARG_CHECK((threads / (2 * P)) * 2 * P * 3 <= kMaxP * (kMaxP + 1),
                "too many slices for the reduction scratch");
  const size_t smem = sizeof(Smem);
  // two CTAs per environment (a cluster sharing its wake induction) when the
  // sweep leaves half of the SMs idle with one
  const int cl = 2 * p.n_env <= fvx::device_sm_count() ? 2 : 1;
  static bool attr_done[4] = {false, false, false, false};
  auto launch = [&](auto kernel, int idx) -> int {
    if (!attr_done[idx]) {
      FVX_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem)));
      attr_done[idx] = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(p.n_env * cl));
    cfg.blockDim = dim3(static_cast<unsigned>(threads));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = static_cast<cudaStream_t>(stream);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cl);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FVX_CUDA_TRY(cudaLaunchKernelEx(&cfg, kernel, p, *state, step_end));
    fvx::note_launch();
    return FVX_OK;
  };
  if (cl == 2) {
    if (precision == FVX_PREC_F32C) return launch(sweep_kernel<true, 2>, 3);
    return launch(sweep_kernel<false, 2>, 2);
  }
  if (precision == FVX_PREC_F32C) return launch(sweep_kernel<true, 1>, 1);
  return launch(sweep_kernel<false, 1>, 0);
}
