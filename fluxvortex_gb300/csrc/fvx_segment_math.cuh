// fvx_segment_math.cuh -- per-pair arithmetic of the PteraSoftware line
// vortex (Lamb-Oseen + Squire core), shared by the Biot-Savart sweeps
// (fvx_segments.cu) and the panel-method kernels (fvx_uvlm.cu).
//
// Follows src/fluxvortex/warp_kernels.py:46-96 operation by operation (FMA
// contraction aside), with the legs of one vortex fused: corner offsets and
// their lengths are computed once and shared by the two legs meeting at a
// corner, and the per-leg constants are hoisted into a VortexRec.
#pragma once

#include "fvx_common.cuh"

namespace fvx {
namespace seg {

constexpr double kEps0 = 2.22e-16;           // warp_kernels.py:52
constexpr double kTol = 1.0e-10;             // warp_kernels.py:70,81
constexpr double kFourLamb = 5.02572;        // 4 * 1.25643, warp_kernels.py:88
constexpr double kSquire = 1.0e-4;           // warp_kernels.py:88
constexpr double kInv4Pi = 0.07957747154594767;  // warp_kernels.py:89

template <int LEGS>
struct Legs;
template <>
struct Legs<FVX_LEGS_RING> {
  static constexpr int n = 4;
  __device__ static constexpr int s(int l) { return l; }
  __device__ static constexpr int e(int l) { return (l + 1) & 3; }
};
template <>
struct Legs<FVX_LEGS_CHORDWISE> {
  static constexpr int n = 2;
  __device__ static constexpr int s(int l) { return l == 0 ? 0 : 2; }
  __device__ static constexpr int e(int l) { return l == 0 ? 1 : 3; }
};
template <>
struct Legs<FVX_LEGS_HORSESHOE> {
  static constexpr int n = 3;
  __device__ static constexpr int s(int l) { return l; }
  __device__ static constexpr int e(int l) { return l + 1; }
};

// Hoisted per-vortex record (shared memory, read by broadcast).
struct VortexRec {
  double c[4][3];   // corners BR, FR, FL, BL
  double r0sq[4];   // |end - start|^2 per leg
  double tol[4];    // 1e-10 |end - start| per leg
  double c2[4];     // |end - start|^2 * r_c^2 per leg
  double c1;        // Gamma / (4 pi)
  int valid;        // bit l: leg l passes the zero-length test
  int pad;
};

template <int LEGS>
__device__ __forceinline__ void prep_vortex(VortexRec& R, const double* br, const double* fr,
                                            const double* fl, const double* bl, double strength,
                                            double rc0, double age, double nu) {
  const double* cs[4] = {br, fr, fl, bl};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    R.c[c][0] = cs[c][0];
    R.c[c][1] = cs[c][1];
    R.c[c][2] = cs[c][2];
  }
  double rc_sq = rc0 * rc0 + kFourLamb * (nu + kSquire * fabs(strength)) * age;
  R.c1 = strength * kInv4Pi;
  int valid = 0;
#pragma unroll
  for (int l = 0; l < Legs<LEGS>::n; ++l) {
    const double* s = cs[Legs<LEGS>::s(l)];
    const double* e = cs[Legs<LEGS>::e(l)];
    double r0x = e[0] - s[0], r0y = e[1] - s[1], r0z = e[2] - s[2];
    double r0_sq = r0x * r0x + r0y * r0y + r0z * r0z;
    double r0_len = sqrt(r0_sq);
    R.r0sq[l] = r0_sq;
    R.tol[l] = r0_len * kTol;
    R.c2[l] = r0_sq * rc_sq;
    if (!(r0_len < kEps0)) valid |= 1 << l;
  }
  R.valid = valid;
}

// Velocity of one vortex (all legs) at point p; cnt[k] counts skips.
template <int LEGS>
__device__ __forceinline__ void vortex_velocity(const VortexRec& R, double px, double py,
                                                double pz, double& vx, double& vy, double& vz,
                                                int cnt[4]) {
  double dx[4], dy[4], dz[4], len[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    dx[c] = R.c[c][0] - px;
    dy[c] = R.c[c][1] - py;
    dz[c] = R.c[c][2] - pz;
    len[c] = sqrt(dx[c] * dx[c] + dy[c] * dy[c] + dz[c] * dz[c]);
  }
  const int valid = R.valid;
#pragma unroll
  for (int l = 0; l < Legs<LEGS>::n; ++l) {
    const int a = Legs<LEGS>::s(l), b = Legs<LEGS>::e(l);
    if (!((valid >> l) & 1)) {
      cnt[0]++;
      continue;
    }
    const double tol = R.tol[l];
    if (len[a] < tol) {
      cnt[1]++;
      continue;
    }
    if (len[b] < tol) {
      cnt[2]++;
      continue;
    }
    double r3x = dy[a] * dz[b] - dz[a] * dy[b];
    double r3y = dz[a] * dx[b] - dx[a] * dz[b];
    double r3z = dx[a] * dy[b] - dy[a] * dx[b];
    double r3_sq = r3x * r3x + r3y * r3y + r3z * r3z;
    double r1r2 = len[a] * len[b];
    double thr = kTol * r1r2;
    if (r3_sq < 2.0 * thr * thr && sqrt(r3_sq) < thr) {
      cnt[3]++;
      continue;
    }
    double c3 = dx[a] * dx[b] + dy[a] * dy[b] + dz[a] * dz[b];
    double c4 = R.c1 * (len[a] + len[b]) * (r1r2 - c3) / (r1r2 * (r3_sq + R.c2[l]));
    vx += c4 * r3x;
    vy += c4 * r3y;
    vz += c4 * r3z;
  }
}

}  // namespace seg
}  // namespace fvx
