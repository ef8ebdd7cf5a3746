// fvx_pair_math.cuh -- per-pair arithmetic of the vortex-particle sweeps
// (regularising cores and the per-mode accumulations), shared by the direct
// all-pairs kernels (fvx_particles.cu) and the treecode near field
// (fvx_tree.cu).  See fvx_particles.cu for the closed forms.
#pragma once

#include "fvx_common.cuh"

namespace fvx {
namespace pair {

constexpr double kSqrt2OverPi = 0.79788456080286535588;
constexpr double kInvSqrt2 = 0.70710678118654752440;

template <int MODE>
struct ModeInfo;
template <>
struct ModeInfo<FVX_PAIR_VELOCITY> {
  static constexpr int ncomp = 3, na = 3;
  static constexpr bool need_fpr = false, need_tg = false;
};
template <>
struct ModeInfo<FVX_PAIR_STRETCH> {
  static constexpr int ncomp = 3, na = 3;
  static constexpr bool need_fpr = true, need_tg = true;
};
template <>
struct ModeInfo<FVX_PAIR_VELOCITY_STRETCH> {
  static constexpr int ncomp = 6, na = 3;
  static constexpr bool need_fpr = true, need_tg = true;
};
template <>
struct ModeInfo<FVX_PAIR_JACOBIAN> {
  static constexpr int ncomp = 9, na = 9;
  static constexpr bool need_fpr = true, need_tg = false;
};
template <>
struct ModeInfo<FVX_PAIR_VORTICITY> {
  static constexpr int ncomp = 3, na = 3;
  static constexpr bool need_fpr = true, need_tg = false;
};

// ---- regularising cores -----------------------------------------------------
// Series coefficients of h(rho) = g(rho)/rho^3 for the Gaussian-erf core:
// g(rho) = sqrt(2/pi) int_0^rho t^2 exp(-t^2/2) dt, so
// h = sqrt(2/pi) sum_k a_k rho^(2k), a_k = (-1)^k / (2^k k! (2k+3)).
#define FVX_GA0 (1.0 / 3.0)
#define FVX_GA1 (-1.0 / 10.0)
#define FVX_GA2 (1.0 / 56.0)
#define FVX_GA3 (-1.0 / 432.0)
#define FVX_GA4 (1.0 / 4224.0)
#define FVX_GA5 (-1.0 / 49920.0)
#define FVX_GA6 (1.0 / 691200.0)
#define FVX_GA7 (-1.0 / 10967040.0)
#define FVX_GA8 (1.0 / 196116480.0)
#define FVX_GA9 (-1.0 / 3901685760.0)
#define FVX_GA10 (1.0 / 85463500800.0)

// Staged per-source constants: s2 = sigma^2, k2 = 2.5 sigma^2 (Winckelmans)
// or 1/sigma (Gaussian).
template <int KERNEL, bool NEED_FPR>
__device__ __forceinline__ void core_f64(double r2, double s2, double k2, double& f,
                                         double& fpr) {
  if (KERNEL == FVX_KERNEL_WINCKELMANS) {
    double q = r2 + s2;
    double t = rsqrt(q);
    double t2 = t * t;
    double t5 = t2 * t2 * t;
    f = (r2 + k2) * t5;
    if (NEED_FPR) fpr = -(3.0 * r2 + 10.5 * s2) * (t5 * t2);
  } else {
    const double inv_s = k2;
    const double x = r2 * inv_s * inv_s;  // rho^2
    if (x < 0.25) {
      double h = FVX_GA10;
      h = fma(h, x, FVX_GA9);
      h = fma(h, x, FVX_GA8);
      h = fma(h, x, FVX_GA7);
      h = fma(h, x, FVX_GA6);
      h = fma(h, x, FVX_GA5);
      h = fma(h, x, FVX_GA4);
      h = fma(h, x, FVX_GA3);
      h = fma(h, x, FVX_GA2);
      h = fma(h, x, FVX_GA1);
      h = fma(h, x, FVX_GA0);
      const double is3 = inv_s * inv_s * inv_s;
      f = kSqrt2OverPi * h * is3;
      if (NEED_FPR) {
        double d = 20.0 * FVX_GA10;
        d = fma(d, x, 18.0 * FVX_GA9);
        d = fma(d, x, 16.0 * FVX_GA8);
        d = fma(d, x, 14.0 * FVX_GA7);
        d = fma(d, x, 12.0 * FVX_GA6);
        d = fma(d, x, 10.0 * FVX_GA5);
        d = fma(d, x, 8.0 * FVX_GA4);
        d = fma(d, x, 6.0 * FVX_GA3);
        d = fma(d, x, 4.0 * FVX_GA2);
        d = fma(d, x, 2.0 * FVX_GA1);
        fpr = kSqrt2OverPi * d * is3 * inv_s * inv_s;
      }
    } else if (x > 90.0) {
      // rho > 9.4: 1 - erf(rho/sqrt2) and rho exp(-rho^2/2) are below 1e-18,
      // so g = 1 (and g' ~ 0) in FP64: the core is the singular kernel.
      const double ir = rsqrt(r2);
      const double ir2 = ir * ir;
      f = ir2 * ir;
      if (NEED_FPR) fpr = -3.0 * f * ir2;
    } else {
      double r = sqrt(r2);
      double rho = r * inv_s;
      double e = exp(-0.5 * x);
      double g = erf(rho * kInvSqrt2) - kSqrt2OverPi * rho * e;
      double ir = 1.0 / r;
      double ir3 = ir * ir * ir;
      f = g * ir3;
      if (NEED_FPR) {
        double dg = kSqrt2OverPi * x * e;
        fpr = (dg * inv_s - 3.0 * g * ir) * ir3 * ir;
      }
    }
  }
}

template <int KERNEL, bool NEED_FPR>
__device__ __forceinline__ void core_f32(float r2, float s2, float k2, float& f, float& fpr) {
  if (KERNEL == FVX_KERNEL_WINCKELMANS) {
    float q = r2 + s2;
    float t = rsqrtf(q);
    float t2 = t * t;
    float t5 = t2 * t2 * t;
    f = (r2 + k2) * t5;
    // (3 r2 + 10.5 s2) t^2 <= 10.5 first: t^7 alone overflows FP32 once
    // r^2 + s^2 < ~1e-11 (cores near the integrator's 1e-6 floor), and the
    // self pair's 0 x inf would then be NaN where the FP64 sum gives 0
    if (NEED_FPR) fpr = -((3.0f * r2 + 10.5f * s2) * t2) * t5;
  } else {
    const float inv_s = k2;
    const float x = r2 * inv_s * inv_s;
    if (x < 0.25f) {
      float h = static_cast<float>(FVX_GA6);
      h = fmaf(h, x, static_cast<float>(FVX_GA5));
      h = fmaf(h, x, static_cast<float>(FVX_GA4));
      h = fmaf(h, x, static_cast<float>(FVX_GA3));
      h = fmaf(h, x, static_cast<float>(FVX_GA2));
      h = fmaf(h, x, static_cast<float>(FVX_GA1));
      h = fmaf(h, x, static_cast<float>(FVX_GA0));
      const float is3 = inv_s * inv_s * inv_s;
      f = static_cast<float>(kSqrt2OverPi) * h * is3;
      if (NEED_FPR) {
        float d = static_cast<float>(12.0 * FVX_GA6);
        d = fmaf(d, x, static_cast<float>(10.0 * FVX_GA5));
        d = fmaf(d, x, static_cast<float>(8.0 * FVX_GA4));
        d = fmaf(d, x, static_cast<float>(6.0 * FVX_GA3));
        d = fmaf(d, x, static_cast<float>(4.0 * FVX_GA2));
        d = fmaf(d, x, static_cast<float>(2.0 * FVX_GA1));
        fpr = static_cast<float>(kSqrt2OverPi) * d * is3 * inv_s * inv_s;
      }
    } else if (x > 50.0f) {
      // rho > 7.1: g = 1 and g' ~ 0 to FP32 round-off (terms below 1e-9)
      const float ir = rsqrtf(r2);
      const float ir2 = ir * ir;
      f = ir2 * ir;
      if (NEED_FPR) fpr = -3.0f * f * ir2;
    } else {
      float ir = rsqrtf(r2);
      float r = r2 * ir;
      float rho = r * inv_s;
      float e = expf(-0.5f * x);
      float g = erff(rho * static_cast<float>(kInvSqrt2)) -
                static_cast<float>(kSqrt2OverPi) * rho * e;
      float ir3 = ir * ir * ir;
      f = g * ir3;
      if (NEED_FPR) {
        float dg = static_cast<float>(kSqrt2OverPi) * x * e;
        fpr = (dg * inv_s - 3.0f * g * ir) * ir3 * ir;
      }
    }
  }
}

// ---- per-pair accumulation ----------------------------------------------------
template <int MODE, typename T>
__device__ __forceinline__ void accumulate(T* acc, T dx, T dy, T dz, T r2, T ax, T ay, T az,
                                           T f, T fpr, T gx, T gy, T gz) {
  if (MODE == FVX_PAIR_VELOCITY || MODE == FVX_PAIR_VELOCITY_STRETCH) {
    // u += (f d) x a
    const T ex = f * dx, ey = f * dy, ez = f * dz;
    acc[0] += ey * az - ez * ay;
    acc[1] += ez * ax - ex * az;
    acc[2] += ex * ay - ey * ax;
  }
  if (MODE == FVX_PAIR_STRETCH || MODE == FVX_PAIR_VELOCITY_STRETCH) {
    // S += f (G x a) + w (d x a) = (f G + w d) x a,  w = fpr (d . G)
    constexpr int o = MODE == FVX_PAIR_STRETCH ? 0 : 3;
    const T w = fpr * (dx * gx + dy * gy + dz * gz);
    const T vx = f * gx + w * dx, vy = f * gy + w * dy, vz = f * gz + w * dz;
    acc[o + 0] += vy * az - vz * ay;
    acc[o + 1] += vz * ax - vx * az;
    acc[o + 2] += vx * ay - vy * ax;
  }
  if (MODE == FVX_PAIR_JACOBIAN) {
    const T cx = dy * az - dz * ay;
    const T cy = dz * ax - dx * az;
    const T cz = dx * ay - dy * ax;
    const T px = fpr * cx, py = fpr * cy, pz = fpr * cz;
    acc[0] += px * dx;
    acc[1] += px * dy + f * az;
    acc[2] += px * dz - f * ay;
    acc[3] += py * dx - f * az;
    acc[4] += py * dy;
    acc[5] += py * dz + f * ax;
    acc[6] += pz * dx + f * ay;
    acc[7] += pz * dy - f * ax;
    acc[8] += pz * dz;
  }
  if (MODE == FVX_PAIR_VORTICITY) {
    // omega += d (fpr (d . a)) - a (fpr r^2 + 2 f)
    const T s1 = fpr * (dx * ax + dy * ay + dz * az);
    const T s2 = fpr * r2 + (f + f);
    acc[0] += dx * s1 - ax * s2;
    acc[1] += dy * s1 - ay * s2;
    acc[2] += dz * s1 - az * s2;
  }
}

}  // namespace pair
}  // namespace fvx
