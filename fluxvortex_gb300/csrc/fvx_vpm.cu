// fvx_vpm.cu -- element-wise stages of the vortex-particle integrator (FP64).
//
// Restates the per-particle arithmetic of VortexParticleField.advect_rk3
// (src/fluxvortex/particles.py:85-199) and _relax_pedrizzetti (:202-246) as
// stream-ordered kernels over a device-resident AoS particle store; the
// all-pairs sweeps between stages are fvx_particle_pairs.  One RK3 stage
// (a, b) is:
//   U     = U_particles + U_inf (+ optional extra)        particles.py:110-123
//   |U| <= 50 (rescaled)                                    :125-130
//   rkX   = a rkX + dt U;  x += b rkX                       :132-134
//   [stretch]  S = J(x_new, G) . G                           :136-141
//   Z     = 0.2 (S . G)/|G|^2 if |G|^2 > 1e-20, |Z| <= 10/max(dt,1e-10)
//   dG    = S - 3 Z G;  ds = -s Z (+ nu / max(s, 1e-10))      :143-158
//   rkG   = a rkG + dt dG;  rks = a rks + dt ds; G += b rkG; s += b rks
//   |G|^2 <= 1e4 (rescaled); s in [1e-6, 5]                  :163-173
// then the NaN/Inf guard (:175-180), age += dt, and the relaxation pass.
#include "fvx_common.cuh"

namespace fvx {
namespace {

constexpr int kThreads = 256;

__global__ void stage_position_kernel(int64_t n, double a, double b, double dt, double ux,
                                      double uy, double uz, const double* __restrict__ u_part,
                                      const double* __restrict__ u_extra, double* __restrict__ pos,
                                      double* __restrict__ rk_x) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // (U_part + U_extra) + U_inf, the reference's order (particles.py:123)
  double u0 = 0.0, u1 = 0.0, u2 = 0.0;
  if (u_part) {
    u0 = u_part[3 * i];
    u1 = u_part[3 * i + 1];
    u2 = u_part[3 * i + 2];
  }
  if (u_extra) {
    u0 += u_extra[3 * i];
    u1 += u_extra[3 * i + 1];
    u2 += u_extra[3 * i + 2];
  }
  u0 += ux;
  u1 += uy;
  u2 += uz;
  const double sp = sqrt(u0 * u0 + u1 * u1 + u2 * u2);
  if (sp > 50.0) {
    const double k = 50.0 / sp;
    u0 *= k;
    u1 *= k;
    u2 *= k;
  }
  // a == 0 starts the RK3 registers from zero (particles.py:98-101)
  const bool first = a == 0.0;
  double r0 = (first ? 0.0 : a * rk_x[3 * i]) + dt * u0;
  double r1 = (first ? 0.0 : a * rk_x[3 * i + 1]) + dt * u1;
  double r2 = (first ? 0.0 : a * rk_x[3 * i + 2]) + dt * u2;
  rk_x[3 * i] = r0;
  rk_x[3 * i + 1] = r1;
  rk_x[3 * i + 2] = r2;
  pos[3 * i] += b * r0;
  pos[3 * i + 1] += b * r1;
  pos[3 * i + 2] += b * r2;
}

__global__ void stage_strength_kernel(int64_t n, double a, double b, double dt, double nu,
                                      const double* __restrict__ S, double* __restrict__ gam,
                                      double* __restrict__ sig, double* __restrict__ rk_g,
                                      double* __restrict__ rk_s) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double g0 = gam[3 * i], g1 = gam[3 * i + 1], g2 = gam[3 * i + 2];
  const double s0 = S[3 * i], s1 = S[3 * i + 1], s2 = S[3 * i + 2];
  const double gsq = g0 * g0 + g1 * g1 + g2 * g2;
  double Z = 0.0;
  if (gsq > 1e-20) Z = 0.2 * (s0 * g0 + s1 * g1 + s2 * g2) / gsq;
  const double zmax = 10.0 / fmax(dt, 1e-10);
  Z = fmin(fmax(Z, -zmax), zmax);
  const double sg = sig[i];
  double ds = -sg * Z;
  if (nu > 0.0) ds += nu / fmax(sg, 1e-10);
  const double d0 = s0 - 3.0 * Z * g0, d1 = s1 - 3.0 * Z * g1, d2 = s2 - 3.0 * Z * g2;
  const bool first = a == 0.0;
  const double q0 = (first ? 0.0 : a * rk_g[3 * i]) + dt * d0;
  const double q1 = (first ? 0.0 : a * rk_g[3 * i + 1]) + dt * d1;
  const double q2 = (first ? 0.0 : a * rk_g[3 * i + 2]) + dt * d2;
  const double qs = (first ? 0.0 : a * rk_s[i]) + dt * ds;
  rk_g[3 * i] = q0;
  rk_g[3 * i + 1] = q1;
  rk_g[3 * i + 2] = q2;
  rk_s[i] = qs;
  double n0 = g0 + b * q0, n1 = g1 + b * q1, n2 = g2 + b * q2;
  double ns = sg + b * qs;
  const double nsq = n0 * n0 + n1 * n1 + n2 * n2;
  if (nsq > 1e4) {
    const double k = sqrt(1e4 / nsq);
    n0 *= k;
    n1 *= k;
    n2 *= k;
  }
  ns = fmin(fmax(ns, 1e-6), 5.0);
  gam[3 * i] = n0;
  gam[3 * i + 1] = n1;
  gam[3 * i + 2] = n2;
  sig[i] = ns;
}

__global__ void finalize_kernel(int64_t n, double dt, const double* __restrict__ pos,
                                double* __restrict__ gam, double* __restrict__ age) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool ok = isfinite(pos[3 * i]) && isfinite(pos[3 * i + 1]) && isfinite(pos[3 * i + 2]) &&
            isfinite(gam[3 * i]) && isfinite(gam[3 * i + 1]) && isfinite(gam[3 * i + 2]);
  if (!ok) {
    gam[3 * i] = 0.0;
    gam[3 * i + 1] = 0.0;
    gam[3 * i + 2] = 0.0;
    flag_status(kStatusNonFinite);
  }
  age[i] += dt;
}

// particles.py:210-246 given the vorticity omega at every particle.
__global__ void relax_kernel(int64_t n, double rlxf, const double* __restrict__ omega,
                             double* __restrict__ gam) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double g0 = gam[3 * i], g1 = gam[3 * i + 1], g2 = gam[3 * i + 2];
  const double gn = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
  const double w0 = omega[3 * i], w1 = omega[3 * i + 1], w2 = omega[3 * i + 2];
  const double wn = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
  if (!(gn > 1e-15) || !(wn > 1e-12)) return;
  const double h0 = w0 / wn, h1 = w1 / wn, h2 = w2 / wn;
  g0 = (1.0 - rlxf) * g0 + rlxf * gn * h0;
  g1 = (1.0 - rlxf) * g1 + rlxf * gn * h1;
  g2 = (1.0 - rlxf) * g2 + rlxf * gn * h2;
  double b2 = 1.0 - 2.0 * (1.0 - rlxf) * rlxf *
                        (1.0 - (g0 * h0 + g1 * h1 + g2 * h2) / fmax(gn, 1e-12));
  b2 = fmax(b2, 0.01);
  const double k = sqrt(b2);
  gam[3 * i] = g0 / k;
  gam[3 * i + 1] = g1 / k;
  gam[3 * i + 2] = g2 / k;
}

unsigned blocks(int64_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

}  // namespace
}  // namespace fvx

extern "C" {

int fvx_vpm_stage_position(int64_t n, double a, double b, double dt, const double* u_inf,
                           const double* u_part, const double* u_extra, double* pos,
                           double* rk_x, void* stream) {
  FVX_ARG_CHECK(n >= 0 && u_inf, "bad arguments");
  if (n == 0) return FVX_OK;
  FVX_ARG_CHECK(pos && rk_x, "null state");
  fvx::stage_position_kernel<<<fvx::blocks(n), fvx::kThreads, 0,
                               static_cast<cudaStream_t>(stream)>>>(
      n, a, b, dt, u_inf[0], u_inf[1], u_inf[2], u_part, u_extra, pos, rk_x);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_vpm_stage_strength(int64_t n, double a, double b, double dt, double nu,
                           const double* stretch, double* gamma, double* sigma, double* rk_g,
                           double* rk_s, void* stream) {
  FVX_ARG_CHECK(n >= 0, "bad size");
  if (n == 0) return FVX_OK;
  FVX_ARG_CHECK(stretch && gamma && sigma && rk_g && rk_s, "null state");
  fvx::stage_strength_kernel<<<fvx::blocks(n), fvx::kThreads, 0,
                               static_cast<cudaStream_t>(stream)>>>(n, a, b, dt, nu, stretch,
                                                                    gamma, sigma, rk_g, rk_s);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_vpm_finalize(int64_t n, double dt, const double* pos, double* gamma, double* age,
                     void* stream) {
  FVX_ARG_CHECK(n >= 0, "bad size");
  if (n == 0) return FVX_OK;
  FVX_ARG_CHECK(pos && gamma && age, "null state");
  fvx::finalize_kernel<<<fvx::blocks(n), fvx::kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      n, dt, pos, gamma, age);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

int fvx_vpm_relax(int64_t n, double rlxf, const double* omega, double* gamma, void* stream) {
  FVX_ARG_CHECK(n >= 0, "bad size");
  if (n == 0 || !(rlxf > 0.0)) return FVX_OK;
  FVX_ARG_CHECK(omega && gamma, "null state");
  fvx::relax_kernel<<<fvx::blocks(n), fvx::kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      n, rlxf, omega, gamma);
  FVX_LAUNCH_CHECK();
  return FVX_OK;
}

}  // extern "C"
