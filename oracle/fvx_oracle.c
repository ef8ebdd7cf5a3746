/*
 * fvx_oracle.c -- CPU oracle for the vortex-induction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C (FP64, no FMA
 * contraction: build with -ffp-contract=off), the arithmetic of the reference
 * implementation so that the CUDA kernels of fluxvortex_gb300 can be checked
 * against it.  Only tests/, __graft_entry__.smoke() and the cpu_baseline leg of
 * bench.py may load it; the product path never does.
 *
 * Restated reference code (paths inside the FLUXVortex project):
 *   - line-vortex Biot-Savart with the PteraSoftware Lamb-Oseen + Squire core:
 *       src/fluxvortex/warp_kernels.py:26-97   (_collapsed_line_vortex_bs)
 *       src/fluxvortex/warp_kernels.py:102-173 (_expanded_line_vortex_bs)
 *     leg sets of the five public wrappers:
 *       ring       warp_kernels.py:268-273
 *       chordwise  warp_kernels.py:296-299
 *       horseshoe  warp_kernels.py:350-354 (ages forced to zero, :348)
 *   - vortex-particle velocity / velocity gradient:
 *       src/fluxvortex/kernel.py:69-116  (velocity_from_particles)
 *       src/fluxvortex/kernel.py:119-190 (jacobian_from_particles)
 *     cores: Gaussian-erf kernel.py:16-31, Winckelmans kernel.py:42-55
 *
 * Summation order: for a collapsed call each point sums leg 0 over all
 * vortices, then leg 1, ... (the order of the reference's per-leg launches,
 * warp_kernels.py:202-212).  Skip categories counted into counts[4]:
 *   0: zero-length leg          (warp_kernels.py:52)
 *   1: point at the leg start   (warp_kernels.py:72)
 *   2: point at the leg end     (warp_kernels.py:74)
 *   3: point on the leg's line  (warp_kernels.py:81)
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_LEGS_RING 0
#define ORC_LEGS_CHORDWISE 1
#define ORC_LEGS_HORSESHOE 2

#define ORC_KERNEL_GAUSSIANERF 0
#define ORC_KERNEL_WINCKELMANS 1

/* One (point, line vortex) pair, warp_kernels.py:42-96.  Returns -1 when the
 * pair contributed, else the skip category 0..3. */
static int orc_line_pair(const double *p, const double *s, const double *e,
                         double strength, double rc0, double age, double nu,
                         double vel[3])
{
    double r0x = e[0] - s[0];
    double r0y = e[1] - s[1];
    double r0z = e[2] - s[2];
    double r0_sq = r0x * r0x + r0y * r0y + r0z * r0z;
    double r0_len = sqrt(r0_sq);
    if (r0_len < 2.22e-16) return 0;

    double r1x = s[0] - p[0];
    double r1y = s[1] - p[1];
    double r1z = s[2] - p[2];
    double r2x = e[0] - p[0];
    double r2y = e[1] - p[1];
    double r2z = e[2] - p[2];

    double r3x = r1y * r2z - r1z * r2y;
    double r3y = r1z * r2x - r1x * r2z;
    double r3z = r1x * r2y - r1y * r2x;

    double r1_len = sqrt(r1x * r1x + r1y * r1y + r1z * r1z);
    double r2_len = sqrt(r2x * r2x + r2y * r2y + r2z * r2z);
    double r0_tol = r0_len * 1.0e-10;
    if (r1_len < r0_tol) return 1;
    if (r2_len < r0_tol) return 2;

    double r3_sq = r3x * r3x + r3y * r3y + r3z * r3z;
    double r3_len = sqrt(r3_sq);
    double r1r2 = r1_len * r2_len;
    if (r3_len < 1.0e-10 * r1r2) return 3;

    double rc_sq = rc0 * rc0 + 5.02572 * (nu + 1.0e-4 * fabs(strength)) * age;
    double c1 = strength * 0.07957747154594767;
    double c2 = r0_sq * rc_sq;
    double r1pr2 = r1_len + r2_len;
    double c3 = r1x * r2x + r1y * r2y + r1z * r2z;
    double c4 = c1 * r1pr2 * (r1r2 - c3) / (r1r2 * (r3_sq + c2));
    vel[0] = c4 * r3x;
    vel[1] = c4 * r3y;
    vel[2] = c4 * r3z;
    return -1;
}

/* Leg (start, end) corner indices per leg set; corners 0..3 = BR, FR, FL, BL. */
static int orc_legs(int leg_set, int starts[4], int ends[4])
{
    switch (leg_set) {
    case ORC_LEGS_RING:
        starts[0] = 0; ends[0] = 1;  /* BR -> FR */
        starts[1] = 1; ends[1] = 2;  /* FR -> FL */
        starts[2] = 2; ends[2] = 3;  /* FL -> BL */
        starts[3] = 3; ends[3] = 0;  /* BL -> BR */
        return 4;
    case ORC_LEGS_CHORDWISE:
        starts[0] = 0; ends[0] = 1;  /* BR -> FR */
        starts[1] = 2; ends[1] = 3;  /* FL -> BL */
        return 2;
    case ORC_LEGS_HORSESHOE:
        starts[0] = 0; ends[0] = 1;  /* BR -> FR */
        starts[1] = 1; ends[1] = 2;  /* FR -> FL */
        starts[2] = 2; ends[2] = 3;  /* FL -> BL */
        return 3;
    default:
        return -1;
    }
}

int orc_segments_collapsed(int64_t n_points, const double *points,
                           int64_t n_vort, const double *br, const double *fr,
                           const double *fl, const double *bl,
                           const double *strengths, const double *rc0s,
                           const double *ages, double nu, int leg_set,
                           double *out, int64_t *counts)
{
    int st[4], en[4];
    int nlegs = orc_legs(leg_set, st, en);
    if (nlegs < 0) return 1;
    const double *corner[4] = {br, fr, fl, bl};
    int64_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : c0, c1, c2, c3)
    for (int64_t i = 0; i < n_points; ++i) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int l = 0; l < nlegs; ++l) {
            for (int64_t m = 0; m < n_vort; ++m) {
                double v[3];
                double age = ages ? ages[m] : 0.0;
                int cat = orc_line_pair(points + 3 * i, corner[st[l]] + 3 * m,
                                        corner[en[l]] + 3 * m, strengths[m],
                                        rc0s[m], age, nu, v);
                if (cat < 0) {
                    acc[0] += v[0];
                    acc[1] += v[1];
                    acc[2] += v[2];
                } else if (cat == 0) c0++;
                else if (cat == 1) c1++;
                else if (cat == 2) c2++;
                else c3++;
            }
        }
        out[3 * i + 0] = acc[0];
        out[3 * i + 1] = acc[1];
        out[3 * i + 2] = acc[2];
    }
    if (counts) {
        counts[0] += c0; counts[1] += c1; counts[2] += c2; counts[3] += c3;
    }
    return 0;
}

int orc_segments_expanded(int64_t n_points, const double *points,
                          int64_t n_vort, const double *br, const double *fr,
                          const double *fl, const double *bl,
                          const double *strengths, const double *rc0s,
                          const double *ages, double nu, int leg_set,
                          double *out, int64_t *counts)
{
    int st[4], en[4];
    int nlegs = orc_legs(leg_set, st, en);
    if (nlegs < 0) return 1;
    const double *corner[4] = {br, fr, fl, bl};
    int64_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : c0, c1, c2, c3)
    for (int64_t i = 0; i < n_points; ++i) {
        for (int64_t m = 0; m < n_vort; ++m) {
            double acc[3] = {0.0, 0.0, 0.0};
            double age = ages ? ages[m] : 0.0;
            for (int l = 0; l < nlegs; ++l) {
                double v[3];
                int cat = orc_line_pair(points + 3 * i, corner[st[l]] + 3 * m,
                                        corner[en[l]] + 3 * m, strengths[m],
                                        rc0s[m], age, nu, v);
                if (cat < 0) {
                    acc[0] += v[0];
                    acc[1] += v[1];
                    acc[2] += v[2];
                } else if (cat == 0) c0++;
                else if (cat == 1) c1++;
                else if (cat == 2) c2++;
                else c3++;
            }
            double *o = out + 3 * (i * n_vort + m);
            o[0] = acc[0];
            o[1] = acc[1];
            o[2] = acc[2];
        }
    }
    if (counts) {
        counts[0] += c0; counts[1] += c1; counts[2] += c2; counts[3] += c3;
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Vortex particles, kernel.py:69-190.                                     */

static const double ORC_PI = 3.14159265358979323846;

/* g and dg/dr of the regularising core at r_bar, kernel.py:26-31, 51-55.
 *
 * Gaussian-erf: the reference evaluates g = erf(r/sqrt2) - c r exp(-r^2/2)
 * directly, which cancels catastrophically as r_bar -> 0 (relative error
 * ~3 eps / r_bar^2; at the self pair, r = 1e-12, g is pure rounding noise that
 * jacobian_from_particles then divides by r^3 = 1e-36).  Below r_bar = 0.5
 * this oracle, like the CUDA kernels, sums the Taylor series of
 * g(r) = c * int_0^r t^2 exp(-t^2/2) dt = c * sum_k (-1/2)^k / k! r^(2k+3)/(2k+3)
 * instead; above it the reference formula is used unchanged.  The
 * reference-faithful form (with SciPy's erf) lives in oracle.py. */
static double orc_gauss_g_series(double rb)
{
    double c = sqrt(2.0 / ORC_PI);
    double r2 = rb * rb;
    double term = rb * r2;            /* (-1/2)^k/k! r^(2k+3) */
    double sum = 0.0;
    for (int k = 0; k <= 10; ++k) {
        sum += term / (double)(2 * k + 3);
        term *= -0.5 * r2 / (double)(k + 1);
    }
    return c * sum;
}

static void orc_core(int kernel, double rb, double *g, double *dgdr)
{
    if (kernel == ORC_KERNEL_WINCKELMANS) {
        double r2 = rb * rb;
        *g = pow(rb, 3.0) * (r2 + 2.5) / pow(r2 + 1.0, 2.5);
        *dgdr = 7.5 * r2 / pow(r2 + 1.0, 3.5);
    } else {
        double c = sqrt(2.0 / ORC_PI);
        double ex = exp(-0.5 * rb * rb);
        if (rb < 0.5)
            *g = orc_gauss_g_series(rb);
        else
            *g = erf(rb / sqrt(2.0)) - c * rb * ex;
        *dgdr = c * rb * rb * ex;
    }
}

/* velocity_from_particles, kernel.py:84-116 (r clamped at 1e-12, :106). */
int orc_particle_velocity(int64_t n_tgt, const double *tgt, int64_t n_src,
                          const double *pos, const double *gam,
                          const double *sig, int kernel, double *out)
{
    const double C = -1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_tgt; ++i) {
        double u0 = 0.0, u1 = 0.0, u2 = 0.0;
        const double *t = tgt + 3 * i;
        for (int64_t j = 0; j < n_src; ++j) {
            const double *s = pos + 3 * j;
            const double *a = gam + 3 * j;
            double dx = t[0] - s[0], dy = t[1] - s[1], dz = t[2] - s[2];
            double r2 = dx * dx + dy * dy + dz * dz;
            double r = sqrt(r2);
            if (r < 1e-12) r = 1e-12;
            double g, dg;
            orc_core(kernel, r / sig[j], &g, &dg);
            double coeff = C * g / pow(r, 3.0);
            double cx = dy * a[2] - dz * a[1];
            double cy = dz * a[0] - dx * a[2];
            double cz = dx * a[1] - dy * a[0];
            u0 += coeff * cx;
            u1 += coeff * cy;
            u2 += coeff * cz;
        }
        out[3 * i + 0] = u0;
        out[3 * i + 1] = u1;
        out[3 * i + 2] = u2;
    }
    return 0;
}

/* jacobian_from_particles, kernel.py:137-190: J[t, i, j] = dU_i/dx_j. */
int orc_particle_jacobian(int64_t n_tgt, const double *tgt, int64_t n_src,
                          const double *pos, const double *gam,
                          const double *sig, int kernel, double *out)
{
    const double C = -1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_tgt; ++i) {
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double *t = tgt + 3 * i;
        for (int64_t j = 0; j < n_src; ++j) {
            const double *s = pos + 3 * j;
            const double *a = gam + 3 * j;
            double d[3] = {t[0] - s[0], t[1] - s[1], t[2] - s[2]};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            double r = sqrt(r2 > 1e-24 ? r2 : 1e-24);
            double g, dg;
            orc_core(kernel, r / sig[j], &g, &dg);
            double r3inv = 1.0 / pow(r, 3.0);
            double kx = C * (d[1] * a[2] - d[2] * a[1]) * r3inv;
            double ky = C * (d[2] * a[0] - d[0] * a[2]) * r3inv;
            double kz = C * (d[0] * a[1] - d[1] * a[0]) * r3inv;
            double aux = dg / (sig[j] * r) - 3.0 * g / (r * r);
            double aux2 = C * g * r3inv;
            J[0] += aux * kx * d[0];
            J[1] += aux * kx * d[1] + aux2 * a[2];
            J[2] += aux * kx * d[2] - aux2 * a[1];
            J[3] += aux * ky * d[0] - aux2 * a[2];
            J[4] += aux * ky * d[1];
            J[5] += aux * ky * d[2] + aux2 * a[0];
            J[6] += aux * kz * d[0] + aux2 * a[1];
            J[7] += aux * kz * d[1] - aux2 * a[0];
            J[8] += aux * kz * d[2];
        }
        memcpy(out + 9 * i, J, sizeof(J));
    }
    return 0;
}

/* Fused velocity + stretching S = J . Gamma_t (particles.py:148-151 with the
 * Jacobian of kernel.py:119-190), one pass. */
int orc_particle_velocity_stretch(int64_t n_tgt, const double *tgt,
                                  const double *tgt_gam, int64_t n_src,
                                  const double *pos, const double *gam,
                                  const double *sig, int kernel, double *u_out,
                                  double *s_out)
{
    const double C = -1.0 / (4.0 * ORC_PI);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n_tgt; ++i) {
        double u[3] = {0, 0, 0};
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double *t = tgt + 3 * i;
        for (int64_t j = 0; j < n_src; ++j) {
            const double *s = pos + 3 * j;
            const double *a = gam + 3 * j;
            double d[3] = {t[0] - s[0], t[1] - s[1], t[2] - s[2]};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            double rv = sqrt(r2);
            if (rv < 1e-12) rv = 1e-12;
            double g, dg;
            orc_core(kernel, rv / sig[j], &g, &dg);
            double cx = d[1] * a[2] - d[2] * a[1];
            double cy = d[2] * a[0] - d[0] * a[2];
            double cz = d[0] * a[1] - d[1] * a[0];
            double coeff = C * g / pow(rv, 3.0);
            u[0] += coeff * cx;
            u[1] += coeff * cy;
            u[2] += coeff * cz;
            double r = sqrt(r2 > 1e-24 ? r2 : 1e-24);
            orc_core(kernel, r / sig[j], &g, &dg);
            double r3inv = 1.0 / pow(r, 3.0);
            double kx = C * cx * r3inv, ky = C * cy * r3inv, kz = C * cz * r3inv;
            double aux = dg / (sig[j] * r) - 3.0 * g / (r * r);
            double aux2 = C * g * r3inv;
            J[0] += aux * kx * d[0];
            J[1] += aux * kx * d[1] + aux2 * a[2];
            J[2] += aux * kx * d[2] - aux2 * a[1];
            J[3] += aux * ky * d[0] - aux2 * a[2];
            J[4] += aux * ky * d[1];
            J[5] += aux * ky * d[2] + aux2 * a[0];
            J[6] += aux * kz * d[0] + aux2 * a[1];
            J[7] += aux * kz * d[1] - aux2 * a[0];
            J[8] += aux * kz * d[2];
        }
        const double *G = tgt_gam + 3 * i;
        u_out[3 * i + 0] = u[0];
        u_out[3 * i + 1] = u[1];
        u_out[3 * i + 2] = u[2];
        s_out[3 * i + 0] = J[0] * G[0] + J[1] * G[1] + J[2] * G[2];
        s_out[3 * i + 1] = J[3] * G[0] + J[4] * G[1] + J[5] * G[2];
        s_out[3 * i + 2] = J[6] * G[0] + J[7] * G[1] + J[8] * G[2];
    }
    return 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
