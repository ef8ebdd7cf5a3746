/*
 * fluxvortex_gb300.h -- C ABI of the GB300 (sm_103a) vortex-induction library.
 *
 * Conventions
 *   - Every entry returns an int status: FVX_OK (0) or an FVX_ERR_* code; the
 *     message of the last failure on the calling thread is fvx_last_error().
 *   - "Device" entries take device pointers and a cudaStream_t (passed as
 *     void*, NULL = legacy default stream); they are stream-ordered and return
 *     without synchronising.  "Host" entries (fvx_host_*) take host pointers,
 *     copy in, run, copy out and synchronise, like the NumPy functions they
 *     replace.
 *   - Point/vector arrays are (n, 3) float64, C-contiguous (AoS), exactly as
 *     the reference passes NumPy arrays; scalar-per-element arrays are (n,).
 *   - Device pointers should be 16-byte aligned (cudaMalloc / torch
 *     allocations are); unaligned inputs are accepted but staged without TMA.
 *
 * Reference interfaces replaced (paths inside the FLUXVortex project):
 *   - src/fluxvortex/warp_kernels.py:251-382, the five PteraSoftware
 *     `_aerodynamics_functions` Biot-Savart functions swapped in by
 *     src/fluxvortex/warp_patch.py:43-58;
 *   - src/fluxvortex/kernel.py:69-190, velocity_from_particles and
 *     jacobian_from_particles (and the unused Warp ports of them,
 *     src/fluxvortex/warp_vpm.py:20-173);
 *   - src/fluxvortex/particles.py:85-246, VortexParticleField.advect_rk3 and
 *     _relax_pedrizzetti.
 */
#ifndef FLUXVORTEX_GB300_H
#define FLUXVORTEX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FVX_OK 0
#define FVX_ERR_ARG 1        /* bad shape, pointer, enum or size */
#define FVX_ERR_CUDA 2       /* CUDA runtime error (message has details) */
#define FVX_ERR_CAPACITY 3   /* a fixed capacity would be exceeded */
#define FVX_ERR_TIMEOUT 4    /* a bounded device wait ran out */
#define FVX_ERR_SCRATCH 5    /* scratch buffer missing or too small */

/* ---- enums --------------------------------------------------------------- */
/* Leg sets of a ring given by corners BR, FR, FL, BL:
 *   RING       BR->FR, FR->FL, FL->BL, BL->BR   (warp_kernels.py:268-273)
 *   CHORDWISE  BR->FR, FL->BL                   (warp_kernels.py:296-299)
 *   HORSESHOE  BR->FR, FR->FL, FL->BL           (warp_kernels.py:350-354) */
#define FVX_LEGS_RING 0
#define FVX_LEGS_CHORDWISE 1
#define FVX_LEGS_HORSESHOE 2

/* Regularising cores of kernel.py:10-62. */
#define FVX_KERNEL_GAUSSIANERF 0
#define FVX_KERNEL_WINCKELMANS 1

/* Arithmetic of a particle sweep: FP64 throughout, or FP32 pair arithmetic on
 * tile-recentred coordinates with compensated (two-sum) FP32 accumulation. */
#define FVX_PREC_F64 0
#define FVX_PREC_F32C 1

/* What a particle sweep accumulates per target (C = -1/(4 pi), d = x_t - x_s):
 *   VELOCITY          u (M,3)                        kernel.py:69-116
 *   STRETCH           S = J . Gamma_t (M,3)          particles.py:148-151
 *   VELOCITY_STRETCH  u -> out_a, S -> out_b, same state
 *   JACOBIAN          J[t,i,j] = du_i/dx_j (M,3,3)   kernel.py:119-190
 *   VORTICITY         omega_i = eps_ijk J_kj (M,3)   particles.py:219-225 */
#define FVX_PAIR_VELOCITY 0
#define FVX_PAIR_STRETCH 1
#define FVX_PAIR_VELOCITY_STRETCH 2
#define FVX_PAIR_JACOBIAN 3
#define FVX_PAIR_VORTICITY 4

/* ---- library ------------------------------------------------------------- */
const char* fvx_version(void);
const char* fvx_last_error(void);
/* Number of kernels this library has launched in the process so far. */
unsigned long long fvx_launch_count(void);
/* Reads and clears the device status word (bit 1 = a bounded wait timed out,
 * 2 = non-finite value guarded, 4 = device capacity hit); synchronises
 * `stream`. */
int fvx_status_read_and_clear(unsigned* bits, void* stream);

/* ---- line-vortex segments (ring / chordwise / horseshoe) --------------------
 * Replaces warp_kernels.py:251-302 and :335-357 (collapsed) and :305-332,
 * :360-382 (expanded).  ages may be NULL (zero ages, as the horseshoe
 * wrappers force, warp_kernels.py:348,373).  singularity_counts, if not NULL,
 * is a device int64[4] incremented per (point, leg) pair skipped by the tests
 * of warp_kernels.py:52 (zero-length leg), :72 (point at leg start), :74
 * (point at leg end) and :81 (point on the leg's line).  Empty inputs
 * (n_points == 0 or n_vortices == 0) write zeros (warp_kernels.py:193-194). */
size_t fvx_segments_collapsed_scratch_bytes(int64_t n_points, int64_t n_vortices, int leg_set);
int fvx_segments_collapsed(const double* points, int64_t n_points, const double* br,
                           const double* fr, const double* fl, const double* bl,
                           const double* strengths, const double* r_c0s, const double* ages,
                           double nu, int64_t n_vortices, int leg_set, double* out /*(N,3)*/,
                           int64_t* singularity_counts, void* scratch, size_t scratch_bytes,
                           void* stream);
/* Scratch-free form of fvx_segments_collapsed, for callers that may not
 * allocate device memory while they run (a host that owns the GPU memory
 * budget and passes only input/output buffers; a fixed-rate stepping loop
 * where an allocation's device-wide synchronisation would stall it).  Same
 * arguments and results as fvx_segments_collapsed without the scratch pair:
 * its partial sums live in a 1 MiB array built into the library (held on
 * every GPU that loads it until the process exits).  Calls whose partial sums
 * need more than 1 MiB return FVX_ERR_CAPACITY before launching anything.
 * The first call on each device looks the array's address up
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU race.  This entry
 * point has no counterpart in the reference. */
int fvx_segments_collapsed_noalloc(const double* points, int64_t n_points, const double* br,
                                   const double* fr, const double* fl, const double* bl,
                                   const double* strengths, const double* r_c0s,
                                   const double* ages, double nu, int64_t n_vortices,
                                   int leg_set, double* out, int64_t* singularity_counts,
                                   void* stream);
int fvx_segments_expanded(const double* points, int64_t n_points, const double* br,
                          const double* fr, const double* fl, const double* bl,
                          const double* strengths, const double* r_c0s, const double* ages,
                          double nu, int64_t n_vortices, int leg_set, double* out /*(N,M,3)*/,
                          int64_t* singularity_counts, void* stream);

/* Host-pointer forms: same arguments with host arrays; output written to the
 * caller's host buffer; singularity_counts (host int64[4], may be NULL) is
 * incremented.  Synchronous, like the NumPy functions. */
typedef struct fvx_context fvx_context;
int fvx_context_create(int device, fvx_context** ctx);
void fvx_context_destroy(fvx_context* ctx);
int fvx_host_segments_collapsed(fvx_context* ctx, const double* points, int64_t n_points,
                                const double* br, const double* fr, const double* fl,
                                const double* bl, const double* strengths, const double* r_c0s,
                                const double* ages, double nu, int64_t n_vortices, int leg_set,
                                double* out, int64_t* singularity_counts);
int fvx_host_segments_expanded(fvx_context* ctx, const double* points, int64_t n_points,
                               const double* br, const double* fr, const double* fl,
                               const double* bl, const double* strengths, const double* r_c0s,
                               const double* ages, double nu, int64_t n_vortices, int leg_set,
                               double* out, int64_t* singularity_counts);

/* ---- vortex particles -------------------------------------------------------
 * One all-pairs sweep of n_sources particles (pos (N,3), alpha = vector
 * strength (N,3), sigma (N,)) over n_targets points tgt_pos (M,3).  tgt_gamma
 * (M,3) is required by STRETCH and VELOCITY_STRETCH only.  Outputs per the
 * FVX_PAIR_* table above; out_b is used by VELOCITY_STRETCH only.  The self
 * pair (d = 0) follows kernel.py's r -> 1e-12 clamp limit; the Gaussian-erf
 * core is evaluated without the cancellation of kernel.py:16-18 (series below
 * r/sigma = 0.5). */
size_t fvx_particle_pairs_scratch_bytes(int mode, int precision, int64_t n_targets,
                                        int64_t n_sources);
int fvx_particle_pairs(int mode, int kernel, int precision, const double* tgt_pos,
                       const double* tgt_gamma, int64_t n_targets, const double* src_pos,
                       const double* src_gamma, const double* src_sigma, int64_t n_sources,
                       double* out_a, double* out_b, void* scratch, size_t scratch_bytes,
                       void* stream);
int fvx_host_particle_pairs(fvx_context* ctx, int mode, int kernel, int precision,
                            const double* tgt_pos, const double* tgt_gamma, int64_t n_targets,
                            const double* src_pos, const double* src_gamma,
                            const double* src_sigma, int64_t n_sources, double* out_a,
                            double* out_b);

/* ---- vortex-particle integrator stages (particles.py:85-246) ---------------
 * Element-wise FP64 kernels over a device AoS particle store of n particles;
 * the caller runs the all-pairs sweeps (fvx_particle_pairs) between them.
 * stage_position: U = (u_part + u_extra) + u_inf (u_part, u_extra may be
 *   NULL; u_inf is a host double[3]), |U| clamped to 50, rk_x = a rk_x + dt U,
 *   pos += b rk_x.
 * stage_strength: rVPM update from stretch S = J . Gamma (Z = 0.2 S.G/|G|^2,
 *   |Z| <= 10/dt), viscous core growth nu / sigma, |G|^2 <= 1e4,
 *   sigma in [1e-6, 5].
 * finalize: zero the strength of particles with a non-finite position or
 *   strength (status bit 2), age += dt.
 * relax: Pedrizzetti realignment of gamma toward omega with factor rlxf. */
int fvx_vpm_stage_position(int64_t n, double a, double b, double dt, const double* u_inf,
                           const double* u_part, const double* u_extra, double* pos,
                           double* rk_x, void* stream);
int fvx_vpm_stage_strength(int64_t n, double a, double b, double dt, double nu,
                           const double* stretch, double* gamma, double* sigma, double* rk_g,
                           double* rk_s, void* stream);
int fvx_vpm_finalize(int64_t n, double dt, const double* pos, double* gamma, double* age,
                     void* stream);
int fvx_vpm_relax(int64_t n, double rlxf, const double* omega, double* gamma, void* stream);

/* ---- cell-binned treecode for particle self-induction sweeps ----------------------
 * Approximates fvx_particle_pairs with targets = sources = the n particles
 * (the self-sweeps of particles.py:122,148,219).  Near leaves: direct FP32
 * pairs (compensated); accepted cells (|dc|^2 > 3/4 (h_T + h_S)^2/theta^2):
 * quadrupole expansion of the vector potential, FP32.  Modes VELOCITY,
 * STRETCH (tgt_gamma = the particles' own strengths), VELOCITY_STRETCH and
 * VORTICITY.  The handle owns its device workspace (grown on demand) and the
 * call synchronises `stream` three times (bounding box, cell counts, list
 * sizes).  stats (host int64[8], may be NULL; also checks traversal overflow):
 * levels, leaves, near leaf pairs, far cell interactions, cells.  The
 * reference has no tree (its sweeps are direct); its notes call for one
 * (docs/phase0A_findings.md:33-35). */
typedef struct fvx_tree fvx_tree;
int fvx_tree_create(fvx_tree** tree);
void fvx_tree_destroy(fvx_tree* tree);
int fvx_tree_sweep(fvx_tree* tree, int mode, int kernel, const double* pos, const double* alpha,
                   const double* sigma, const double* tgt_gamma, int64_t n, double theta,
                   int leaf_target, double* out_a, double* out_b, int64_t* stats, void* stream);
/* Device time of the last sweep's evaluation kernel (waits for it).  stats
 * of the same sweep: [6] near particle pairs, [7] far (target, cell) pairs. */
int fvx_tree_last_eval_ms(fvx_tree* tree, float* ms);
/* Far-field method of the pairs beyond theta_local (new; no reference
 * counterpart).  FVX_FAR_M2P (default): every accepted cell is evaluated at
 * every target particle of the leaf from its quadrupole expansion.  The other
 * two move the accepted cells with |dc|^2 > 3/4 (h_T + h_S)^2 / theta_local^2
 * (all of them when theta_local = theta; stats[4] = their number) to a
 * local-expansion path: one evaluation per (target leaf, source cell) pair
 * gives the second-order local expansion (u, grad u, grad grad u) at the leaf
 * centre, summed per leaf and applied to each target particle.
 * FVX_FAR_M2L: the expansion is the analytic multipole-to-local translation
 * of the quadrupole.  FVX_FAR_LEARNED: the analytic translation plus the
 * tensor-core MLP's learned residual (W, b in the fvx_mlp_forward packing;
 * device pointers kept by the handle).
 * fvx_tree_last_local_ms: device time of the last sweep's local-expansion
 * stage (waits for it).
 * fvx_tree_sample_pairs: features X[k][48] (BF16), exact FP64-summed
 * normalised targets T[k][32] (FP32) and, if A is not NULL, the analytic
 * translation A[k][32] of k <= max_pairs local-path pairs of the last sweep,
 * strided evenly over the list (*n_out = k): list 0 = the leaves' own pairs,
 * 1 = the pairs shared through a parent of leaves (two-level lists, used when
 * theta_local = theta). */
#define FVX_FAR_M2P 0
#define FVX_FAR_M2L 1
#define FVX_FAR_LEARNED 2
int fvx_tree_set_far_field(fvx_tree* tree, int method, const void* W, const float* b,
                           double theta_local);
int fvx_tree_last_local_ms(fvx_tree* tree, float* ms);
/* The FP64 judge of the local-expansion path and its FP64 fallback (new; no
 * reference counterpart).  A sweep with FVX_FAR_M2L or FVX_FAR_LEARNED is
 * judged when `samples` > 0.  Every (target, cell) pair of the path falls in
 * one of 16 classes: its list (leaves' own pairs / pairs shared through
 * parents of leaves) x whether the cell is larger than the target x four bins
 * of the opening ratio mu = sqrt(3)/2 (h_T + h_S)/d against theta_local
 * (mu/theta >= 0.9, 0.8, 0.65, below).  A judged sweep samples each class
 * (samples/16 pairs per class, drawn at random anew every judged sweep, all
 * pairs of smaller classes), sums each sampled cell directly in FP64 at its
 * target's centre, and runs the sweep's own translation and network kernels
 * on the samples.  The error of an expansion is that across the target,
 * e = (|du| + rho |dJ| + rho^2/2 |dH|) / (|u| + rho |J| + rho^2/2 |H|), rho =
 * sqrt(3)/2 h_T/d, for the translation plus the network (e_l) and the
 * translation alone (e_a).  Per class, with f the fraction of its samples
 * whose e exceeds tol: f_l <= 1/4 keeps the network; else f_a <= 1/4 drops the
 * network for the class (translation alone); else every pair of the class is
 * summed directly in FP64 at every particle of its target.  Sampled pairs of
 * the expanded classes whose applied e exceeds tol are summed directly in
 * FP64 as well.  The decision is kept per sweep mode for the sweeps that are
 * not judged (samples = 0), until the next judged sweep; a new far-field
 * method starts with every class expanded.  Defaults: 256 samples, tol 0.1.
 * fvx_tree_last_validation: out[4] = pairs judged, pairs summed directly in
 * FP64, mean applied e, max applied e of the last judged sweep (waits for it).
 * fvx_tree_last_judge: the full record of the last judged sweep, up to n_out
 * doubles of: [0] pairs judged, [1] sampled pairs repaired, [2] pairs summed
 * directly in FP64 (whole classes + repairs), [3] mean and [4] max applied
 * e, [5] estimated fraction of the path's pairs left above tol (sum over the
 * expanded classes of n_k f_k / sum n_k), [6] pairs on the path, [7] 0, then
 * per class k = 0..15 five values at 8 + 5k: pairs, samples, samples with
 * e_l > tol, samples with e_a > tol, action (0 network, 1 translation alone,
 * 2 FP64 direct).  Class k = 8 list + 4 (cell larger) + distance bin. */
int fvx_tree_set_validation(fvx_tree* tree, int samples, double tol);
/* fvx_tree_hint_same_positions: the next sweep's particle positions are those
 * of the last full build (the caller has not moved them): the grid, sort,
 * cells and interaction lists are reused, while strengths, cores and target
 * strengths are gathered anew and the moments, expansions, validation and
 * evaluation recomputed.  A sweep with another position array, count, opening
 * angle, leaf size or far-field method builds anew whatever the hint. */
int fvx_tree_hint_same_positions(fvx_tree* tree);
/* fvx_tree_set_list_slots: capacities of the one-pass form of the two-level
 * lists (near leaves and local cells per leaf, cells per parent; defaults 512,
 * 1024, 1024): the lists are written into fixed slots without a counting pass,
 * a slot overflow falls back to counting; any 0 = always count. */
int fvx_tree_set_list_slots(fvx_tree* tree, int near, int lrn, int par);
int fvx_tree_last_validation(fvx_tree* tree, double* out);
int fvx_tree_last_judge(fvx_tree* tree, double* out, int n_out);
int fvx_tree_sample_pairs(fvx_tree* tree, int list, int max_pairs, void* X, float* T, float* A,
                          int* n_out, void* stream);

/* ---- panel side of the hybrid panel-particle step (FP64) ------------------------
 * Replaces the PteraSoftware solver stages that HybridSolver runs around the
 * Biot-Savart calls (tests/experiment_hybrid_panel_particle.py:114-204 and the
 * PS step order of idea-stage/architecture_analysis.md:7-27).  A wing is a
 * vertex grid verts[(nc+1)*w][3] (chordwise rows LE->TE, spanwise columns
 * left->right).  Several lifting surfaces with the same nc (PS airplanes with
 * several wings, e.g. tests/benchmark_flapping.py:28-141) share one grid, their
 * columns side by side, described by an FvxSurfaces layout: ring strip j spans
 * vertex columns col[j] and col[j]+1, ring k = i ns + j, P = nc*ns panels, and
 * vertex column c moves with surface surf[c], whose row of the motion table is
 * (heave_amp, flap_amp, omega, y0): heave h(t) = heave_amp sin(omega t) and
 * flapping theta(t) = flap_amp sin(omega t) about the x axis through the hinge
 * line y = +-y0 of each half wing (mirrored).  col NULL: one surface, strip j
 * spans columns j, j+1 (w = ns + 1); surf NULL: every column is surface 0.
 * The layout struct is read on the host at each call; its arrays are device
 * memory.
 *
 * kinematics: vertices at time t.
 * lattice: quarter-chord ring corners (br, fr, fl, bl: (P,3)), 3/4-chord
 *   collocation points, unit normals, areas, bound-leg centres and FR->FL
 *   vectors (P,3), trailing-edge back edge te_back (w,3).
 * aic: AIC[b][i][j] = (unit ring j at collocation i) . n_i for n_systems
 *   systems stored back to back (expanded ring Biot-Savart fused with n).
 * rhs: rhs_i = -((u_inf - v_body) + v1 + v2) . n_i (v1, v2 may be NULL).
 * lu_solve_batched: solves A x = b in place (x -> b) for n_systems P x P
 *   systems, partial pivoting; a zero pivot sets status bit 2.  P <= 192 runs
 *   on a cluster of 8 CTAs per system (thread-block clusters), larger P on
 *   one CTA per system; both give the same results.  A's contents afterwards
 *   are unspecified (the one-CTA form works in it).
 * lu_factor_batched / lu_solve_factored_batched (P <= 192): the same solve in
 *   two launches, so that the factorisation of A can overlap the work that
 *   forms b.  lu_factor_batched reads A and leaves the factorisation in
 *   `work` (lu_workspace_bytes(P) bytes per system, back to back); A is not
 *   written.  lu_solve_factored_batched then solves in place (x -> b) by
 *   replaying the fused kernel's elimination in its order, so x is the same
 *   bit for bit as lu_solve_batched's.  lu_workspace_bytes returns 0 for P
 *   outside 1..192.
 * loads: Kutta-Joukowski force on each bound leg, rho (G_ij - G_i-1,j) (V x l),
 *   V = u_inf - v_body + v1 + v2 + v3, minus rho dG/dt A n (gamma_prev NULL:
 *   no unsteady term); writes CL and CDi (device scalars) on the reference
 *   area s_ref (<= 0: the sum of the panel areas) and optionally the
 *   per-panel forces.
 * wake_rings: ring-wake vertex lattice W[(R+1)*w][3] with row strengths
 *   gam[R*ns] and row ages age[R] -> the ring layout of the Biot-Savart entries.
 * loads_bernoulli: the unsteady Bernoulli form of the loads
 *   (newton_pc/adapters/flap.py:357-377): per panel dp = rho (V . t_c dG/dc +
 *   V . t_s dG/ds + dG/dt) over the panel area along the normal (negated: the
 *   reference's rings circulate opposite to these), with t_c, t_s
 *   between the midpoints of the panel's vertex edges (verts = the grid of the
 *   step), the gradients restarting at the first row and at each surface's
 *   first strip, V = u_inf - v_body + v1 + v2 at the collocation points (no
 *   bound self-induction); CL, CDi and per-panel forces as for loads.
 * shed: W_new = [te_next; W_old + V dt], gam_new = [TE ring strengths;
 *   gam_old], age_new = [0; age_old + dt]; V = u_inf (prescribed wake) or, for
 *   a free ring wake, u_inf + v1 + v2 + v3 with v1..v3 ((R_old+1) w, 3) the
 *   velocities induced at the old vertices (any may be NULL; all NULL: the
 *   prescribed wake).
 * convert: rows r >= n_keep of W -> 4 particles per ring at leg midpoints
 *   with alpha = Gamma (b - a), skipping |Gamma| < 1e-15 and |alpha|^2 <= 1e-30
 *   (experiment_hybrid_panel_particle.py:173-200); sigma = sigma_vdt
 *   (sigma_rule 0) or 1.3 x the ring's mean edge (sigma_rule 1); appended at
 *   *count (device int64), clipped at capacity (status bit 4). */
typedef struct FvxSurfaces {
  int32_t ns;           /* ring strips per chordwise row */
  int32_t w;            /* vertex columns */
  const int32_t* col;   /* device (ns) or NULL */
  const int32_t* surf;  /* device (w) or NULL */
  const double* motion; /* device (4 per surface) */
} FvxSurfaces;

int fvx_uvlm_kinematics(int nc, const FvxSurfaces* s, const double* base, double t, double* out,
                        void* stream);
int fvx_uvlm_lattice(const double* verts, int nc, const FvxSurfaces* s, double* br, double* fr,
                     double* fl, double* bl, double* colloc, double* normal, double* area,
                     double* leg_center, double* leg_vec, double* te_back, void* stream);
int fvx_uvlm_aic(int n_systems, int P, const double* colloc, const double* normal,
                 const double* br, const double* fr, const double* fl, const double* bl,
                 double rc0, double nu, double* aic, void* stream);
int fvx_uvlm_rhs(int nc, const FvxSurfaces* s, const double* colloc, const double* normal,
                 const double* v1, const double* v2, const double* u_inf, double t, double* rhs,
                 void* stream);
int fvx_lu_solve_batched(int n_systems, int P, double* A, double* b, void* stream);
int64_t fvx_lu_workspace_bytes(int P);
int fvx_lu_factor_batched(int n_systems, int P, double* A, double* work, void* stream);
int fvx_lu_solve_factored_batched(int n_systems, int P, const double* work, double* b,
                                  void* stream);
int fvx_uvlm_loads(int nc, const FvxSurfaces* s, const double* gamma, const double* gamma_prev,
                   const double* leg_center, const double* leg_vec, const double* area,
                   const double* normal, const double* v1, const double* v2, const double* v3,
                   const double* u_inf, double rho, double dt, double t, double s_ref,
                   double* cl, double* cdi, double* force, void* stream);
int fvx_uvlm_wake_rings(int R, const FvxSurfaces* s, const double* W, const double* gam,
                        const double* age, double rc0, double* br, double* fr, double* fl,
                        double* bl, double* strength, double* rc0s, double* ages, void* stream);
int fvx_uvlm_loads_bernoulli(int nc, const FvxSurfaces* s, const double* verts,
                             const double* gamma, const double* gamma_prev, const double* colloc,
                             const double* area, const double* normal, const double* v1,
                             const double* v2, const double* u_inf, double rho, double dt,
                             double t, double s_ref, double* cl, double* cdi, double* force,
                             void* stream);
int fvx_uvlm_shed(int R_old, int nc, const FvxSurfaces* s, const double* W_old,
                  const double* gam_old, const double* age_old, const double* te_next,
                  const double* gamma, const double* u_inf, double dt, const double* v1,
                  const double* v2, const double* v3, double* W_new, double* gam_new,
                  double* age_new, void* stream);
int fvx_uvlm_convert(int R, int n_keep, const FvxSurfaces* s, const double* W,
                     const double* gam, int sigma_rule, double sigma_vdt, int64_t capacity,
                     int64_t* count, double* pos, double* alpha, double* sigma, double* age,
                     void* stream);

/* ---- particle population control (FP64) -------------------------------------------
 * The population control of the reference's flapping adapter
 * (newton_pc/adapters/flap.py:466-563), which keeps a long run's particle count
 * bounded.  Both entries work in place on the first n particles (pos, alpha:
 * (n,3); sigma, age: (n); device), keep the survivors in their order, return
 * the new count in *n_out (host) and synchronise the stream; n <= 2^22.
 * drop_oldest: keeps the newest `keep` particles (the oldest are at the front).
 * merge_pass: one pass of pairwise moment-conserving merging.  Candidates are
 *   the particles but the newest protect_newest, or, with protect_dist > 0, the
 *   particles farther than protect_dist from wing_c (nothing merges while
 *   n < 2 protect_newest).  Each is hashed to a cell of size 0.1 + 0.15 |x -
 *   wing_c|; consecutive candidates of a cell in the stable lexicographic order
 *   of the cell keys pair greedily when their strengths are aligned; a pair
 *   becomes alpha = a1 + a2 at the |a|-weighted centroid with the larger core,
 *   accepted when the velocity it induces at the n_ref (1..64) wing reference
 *   points ref_pts (device, (n_ref,3)) changes by less than eps x speed.
 *   wing_c (host, 3) = the mean of ref_pts; *n_merged (host) = merges accepted. */
size_t fvx_vpm_population_scratch_bytes(int64_t n);
int fvx_vpm_drop_oldest(int64_t n, int64_t keep, double* pos, double* alpha, double* sigma,
                        double* age, int64_t* n_out, void* scratch, size_t scratch_bytes,
                        void* stream);
int fvx_vpm_merge_pass(int64_t n, double* pos, double* alpha, double* sigma, double* age,
                       const double* ref_pts, int n_ref, const double* wing_c, double speed,
                       double eps, int64_t protect_newest, double protect_dist, int64_t* n_out,
                       int64_t* n_merged, void* scratch, size_t scratch_bytes, void* stream);

/* ---- batched aeroelastic flutter sweep ------------------------------------------
 * Replaces the reference's per-airspeed AeroelasticSolver runs
 * (src/fluxvortex/aeroelastic_solver.py:68-221 with beam_fe.py:231-351, driven
 * by tests/benchmark_goland.py:100-248) by one persistent launch: CTA e runs
 * environment e (airspeed u_inf[e]) from its stored step to
 * min(step_end, n_steps[e]) and stores its state back, so a sweep can be
 * advanced in one launch or in chunks (a CUDA graph may capture them).  The
 * coupled model per step: beam-deformed ring lattice, AIC, wake rings and
 * particles at collocation points and bound legs (particles in FP64, or FP32
 * with compensated sums for precision FVX_PREC_F32C), FP64 LU solve,
 * Kutta-Joukowski loads, station lift/torque about the elastic axis
 * distributed to the nodes, Newmark average-acceleration beam step with the
 * precomputed inverse effective stiffness, tip history, wake convection,
 * shedding and conversion of the ring row past n_keep into particles
 * (FIFO store of max_particles per environment).  threads: a multiple of
 * 2 x nc x ns and of 32, at most 512.  Limits: nc x ns <= 64, ns <= 16,
 * n_keep <= 15, 3 x nnodes <= 48.  A zero pivot sets status bit 2.
 * Layouts (env-major, FP64 unless noted): base_verts[(nc+1)(ns+1)][3];
 * vert_node/vert_xi: the span interpolation of each vertex; station_node/
 * station_xi: of each spanwise column's load station; kinv, mr, cr:
 * [nf][nf] (nf = 3 nnodes - 3, root clamped); u_inf[E][3]; n_steps[E] (int).
 * State: d, v, a [E][3 nnodes]; W[E][n_keep+2][ns+1][3], wgam[E][n_keep+1][ns],
 * wage[E][n_keep+1], nrows[E] (int); ppos, palp [E][max_particles][3],
 * psig[E][max_particles], phead, pcount [E] (int); gprev[E][nc ns],
 * has_prev[E] (int); hist_w, hist_th [E][max_steps]; step[E] (int). */
/* coupling: 0 = the physical model (motion velocity in the boundary
 * condition and the loads, torque about the elastic axis, deformation at every
 * vertex); 1 = the reference's coupling (aeroelastic_solver.py:68-221): every
 * panel moved with the beam's heave and twist at its collocation span station
 * (corners, ring vertices, collocation height), no motion velocity, station
 * lift and its moment about x = 0 with the collocation point's chordwise
 * position as the arm, the beam coupled from step 1 to the step before the
 * last, each coupling's displacements shaping the next step (state.gd);
 * hist_* then hold n_steps - 2 entries. */
typedef struct FlutterParams {
  int n_env, nc, ns, nnodes, n_keep, max_particles, max_steps, coupling;
  double x_ea, rc0, nu, rho, dt, beta, gamma, pad1;
  const double* base_verts;
  const int* vert_node;
  const double* vert_xi;
  const int* station_node;
  const double* station_xi;
  const double* kinv;
  const double* mr;
  const double* cr;
  const double* u_inf;
  const int* n_steps;
} FlutterParams;
typedef struct FlutterState {
  double *d, *v, *a;
  double *W, *wgam, *wage;
  int* nrows;
  double *ppos, *palp, *psig;
  int *phead, *pcount;
  double* gprev;
  int* has_prev;
  double *hist_w, *hist_th;
  int* step;
  double* gd;  /* coupling 1: the displacements that shape the geometry */
  /* optional (NULL: tip only): every node's (w, theta) per recorded step,
   * [env][max_steps][nnodes][2] */
  double* hist_nodes;
} FlutterState;
int fvx_flutter_sweep(const FlutterParams* params, const FlutterState* state, int step_end,
                      int precision, int threads, void* stream);

/* ---- learned far-field operator: BF16 tensor-core MLP (tcgen05) ---------------
 * No reference counterpart: the reference's notes plan a learned far field in
 * a treecode (docs/phase0A_findings.md:33-35); the operator is new.
 * Network: 48 inputs (35 used) -> 3 x 128 SiLU -> 32 outputs (30 used); W
 * packed [out][in] BF16 (W1 128x48, W2 128x128, W3 128x128, W4 32x128 = 45056
 * elements), bias packed FP32 (3 x 128 + 32 = 416).  For a (target leaf T,
 * source cell S) pair with R = c_T - c_S, d = |R| and m = |M0| + |M1|/h_S +
 * |M2|/h_S^2 (Frobenius norms of the cell's moments), the inputs are R/d,
 * h_S/d, h_T/d, M0/m, M1/(m h_S), M2/(m h_S^2) and the outputs the local
 * expansion of S's singular Biot-Savart field at c_T: u d^2/m (3), du/dx d^3/m
 * (9, [i][n] = du_i/dx_n), d2u/dx2 d^4/m (18, per component xx xy xz yy yz zz).
 * fvx_mlp_forward: Y[rows][32] FP32 from X[rows][48] BF16; z_store
 *   (3 x rows x 128 FP32) and h_store (3 x rows x 128 BF16), if not NULL,
 *   receive the hidden pre-activations and activations for training.  With
 *   both NULL (inference) the kernel runs the treecode far field's form: BF16
 *   operands, the hidden layers' weights and biases halved while staged in
 *   shared memory, each pair of SiLUs one packed BF16 add, tanh and FMA.
 * fvx_mlp_gemm: C[M][N] (+)= sum_k opA[m][k] opB[n][k], opA[m][k] = tA ?
 *   A[k*lda + m] : A[m*lda + k] (same for B), BF16 in, FP32 out, split over K
 *   into split_k slices added with atomics (accumulate != 0 adds into C).
 * fvx_mlp_loss_grad: weighted mean-square loss over the 30 used outputs:
 *   loss += sum w_r (Y - T)^2 (device scalar), dY = 2 w_r (Y - T) / (30 rows)
 *   in BF16 and FP32; row_weight (w_r, FP32 [rows]) may be NULL (w_r = 1).
 * fvx_mlp_silu_back: dZ = dH SiLU'(Z) (BF16 out), db[c] += sum_r dZ[r][c].
 * fvx_mlp_colsum: db[c] += sum_r G[r][c].
 * fvx_mlp_adam: Adam step `step` (1-based) on FP32 master weights w with
 *   moments m, v; writes the BF16 copy wb when not NULL.
 * fvx_tc_gemm_probe: C[128][N] = A[128][K] B[N][K]^T on one CTA (layout check;
 *   stride_mode 0 is the convention every kernel uses). */
int fvx_mlp_forward(const void* X, int rows, const void* W, const float* bias, float* Y,
                    float* z_store, void* h_store, void* stream);
int fvx_mlp_gemm(const void* A, int lda, int tA, const void* B, int ldb, int tB, float* C,
                 int ldc, int M, int N, int K, int split_k, int accumulate, void* stream);
int fvx_mlp_loss_grad(int rows, const float* Y, const float* T, const float* row_weight, void* dY,
                      float* dY32, float* loss, void* stream);
int fvx_mlp_silu_back(int rows, int cols, const float* dH, const float* Z, void* dZ, float* db,
                      void* stream);
int fvx_mlp_colsum(int rows, int cols, const float* G, float* db, void* stream);
int fvx_mlp_adam(int n, float* w, const float* g, float* m, float* v, void* wb, float lr,
                 float b1, float b2, float eps, int step, void* stream);
int fvx_tc_gemm_probe(const void* A, const void* B, int N, int K, float* C, int stride_mode,
                      void* stream);

/* ---- diagnostics -------------------------------------------------------------
 * Launches blocks_per_sm x SMs CTAs of 256 threads, each running `iters`
 * rounds of 8 independent FP32 FMAs (16 flop per round per thread): the
 * measured FP32 CUDA-core peak used as the particle sweeps' roofline.  No
 * reference counterpart (measurement only). */
int fvx_probe_fp32_fma(int blocks_per_sm, int iters, float* sink, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FLUXVORTEX_GB300_H */
