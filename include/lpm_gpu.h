/*
 * lpm_gpu.h -- C ABI of the GB300 direct-sum library (liblpm_gpu.so).
 *
 * Drop-in replacements for the all-pairs direct sums of lpm-v2 that build each RK4
 * stage's right-hand side.  Every entry point takes plain host pointers and sizes,
 * copies to the GPU, runs the hand-written sm_103a kernels and copies the results back
 * before returning (synchronous, like the Fortran routines they replace).  A Fortran
 * caller binds them through iso_c_binding.
 *
 * Conventions shared by every entry point
 *  - Arrays are contiguous, length n, in particle order (Fortran 1-based array base
 *    pointers pass straight through); 1 <= n <= 2^31 - 1, the range of the 32-bit particle
 *    indices the library keeps.
 *  - active[j] is 1 for active (panel-centre) particles and 0 for passive (vertex)
 *    particles: the Fortran logical(klog) mask converted once with merge(1,0,mask).
 *  - i_begin/i_end are 1-based and inclusive, the MPISetup indexStart/indexEnd of the
 *    calling rank (src/MPISetup.f90:132-146).  Only outputs i_begin..i_end are written;
 *    other entries are left untouched, as the reference leaves them for MPI_BCAST.
 *  - mode selects the arithmetic:
 *      LPM_MODE_FP64  : FP64, the reference expression association with no fused
 *                       multiply-add, sources swept in ascending index order: results are
 *                       bit-identical to the Fortran loop built without FMA contraction.
 *      LPM_MODE_FP32C : pair arithmetic in FP32 with hi/lo positions, chord-form
 *                       denominators, per-tile compensated (TwoSum) accumulation and an
 *                       FP64 cross-tile reduction (velocity relative error <= 1e-6).
 *    OR-ing LPM_FLAG_CHECK_FINITE makes the call fail with LPM_ERR_NONFINITE when an
 *    output is NaN or Inf.
 *  - Return value: LPM_OK (0) or a negative LPM_ERR_* code; lpm_last_error_string()
 *    describes the last failure of the calling thread.  Nothing is thrown across the ABI.
 */
#ifndef LPM_GPU_H
#define LPM_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  LPM_OK = 0,
  LPM_ERR_ARG = -1,       /* bad argument (null pointer, n out of range, bad range or mode) */
  LPM_ERR_CUDA = -2,      /* a CUDA runtime call failed */
  LPM_ERR_TIMEOUT = -3,   /* a bounded device-side wait gave up */
  LPM_ERR_NONFINITE = -4, /* LPM_FLAG_CHECK_FINITE found a NaN/Inf output */
  LPM_ERR_ALLOC = -5,     /* device or host allocation failed */
  LPM_ERR_NO_DEVICE = -6, /* no usable CUDA device */
  LPM_ERR_STATE = -7      /* call in a wrong state (another device current, wrong handle mode) */
};

enum { LPM_MODE_FP64 = 0, LPM_MODE_FP32C = 1 };
#define LPM_MODE_MASK 0xff
#define LPM_FLAG_CHECK_FINITE 0x100

/* PSE kernel selector */
enum {
  LPM_PSE_K8_GEODESIC = 0, /* bivariateLaplacianKernel8 of the great-circle distance */
  LPM_PSE_GAUSS_CHORD = 1, /* second-order Gaussian, 4 exp(-r^2)/pi, chord distance    */
  LPM_PSE_K8_CHORD = 2     /* bivariateLaplacianKernel8 of the chord distance          */
};

const char* lpm_last_error_string(void);
/* Library version string and the compiled GPU architecture. */
const char* lpm_version(void);

/* ------------------------------------------------------------------ direct sums */

/* Replaces BVESphereVelocity (src/SphereBVESolver.f90:377-430):
 *   u_i = sum_{j != i, active} (x_i x x_j) * (-zeta_j A_j) / (4 pi a (a^2 - x_i.x_j))
 * for i in [i_begin, i_end].  zeta is the RELATIVE vorticity.  rotationRate is not an
 * argument because the reference sum never reads it. */
int lpm_bve_velocity(int64_t n, const double* x, const double* y, const double* z,
                     const double* zeta, const double* area, const int32_t* active,
                     double radius, int64_t i_begin, int64_t i_end, double* u, double* v,
                     double* w, int mode);

/* Replaces setVelocityFromVorticity (src/SphereBVE.f90:489-531): the same sum with the
 * denominator associated as a^2 - sum(x_i*x_j).  In LPM_MODE_FP32C it is identical to
 * lpm_bve_velocity. */
int lpm_bve_set_velocity_from_vorticity(int64_t n, const double* x, const double* y,
                                        const double* z, const double* zeta,
                                        const double* area, const int32_t* active,
                                        double radius, int64_t i_begin, int64_t i_end,
                                        double* u, double* v, double* w, int mode);

/* Replaces planarIncompressibleVelocity (src/PlaneIncompressibleSolver.f90:278-316):
 *   u_i = -sum omega_j A_j (y_i-y_j) / (2 pi (r^2 + delta^2)),
 *   v_i = +sum omega_j A_j (x_i-x_j) / (2 pi (r^2 + delta^2)),  j != i, active.
 * delta = 0 is the reference's singular kernel. */
int lpm_plane_velocity(int64_t n, const double* x, const double* y, const double* omega,
                       const double* area, const int32_t* active, double delta,
                       int64_t i_begin, int64_t i_end, double* u, double* v, int mode);

/* Replaces PSESphereLaplacianAtParticles (src/PSEDirectSum.f90:502-535) with
 * kernel = LPM_PSE_K8_GEODESIC, and the Gaussian chord-distance variant with
 * LPM_PSE_GAUSS_CHORD:
 *   lap_i = eps^-4 sum_{j active} (f_j - f_i) A_j K(d_ij / eps)
 * radius is the sphere radius used by the great-circle distance. */
int lpm_pse_sphere_laplacian(int64_t n, const double* x, const double* y, const double* z,
                             const double* f, const double* area, const int32_t* active,
                             double eps, double radius, int kernel, int64_t i_begin,
                             int64_t i_end, double* lap, int mode);

/* Replaces PSEPlaneLaplacianAtParticles (src/PSEDirectSum.f90:467-500): K8 of the planar
 * distance (kernel = LPM_PSE_K8_CHORD) or the Gaussian (LPM_PSE_GAUSS_CHORD). */
int lpm_pse_plane_laplacian(int64_t n, const double* x, const double* y, const double* f,
                            const double* area, const int32_t* active, double eps,
                            int kernel, int64_t i_begin, int64_t i_end, double* lap,
                            int mode);

/* Replaces PSESphereGradientAtParticles (src/PSEDirectSum.f90:220-267): the surface gradient
 * (gx, gy, gz) of f with the first-derivative kernel K1 of the great-circle distance,
 * eps**-4 P_i sum_j (f_j + f_i)(x_i - x_j) K1(d/eps) A_j with P_i = SphereProjection(x_i). */
int lpm_pse_sphere_gradient(int64_t n, const double* x, const double* y, const double* z,
                            const double* f, const double* area, const int32_t* active,
                            double eps, double radius, int64_t i_begin, int64_t i_end,
                            double* gx, double* gy, double* gz, int mode);

/* Replaces PSESphereDivergenceAtParticles (src/PSEDirectSum.f90:537-579): the divergence of
 * the vector field (vx, vy, vz), eps**-4 sum_j (P_i (x_i - x_j) K1(d/eps)) . (V_j + V_i) A_j. */
int lpm_pse_sphere_divergence(int64_t n, const double* x, const double* y, const double* z,
                              const double* vx, const double* vy, const double* vz,
                              const double* area, const int32_t* active, double eps,
                              double radius, int64_t i_begin, int64_t i_end, double* div,
                              int mode);

/* The remaining PSE operators have only LPM_MODE_FP64 (the reference's association, like the
 * other FP64 sums); LPM_MODE_FP32C returns LPM_ERR_ARG.  The shallow-water integrals have
 * both modes. */

/* Replaces PSEPlaneGradientAtParticles (src/PSEDirectSum.f90:180-217): (gx, gy) =
 * eps**-4 sum_j (f_j + f_i)(x_i - x_j) K1(|x_i - x_j|/eps) A_j. */
int lpm_pse_plane_gradient(int64_t n, const double* x, const double* y, const double* f,
                           const double* area, const int32_t* active, double eps, int64_t i_begin,
                           int64_t i_end, double* gx, double* gy, int mode);

/* Replaces PSEPlaneSecondPartialsAtParticles (src/PSEDirectSum.f90:269-320): from the gradient
 * field (gx, gy), the second partials (dxx, dxy, dyy); dxy is 0.5 (d_y gx + d_x gy). */
int lpm_pse_plane_second_partials(int64_t n, const double* x, const double* y, const double* gx,
                                  const double* gy, const double* area, const int32_t* active,
                                  double eps, int64_t i_begin, int64_t i_end, double* dxx,
                                  double* dxy, double* dyy, int mode);

/* Replaces PSEPlaneDoubleDotProductAtParticles (src/PSEDirectSum.f90:322-365): the double dot
 * product ux ux + 2 uy vx + vy vy of the velocity (u, v). */
int lpm_pse_plane_double_dot(int64_t n, const double* x, const double* y, const double* u,
                             const double* v, const double* area, const int32_t* active, double eps,
                             int64_t i_begin, int64_t i_end, double* ddot, int mode);

/* Replaces PSESphereDoubleDotProductAtParticles (src/PSEDirectSum.f90:367-418), including its
 * pairing of w_j with v_i in the third row (:399-404).  radius is SphereDistance's radius. */
int lpm_pse_sphere_double_dot(int64_t n, const double* x, const double* y, const double* z,
                              const double* u, const double* v, const double* w, const double* area,
                              const int32_t* active, double eps, double radius, int64_t i_begin,
                              int64_t i_end, double* ddot, int mode);

enum { LPM_GEOMETRY_PLANE = 0, LPM_GEOMETRY_SPHERE = 1 };

/* Replaces PSEPlaneInterpolateScalar (geometry LPM_GEOMETRY_PLANE, chord distance) and
 * PSESphereInterpolateScalar (LPM_GEOMETRY_SPHERE, great-circle distance times radius),
 * src/PSEDirectSum.f90:128-168, evaluated at m query points (qx, qy, qz) at once:
 * out_k = sum_j f_j A_j Kdelta8(dist(q_k, x_j)/eps) / eps**2.  z and qz may be NULL in the
 * plane (zeros). */
int lpm_pse_interpolate_scalar(int64_t n, const double* x, const double* y, const double* z,
                               const double* f, const double* area, const int32_t* active, double eps,
                               double radius, int geometry, int64_t m, const double* qx,
                               const double* qy, const double* qz, double* out, int mode);

/* Replaces SWEPlaneRHSIntegrals (src/SWEPlaneSolver.f90:457-571): velocity (u, v) from
 * vorticity and divergence, the double dot product of the velocity gradient and the PSE
 * Laplacian of the surface height.  surf_height = h + topoFn(x, y), evaluated by the caller
 * (the Fortran shim) once per particle.  LPM_MODE_FP32C: velocity <= 1e-6 of max|u|, double
 * dot product <= 2e-6 of its max, Laplacian as the planar PSE FP32C sweep. */
int lpm_swe_plane_rhs_integrals(int64_t n, const double* x, const double* y, const double* vort,
                                const double* div, const double* surf_height, const double* area,
                                const int32_t* active, double eps, int64_t i_begin, int64_t i_end,
                                double* u, double* v, double* double_dot, double* lap_surf, int mode);

/* Replaces SWESphereRHSIntegrals (src/SphereSWESolver.f90:299-372) as the reference computes
 * it: (u, v, w) from relative vorticity and divergence on the sphere of radius `radius`, the
 * surface-height Laplacian with K8(SphereDistance/eps)/eps**2 (SphereDistance scaled by the
 * SphereGeometry module's SphereRadius, `sphere_radius`; no further 1/eps**2), and
 * double_dot = 0 (the reference never sets it).  surf_height = h + topoFn(x, y, z).
 * LPM_MODE_FP32C: velocity <= 1e-6 of max|u| (one sweep for the rotational and potential
 * parts), Laplacian as the geodesic PSE FP32C sweep. */
int lpm_swe_sphere_rhs_integrals(int64_t n, const double* x, const double* y, const double* z,
                                 const double* relvort, const double* div, const double* surf_height,
                                 const double* area, const int32_t* active, double radius,
                                 double sphere_radius, double eps, int64_t i_begin, int64_t i_end,
                                 double* u, double* v, double* w, double* double_dot,
                                 double* lap_surf, int mode);

/* Replaces BetaPlaneVelocity (src/BetaPlaneSolver.f90:227-268) and the beta plane's
 * setVelocityFromVorticity (src/BetaPlane.f90:359-397), the x-periodic (period 1) sum
 *   u_i = -sum_j sinh(2 pi dy) s_j,  v_i = sum_j sin(2 pi dx) s_j,
 *   s_j = 0.5 zeta_j A_j / (cosh(2 pi dy) - cos(2 pi dx)),  dx = x_i - x_j, dy = y_i - y_j,
 * over active j != i.  LPM_MODE_FP32C evaluates the kernel in FP32 in a form without
 * cancellation (sinh/sin of half angles) with periodic neighbours kept to full precision,
 * velocity error <= 1e-6 of max|u|. */
int lpm_beta_plane_velocity(int64_t n, const double* x, const double* y, const double* zeta,
                            const double* area, const int32_t* active, int64_t i_begin, int64_t i_end,
                            double* u, double* v, int mode);

/* Replaces the beta plane's SetStreamFunctionsOnMesh (src/BetaPlane.f90:399-442):
 * psi = sum_{j != i} log(cosh(2 pi dy) - cos(2 pi dx)) / (4 pi) zeta_j A_j for the relative
 * and the absolute vorticity.  LPM_MODE_FP32C uses the cancellation-free form
 * log(2 (sinh^2 + sin^2)) of the half angles, <= 1e-6 of max|psi|. */
int lpm_beta_plane_stream_functions(int64_t n, const double* x, const double* y, const double* relvort,
                                    const double* absvort, const double* area, const int32_t* active,
                                    int64_t i_begin, int64_t i_end, double* psi_rel, double* psi_abs,
                                    int mode);

/* Replaces SetStreamFunctionsOnMesh (src/SphereBVE.f90:445-485): psi = sum G zeta A with
 * G = -log(a^2 - x_i.x_j)/(4 pi), for the relative and absolute vorticity, j != i.
 * LPM_MODE_FP64 follows the Fortran loop (its log is CUDA's, so agreement is to ~1e-15
 * relative, not bitwise); LPM_MODE_FP32C forms a^2 - x_i.x_j without cancellation and
 * takes the log on the MUFU unit (error ~1e-7 of max |psi|). */
int lpm_bve_stream_functions(int64_t n, const double* x, const double* y, const double* z,
                             const double* relvort, const double* absvort,
                             const double* area, const int32_t* active, double radius,
                             int64_t i_begin, int64_t i_end, double* psi_rel,
                             double* psi_abs, int mode);

/* Replaces SetStreamFunctionOnMesh (src/PlanarIncompressible.f90:470-505):
 * psi = sum log(|x_i - x_j|)/(2 pi) omega_j A_j, j != i; modes as for the sphere. */
int lpm_plane_stream_function(int64_t n, const double* x, const double* y,
                              const double* omega, const double* area,
                              const int32_t* active, int64_t i_begin, int64_t i_end,
                              double* psi, int mode);

/* ------------------------------------------------------------------ RK4 solvers */

/* Device-resident BVESolver (src/SphereBVESolver.f90:38-353).  create copies the state
 * (New(BVESolver, sphere)); u/v/w are the velocity at the initial positions (the stage-1
 * reuse of the reference) -- pass NULL to have them computed with setVelocityFromVorticity.
 * timestep advances n_steps classical RK4 steps without returning to the host; the four
 * velocity sums of each step are replayed from one captured CUDA graph.  renormalize != 0
 * projects positions back onto the sphere after each step (an extension; the reference
 * does not renormalise). */
typedef struct lpm_bve_solver lpm_bve_solver;
int lpm_bve_solver_create(lpm_bve_solver** solver, int64_t n, const double* x,
                          const double* y, const double* z, const double* relvort,
                          const double* area, const int32_t* active, const double* u,
                          const double* v, const double* w, double radius,
                          double rotation_rate, int mode);
int lpm_bve_timestep(lpm_bve_solver* solver, double dt, int n_steps, int renormalize);
int lpm_bve_get_state(lpm_bve_solver* solver, double* x, double* y, double* z,
                      double* relvort, double* u, double* v, double* w);
int lpm_bve_set_state(lpm_bve_solver* solver, const double* x, const double* y,
                      const double* z, const double* relvort, const double* u,
                      const double* v, const double* w);
/* Replaces the Delete(solver) + New(solver, sphere) pair that follows a remesh
 * (examples/BVESingleGaussianVortex.f90:241-245, src/SphereBVESolver.f90:112-168): loads a
 * new particle set (n may change, and the active mask with it) into the existing solver.
 * The device buffers are reused when the new set fits them and grown with 1/8 headroom
 * when it does not, so a run that remeshes every few steps does not reallocate; the step
 * graph is re-captured at the next lpm_bve_timestep.  u, v, w as for lpm_bve_solver_create
 * (NULL: the velocity is computed from the vorticity).  The state is then identical to a
 * newly created solver's. */
int lpm_bve_solver_remesh(lpm_bve_solver* solver, int64_t n, const double* x, const double* y,
                          const double* z, const double* relvort, const double* area,
                          const int32_t* active, const double* u, const double* v,
                          const double* w);
/* KE = 1/2 sum |u|^2 A, enstrophy = 1/2 sum zeta^2 A, circulation = sum zeta A over
 * active particles (src/SphereBVE.f90:410-441). */
int lpm_bve_diagnostics(lpm_bve_solver* solver, double* kinetic_energy, double* enstrophy,
                        double* circulation);
/* Accumulated device time of the velocity sums launched by lpm_bve_timestep, measured
 * with CUDA events on the solver's stream, and the number of kernels lpm_bve_timestep has
 * launched (stage kernels, direct sums and the per-step source sort). */
int lpm_bve_kernel_timing(lpm_bve_solver* solver, double* total_ms, int64_t* launches);
/* SetStreamFunctionsOnMesh (src/SphereBVE.f90:445-485) at the solver's current state, as
 * the reference's Timestep calls it after every step (src/SphereBVESolver.f90:352): psi_rel
 * and psi_abs (length n, host arrays) from the device-resident positions and vorticity, in
 * the solver's mode.  absvort (length n, host) is the caller's absolute vorticity field; NULL
 * uses zeta + 2 Omega z / a of the current state, which equals the reference's materially
 * conserved field up to rounding when positions are not renormalised. */
int lpm_bve_solver_stream_functions(lpm_bve_solver* solver, const double* absvort, double* psi_rel,
                                    double* psi_abs);

/* Makes the solver enqueue its work on `stream` (a cudaStream_t of the caller's context;
 * NULL restores the solver's own stream), so the caller can time it with events. */
int lpm_bve_solver_set_stream(lpm_bve_solver* solver, void* stream);
/* enable != 0 (the default): lpm_bve_timestep synchronises after every step to accumulate
 * the kernel timing; 0: steps are replayed back to back with one synchronisation at the end. */
int lpm_bve_solver_set_timing(lpm_bve_solver* solver, int enable);
int lpm_bve_solver_destroy(lpm_bve_solver* solver);

/* Device-resident PlaneSolver (src/PlaneIncompressibleSolver.f90:103-259). */
typedef struct lpm_plane_solver lpm_plane_solver;
int lpm_plane_solver_create(lpm_plane_solver** solver, int64_t n, const double* x,
                            const double* y, const double* omega, const double* area,
                            const int32_t* active, const double* u, const double* v,
                            double delta, int mode);
int lpm_plane_timestep(lpm_plane_solver* solver, double dt, int n_steps);
int lpm_plane_get_state(lpm_plane_solver* solver, double* x, double* y, double* u,
                        double* v);
/* The planar counterpart of lpm_bve_solver_remesh (the Delete + New of the solver after a
 * remesh in examples/CollidingDipoles.f90): loads a new particle set into the solver,
 * reusing its device buffers when the set fits them. */
int lpm_plane_solver_remesh(lpm_plane_solver* solver, int64_t n, const double* x, const double* y,
                            const double* omega, const double* area, const int32_t* active,
                            const double* u, const double* v);
int lpm_plane_diagnostics(lpm_plane_solver* solver, double* kinetic_energy,
                          double* enstrophy, double* circulation);
int lpm_plane_solver_destroy(lpm_plane_solver* solver);

/* ------------------------------------------------------------------ ensembles */

/* Many independent sphere-BVE instances of uneven size advanced together.  Instance k
 * owns particles offsets[k] .. offsets[k+1]-1 of the concatenated arrays.  Each RK4 stage
 * of all instances is one persistent launch over a flattened (instance, target block,
 * source range) work queue; the steps are replayed from a captured CUDA graph.  mode must
 * be LPM_MODE_FP32C or LPM_MODE_FP64 (FP64 runs the bit-exact sweep instance by instance).
 * renormalize has the meaning of lpm_bve_timestep's. */
typedef struct lpm_ensemble lpm_ensemble;
int lpm_ensemble_create(lpm_ensemble** ens, int n_instances, const int64_t* offsets,
                        const double* x, const double* y, const double* z,
                        const double* relvort, const double* area, const int32_t* active,
                        const double* radius, const double* rotation_rate, int mode);
int lpm_ensemble_timestep(lpm_ensemble* ens, double dt, int n_steps, int renormalize);
/* One velocity evaluation of every instance at the current state. */
int lpm_ensemble_velocity(lpm_ensemble* ens);
int lpm_ensemble_get_state(lpm_ensemble* ens, double* x, double* y, double* z,
                           double* relvort, double* u, double* v, double* w);
int lpm_ensemble_kernel_timing(lpm_ensemble* ens, double* total_ms, int64_t* launches);
/* The persistent sweep's configuration the autotuner chose at creation (LPM_MODE_FP32C; all
 * zero in LPM_MODE_FP64): CTA threads, targets per thread, CTAs per SM, and the work items
 * per resident CTA the source ranges were cut for.  Any pointer may be NULL. */
int lpm_ensemble_sweep_shape(lpm_ensemble* ens, int* threads, int* targets_per_thread,
                             int* ctas_per_sm, int* items_per_slot);
/* Replaces the autotuner's choice with a given one (LPM_MODE_FP32C): threads x
 * targets_per_thread must be 128 x 4 or 128 x 8, items_per_slot 4, 8 or 16; anything else
 * fails with LPM_ERR_ARG.  For reproducible timings, or to test every shape. */
int lpm_ensemble_select_sweep(lpm_ensemble* ens, int threads, int targets_per_thread,
                              int items_per_slot);
int lpm_ensemble_destroy(lpm_ensemble* ens);

/* ------------------------------------------------------------------ allocation-free call */

/* lpm_bve_velocity_noalloc has no counterpart in the reference.  It is for callers that
 * cannot allocate device memory while they run: a host code whose own pool allocator
 * already holds the GPU's memory, or a time loop that cannot pay the device-wide
 * synchronisation cudaMalloc/cudaFree may cause.  Every input and output is a DEVICE
 * pointer owned by the caller (same meaning as lpm_bve_velocity, 1-based i_begin..i_end,
 * outputs outside the block untouched); the call computes the LPM_MODE_FP32C sum and
 * allocates nothing -- no cudaMalloc, cudaFree or allocating library routine.  Its scratch
 * is one file-scope device array of about 24 MiB, which limits n to
 * LPM_NOALLOC_MAX_PARTICLES; larger n fails with LPM_ERR_ARG.  Under CUDA's lazy module
 * loading (the default) the array is reserved on a device by the first call made there, and
 * held until the context is destroyed: a caller whose pool takes most of HBM should make one
 * call before the pool does.  The first call in a CUDA context also looks up the array's
 * device address, so make it before any stream capture.  All calls on a device share the
 * array: calls that overlap on the GPU (several host threads or streams) race, so serialise
 * them.  Work is enqueued on `stream` (a cudaStream_t, NULL for the default stream) and the
 * call returns after the stream has finished it; on an error return u, v and w are left as
 * they were. */
#define LPM_NOALLOC_MAX_PARTICLES 262144
int lpm_bve_velocity_noalloc(int64_t n, const double* x, const double* y, const double* z,
                             const double* zeta, const double* area, const int32_t* active,
                             double radius, int64_t i_begin, int64_t i_end, double* u,
                             double* v, double* w, void* stream);

/* ------------------------------------------------------------------ workspace and test hooks */

/* Frees the device workspace the host-buffer calls keep between calls (it grows to the
 * largest sum seen and is otherwise held until the process exits).  Synchronous; the next
 * host-buffer call allocates again.  No counterpart in the reference, which has no device
 * memory; the analogue of releasing a cached allocator's free blocks. */
int lpm_release_workspace(void);

/* Test hooks (no counterpart in the reference; they exercise the error paths that the
 * Fortran shim maps to LogMessage(..., ERROR_LOGGING_LEVEL, ...), src/Logger.f90:159).
 *
 * lpm_debug_fail_device_alloc(k): the k-th device allocation the library makes from now on
 * (k >= 1) fails as if cudaMalloc had run out of memory, and the call that made it returns
 * LPM_ERR_ALLOC; k = 0 disarms.  Every handle or workspace allocated before the failure is
 * released or kept consistent, so the next call succeeds.
 *
 * lpm_debug_inject_wait_timeout(skip_tile, budget_ns): the next host-buffer LPM_MODE_FP32C
 * sphere-BVE sum (lpm_bve_velocity, lpm_bve_set_velocity_from_vorticity; block-synchronous
 * tile pipeline) or sphere PSE sum (lpm_pse_sphere_laplacian, _gradient, _divergence;
 * warp-decoupled pipeline) does not issue the copy of source tile `skip_tile` and bounds its
 * waits by budget_ns (0 < budget_ns <= 1e9) instead of 1 s.  The waits for that tile run out, the call returns LPM_ERR_TIMEOUT with the
 * caller's outputs untouched, and the context stays usable.  Nothing faults: no copy is in
 * flight for the skipped tile.  One-shot. */
int lpm_debug_fail_device_alloc(int64_t k);
int lpm_debug_inject_wait_timeout(int64_t skip_tile, int64_t budget_ns);

/* ------------------------------------------------------------------ calibration */

/* Runs a fused multiply-add throughput loop on every SM for about `ms_target` ms and
 * returns the achieved FP32 rate in TFLOP/s (2 flops per FMA): the measured CUDA-core peak
 * that the direct-sum kernels are reported against. */
int lpm_measure_fp32_peak(double ms_target, double* tflops);

#ifdef __cplusplus
}
#endif
#endif
