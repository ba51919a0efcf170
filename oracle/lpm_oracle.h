/*
 * lpm_oracle.h -- CPU restatement of the lpm-v2 direct sums and RK4 steppers.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker, never the product: only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The shipped library (liblpm_gpu.so) neither links nor calls anything here.
 *
 * Every routine restates one reference loop with the reference's loop order and
 * expression association, in FP64, and is compiled with -ffp-contract=off so that
 * no multiply-add is fused (the association an x86-64 gfortran -O3 build of the
 * reference uses).  Arrays are 0-based; target ranges are half-open [ib, ie).
 *
 * Parity pins: the PSE Laplacian is pinned by the reference's regression
 * thresholds (tests/SpherePSEConvTest.f90:373-390); the BVE sum is pinned by the
 * solid-body known answer of examples/BVESolidBody.f90:231-243; the mesh inputs
 * by the counts and area invariants of tests/IcosTriMeshTester.f90:72-89.  The
 * reference ships no golden vectors for the BVE or planar sums and cannot be
 * built here (Fortran + MPI).  Parity unpinned: beyond the known answers, the BVE
 * and planar sums rest on this restatement alone.
 */
#ifndef LPM_ORACLE_H
#define LPM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* dot-product association of the BVE denominator */
enum { LPMO_ASSOC_SOLVER = 0, /* ((a*a - xi*xj) - yi*yj) - zi*zj : SphereBVESolver.f90:403 */
       LPMO_ASSOC_MESH = 1    /* a*a - sum(xi*xj)                : SphereBVE.f90:509      */ };

/* PSE kernel choice */
enum { LPMO_PSE_K8_GEODESIC = 0, /* PSESphereLaplacianAtParticles  PSEDirectSum.f90:502 */
       LPMO_PSE_GAUSS_CHORD = 1, /* Gaussian, chord distance (4/pi normalised)          */
       LPMO_PSE_K8_CHORD = 2     /* PSEPlaneLaplacianAtParticles   PSEDirectSum.f90:467 */ };

void lpmo_bve_velocity(int64_t n, const double* x, const double* y, const double* z,
                       const double* zeta, const double* area, const int32_t* active,
                       double radius, int assoc, int64_t ib, int64_t ie,
                       double* u, double* v, double* w, int nthreads);

void lpmo_plane_velocity(int64_t n, const double* x, const double* y,
                         const double* omega, const double* area, const int32_t* active,
                         double delta, int64_t ib, int64_t ie,
                         double* u, double* v, int nthreads);

void lpmo_pse_laplacian(int64_t n, const double* x, const double* y, const double* z,
                        const double* f, const double* area, const int32_t* active,
                        double eps, double radius, int kernel, int64_t ib, int64_t ie,
                        double* lap, int nthreads);

void lpmo_bve_stream(int64_t n, const double* x, const double* y, const double* z,
                     const double* relvort, const double* absvort, const double* area,
                     const int32_t* active, double radius, int64_t ib, int64_t ie,
                     double* psi_rel, double* psi_abs, int nthreads);

void lpmo_plane_stream(int64_t n, const double* x, const double* y,
                       const double* omega, const double* area, const int32_t* active,
                       int64_t ib, int64_t ie, double* psi, int nthreads);

/* One or more classical RK4 steps of SphereBVESolver.f90:219-353 (no stream function).
 * x,y,z,zeta are advanced in place; u,v,w hold the velocity at the start of the step on
 * entry (stage-1 reuse) and the velocity at the new positions on exit. */
void lpmo_bve_timestep(int64_t n, double* x, double* y, double* z, double* zeta,
                       const double* area, const int32_t* active, double* u, double* v,
                       double* w, double radius, double omega, double dt, int nsteps,
                       int nthreads);

/* PlaneIncompressibleSolver.f90:171-259 (vorticity is materially conserved). */
void lpmo_plane_timestep(int64_t n, double* x, double* y, const double* omega,
                         const double* area, const int32_t* active, double* u, double* v,
                         double delta, double dt, int nsteps, int nthreads);

/* SphereBVE.f90:410-441 and the circulation sum of examples/BVESingleGaussianVortex.f90:350 */
void lpmo_bve_diagnostics(int64_t n, const double* u, const double* v, const double* w,
                          const double* zeta, const double* area, const int32_t* active,
                          double* ke, double* enstrophy, double* circulation);

/* PSESphereGradientAtParticles, PSEDirectSum.f90:220-267 (gradient of f, 3 components) */
void lpmo_pse_sphere_gradient(int64_t n, const double* x, const double* y, const double* z,
                              const double* f, const double* area, const int32_t* active,
                              double eps, double radius, int64_t ib, int64_t ie, double* gx,
                              double* gy, double* gz, int nthreads);

/* PSESphereDivergenceAtParticles, PSEDirectSum.f90:537-579 (divergence of (vx, vy, vz)) */
void lpmo_pse_sphere_divergence(int64_t n, const double* x, const double* y, const double* z,
                                const double* vx, const double* vy, const double* vz,
                                const double* area, const int32_t* active, double eps,
                                double radius, int64_t ib, int64_t ie, double* div, int nthreads);

/* K8(r) of PSEDirectSum.f90:622-627, the first-derivative kernel K1 of :629-634 and the
 * delta kernel of :611-616 */
double lpmo_k8(double r);
double lpmo_k1(double r);
double lpmo_kdelta8(double r);

/* PSEPlaneGradientAtParticles, PSEDirectSum.f90:180-217 */
void lpmo_pse_plane_gradient(int64_t n, const double* x, const double* y, const double* f,
                             const double* area, const int32_t* active, double eps, int64_t ib,
                             int64_t ie, double* gx, double* gy, int nthreads);

/* PSEPlaneSecondPartialsAtParticles, PSEDirectSum.f90:269-320 (from the gradient field) */
void lpmo_pse_plane_second_partials(int64_t n, const double* x, const double* y, const double* gx,
                                    const double* gy, const double* area, const int32_t* active,
                                    double eps, int64_t ib, int64_t ie, double* dxx, double* dxy,
                                    double* dyy, int nthreads);

/* PSEPlaneDoubleDotProductAtParticles, PSEDirectSum.f90:322-365 */
void lpmo_pse_plane_double_dot(int64_t n, const double* x, const double* y, const double* u,
                               const double* v, const double* area, const int32_t* active, double eps,
                               int64_t ib, int64_t ie, double* ddot, int nthreads);

/* PSESphereDoubleDotProductAtParticles, PSEDirectSum.f90:367-418 */
void lpmo_pse_sphere_double_dot(int64_t n, const double* x, const double* y, const double* z,
                                const double* u, const double* v, const double* w, const double* area,
                                const int32_t* active, double eps, double radius, int64_t ib, int64_t ie,
                                double* ddot, int nthreads);

/* PSEPlaneInterpolateScalar (geometry 0) / PSESphereInterpolateScalar (geometry 1),
 * PSEDirectSum.f90:128-168, at m query points */
void lpmo_pse_interpolate(int64_t n, const double* x, const double* y, const double* z, const double* f,
                          const double* area, const int32_t* active, double eps, double radius, int geometry,
                          int64_t m, const double* qx, const double* qy, const double* qz, double* out,
                          int nthreads);

/* SWEPlaneRHSIntegrals, SWEPlaneSolver.f90:457-571 (sh = h + topoFn(x, y)) */
void lpmo_swe_plane_rhs(int64_t n, const double* x, const double* y, const double* vort, const double* div,
                        const double* sh, const double* area, const int32_t* active, double eps, int64_t ib,
                        int64_t ie, double* u, double* v, double* ddot, double* lap, int nthreads);

/* SWESphereRHSIntegrals, SphereSWESolver.f90:299-372 (sh = h + topoFn(x, y, z)) */
void lpmo_swe_sphere_rhs(int64_t n, const double* x, const double* y, const double* z, const double* relvort,
                         const double* div, const double* sh, const double* area, const int32_t* active,
                         double radius, double sphere_radius, double eps, int64_t ib, int64_t ie, double* u,
                         double* v, double* w, double* ddot, double* lap, int nthreads);

/* BetaPlaneVelocity, BetaPlaneSolver.f90:227-268 (x-periodic kernel, period 1) */
void lpmo_beta_plane_velocity(int64_t n, const double* x, const double* y, const double* zeta,
                              const double* area, const int32_t* active, int64_t ib, int64_t ie, double* u,
                              double* v, int nthreads);

/* SetStreamFunctionsOnMesh of the beta plane, BetaPlane.f90:399-442 */
void lpmo_beta_plane_stream(int64_t n, const double* x, const double* y, const double* relvort,
                            const double* absvort, const double* area, const int32_t* active, int64_t ib,
                            int64_t ie, double* psi_rel, double* psi_abs, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
