/*
 * lpm_oracle.c -- CPU restatement of the lpm-v2 direct sums (TEST INFRASTRUCTURE ONLY).
 *
 * The checker for the CUDA library: the tests compare the GPU results against these
 * loops, and the benchmark's CPU-baseline leg times them on the host cores.  Nothing in
 * the shipped library calls this file.  See lpm_oracle.h for what pins each routine
 * (the PSE Laplacian: the reference's regression thresholds; the BVE and planar sums:
 * parity unpinned beyond known answers, as the reference ships no golden vectors).
 *
 * Build: -O3 -fopenmp -ffp-contract=off (no fused multiply-add, so every product and
 * sum is rounded exactly where the Fortran source rounds it).
 */
#include "lpm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* NumberKindsModule PI, src/TypeDefs.f90:31 */
static const double PI = 3.1415926535897932384626433832795027975;

static int pick_threads(int nthreads)
{
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

/*
 * BVESphereVelocity, src/SphereBVESolver.f90:377-430 (assoc = SOLVER) and
 * setVelocityFromVorticity, src/SphereBVE.f90:489-531 (assoc = MESH).
 * j runs 1..i-1 then i+1..N (:401-419), i.e. ascending j skipping i; inactive j skipped.
 *   strength = -zeta_j A_j / (4 pi a (a^2 - x_i.x_j))
 *   u_i += (y_i z_j - z_i y_j) strength  etc.
 */
void lpmo_bve_velocity(int64_t n, const double* x, const double* y, const double* z,
                       const double* zeta, const double* area, const int32_t* active,
                       double radius, int assoc, int64_t ib, int64_t ie,
                       double* u, double* v, double* w, int nthreads)
{
  const double four_pi = 4.0 * PI; /* gfortran folds 4.0_kreal*PI at compile time */
  const double kden = four_pi * radius;
  const double a2 = radius * radius;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z[i];
    double ui = 0.0, vi = 0.0, wi = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      double den;
      if (assoc == LPMO_ASSOC_SOLVER) {
        den = ((a2 - xi * x[j]) - yi * y[j]) - zi * z[j];
      } else {
        den = a2 - ((xi * x[j] + yi * y[j]) + zi * z[j]);
      }
      const double strength = -((zeta[j] * area[j]) / (kden * den));
      ui = ui + (yi * z[j] - zi * y[j]) * strength;
      vi = vi + (zi * x[j] - xi * z[j]) * strength;
      wi = wi + (xi * y[j] - yi * x[j]) * strength;
    }
    u[i] = ui;
    v[i] = vi;
    w[i] = wi;
  }
}

/*
 * planarIncompressibleVelocity, src/PlaneIncompressibleSolver.f90:278-316.
 *   strength = omega_j A_j / (2 pi ((x_i-x_j)^2 + (y_i-y_j)^2 [+ delta^2]))
 *   u_i -= (y_i - y_j) strength ; v_i += (x_i - x_j) strength
 * delta = 0 is the reference (singular) kernel; adding +0.0 leaves every rounding as is.
 */
void lpmo_plane_velocity(int64_t n, const double* x, const double* y,
                         const double* omega, const double* area, const int32_t* active,
                         double delta, int64_t ib, int64_t ie,
                         double* u, double* v, int nthreads)
{
  const double two_pi = 2.0 * PI;
  const double d2 = delta * delta;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i];
    double ui = 0.0, vi = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      const double dx = xi - x[j];
      const double dy = yi - y[j];
      const double r2 = (dx * dx + dy * dy) + d2;
      const double strength = (omega[j] * area[j]) / (two_pi * r2);
      ui = ui - dy * strength;
      vi = vi + dx * strength;
    }
    u[i] = ui;
    v[i] = vi;
  }
}

/* bivariateLaplacianKernel8, src/PSEDirectSum.f90:622-627.  gfortran expands r**k with
 * its integer-power multiplication chain: r^2 = r*r, r^4 = r^2*r^2, r^6 = r^3*r^3 with
 * r^3 = r*r^2. */
double lpmo_k8(double r)
{
  const double r2 = r * r;
  const double r3 = r * r2;
  const double r4 = r2 * r2;
  const double r6 = r3 * r3;
  return (((40.0 - 40.0 * r2) + 10.0 * r4) - (2.0 * r6) / 3.0) * exp(-(r * r)) / PI;
}

/* SphereDistance (vector form), src/SphereGeometry.f90:107-125, SphereRadius = radius */
static double sphere_distance(double ax, double ay, double az, double bx, double by,
                              double bz, double radius)
{
  const double c1 = ay * bz - by * az;
  const double c2 = bx * az - ax * bz;
  const double c3 = ax * by - bx * ay;
  const double cn = sqrt((c1 * c1 + c2 * c2) + c3 * c3);
  const double dp = (ax * bx + ay * by) + az * bz;
  return atan2(cn, dp) * radius;
}

/* ChordDistance, src/SphereGeometry.f90:67-73: sqrt(sum((b-a)*(b-a))) */
static double chord_distance(double ax, double ay, double az, double bx, double by, double bz)
{
  const double d1 = bx - ax, d2 = by - ay, d3 = bz - az;
  return sqrt((d1 * d1 + d2 * d2) + d3 * d3);
}

/*
 * PSESphereLaplacianAtParticles, src/PSEDirectSum.f90:502-535 (kernel K8_GEODESIC) and
 * PSEPlaneLaplacianAtParticles, :467-500 (kernel K8_CHORD).  j runs over all active
 * particles including j = i (that term is 0).  Per pair:
 *   lap_i += (f_j - f_i) * K8(d/eps) / eps**2 * A_j
 * and the finished field is multiplied by 1/eps**2 (:534).
 * GAUSS_CHORD uses eta(r) = 4 exp(-r^2)/pi in place of K8 with the chord distance: the
 * second-order Gaussian PSE Laplacian (the factor 4 makes (1/eps^2) sum (f_j-f_i)
 * eta(|x_i-x_j|/eps)/eps^2 A_j consistent with the Laplacian).
 */
void lpmo_pse_laplacian(int64_t n, const double* x, const double* y, const double* z,
                        const double* f, const double* area, const int32_t* active,
                        double eps, double radius, int kernel, int64_t ib, int64_t ie,
                        double* lap, int nthreads)
{
  const double eps2 = eps * eps; /* eps**2 */
  const double scale = 1.0 / eps2;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z ? z[i] : 0.0;
    double li = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double xj = x[j], yj = y[j], zj = z ? z[j] : 0.0;
      double k;
      if (kernel == LPMO_PSE_K8_GEODESIC) {
        const double kin = sphere_distance(xi, yi, zi, xj, yj, zj, radius) / eps;
        k = lpmo_k8(kin);
      } else if (kernel == LPMO_PSE_K8_CHORD) {
        const double kin = chord_distance(xi, yi, zi, xj, yj, zj) / eps;
        k = lpmo_k8(kin);
      } else {
        const double kin = chord_distance(xi, yi, zi, xj, yj, zj) / eps;
        k = 4.0 * exp(-(kin * kin)) / PI;
      }
      li = li + (((f[j] - f[i]) * k) / eps2) * area[j];
    }
    lap[i] = li * scale; /* MultiplyFieldByScalar(scalarLap, 1/eps**2) */
  }
}

/* bivariateFirstDerivativeKernel8, src/PSEDirectSum.f90:629-634, with the power chain of
 * lpmo_k8. */
double lpmo_k1(double r)
{
  const double r2 = r * r;
  const double r3 = r * r2;
  const double r4 = r2 * r2;
  const double r6 = r3 * r3;
  return (((-20.0 + 20.0 * r2) - 5.0 * r4) + r6 / 3.0) * exp(-(r * r)) / PI;
}

/* MATMUL(SphereProjection(x), g) (SphereGeometry.f90:578-590): (I - x x^T) g, each row
 * summed left to right. */
static void sphere_project(double xi, double yi, double zi, const double g[3], double out[3])
{
  const double p11 = 1.0 - xi * xi, p21 = -(yi * xi), p31 = -(zi * xi);
  const double p12 = -(xi * yi), p22 = 1.0 - yi * yi, p32 = -(zi * yi);
  const double p13 = -(xi * zi), p23 = -(yi * zi), p33 = 1.0 - zi * zi;
  out[0] = (p11 * g[0] + p12 * g[1]) + p13 * g[2];
  out[1] = (p21 * g[0] + p22 * g[1]) + p23 * g[2];
  out[2] = (p31 * g[0] + p32 * g[1]) + p33 * g[2];
}

/*
 * PSESphereGradientAtParticles, src/PSEDirectSum.f90:220-267: for every active j
 *   grad += (f_j + f_i) (x_i - x_j) K1(SphereDistance(x_j, x_i)/eps) / eps**2 A_j,
 * then grad = MATMUL(SphereProjection(x_i), grad) and the field is multiplied by 1/eps**2.
 */
void lpmo_pse_sphere_gradient(int64_t n, const double* x, const double* y, const double* z,
                              const double* f, const double* area, const int32_t* active,
                              double eps, double radius, int64_t ib, int64_t ie, double* gx,
                              double* gy, double* gz, int nthreads)
{
  const double eps2 = eps * eps;
  const double scale = 1.0 / eps2;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z[i];
    double g[3] = {0.0, 0.0, 0.0};
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double kin = sphere_distance(x[j], y[j], z[j], xi, yi, zi, radius) / eps;
      const double kout = lpmo_k1(kin) / eps2;
      const double fs = f[j] + f[i];
      g[0] = g[0] + ((fs * (xi - x[j])) * kout) * area[j];
      g[1] = g[1] + ((fs * (yi - y[j])) * kout) * area[j];
      g[2] = g[2] + ((fs * (zi - z[j])) * kout) * area[j];
    }
    double pg[3];
    sphere_project(xi, yi, zi, g, pg);
    gx[i] = pg[0] * scale;
    gy[i] = pg[1] * scale;
    gz[i] = pg[2] * scale;
  }
}

/*
 * PSESphereDivergenceAtParticles, src/PSEDirectSum.f90:537-579: for every active j
 *   g = MATMUL(SphereProjection(x_i), (x_i - x_j) K1(SphereDistance(x_j, x_i)/eps) / eps**3),
 *   div += (g . (V_j + V_i)) A_j,
 * and the field is multiplied by 1/eps.
 */
void lpmo_pse_sphere_divergence(int64_t n, const double* x, const double* y, const double* z,
                                const double* vx, const double* vy, const double* vz,
                                const double* area, const int32_t* active, double eps,
                                double radius, int64_t ib, int64_t ie, double* div, int nthreads)
{
  const double denom = eps * (eps * eps); /* eps**3 */
  const double scale = 1.0 / eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z[i];
    double d = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double kin = sphere_distance(x[j], y[j], z[j], xi, yi, zi, radius) / eps;
      const double k1 = lpmo_k1(kin);
      const double g[3] = {((xi - x[j]) * k1) / denom, ((yi - y[j]) * k1) / denom,
                           ((zi - z[j]) * k1) / denom};
      double h[3];
      sphere_project(xi, yi, zi, g, h);
      d = d + (((h[0] * (vx[j] + vx[i]) + h[1] * (vy[j] + vy[i])) + h[2] * (vz[j] + vz[i])) *
               area[j]);
    }
    div[i] = d * scale;
  }
}

/*
 * SetStreamFunctionsOnMesh, src/SphereBVE.f90:445-485: G = -log(a^2 - sum(xi*xj))/(4 pi),
 * psi_rel += G zeta_rel_j A_j, psi_abs += G zeta_abs_j A_j, j != i, active j.
 */
void lpmo_bve_stream(int64_t n, const double* x, const double* y, const double* z,
                     const double* relvort, const double* absvort, const double* area,
                     const int32_t* active, double radius, int64_t ib, int64_t ie,
                     double* psi_rel, double* psi_abs, int nthreads)
{
  const double four_pi = 4.0 * PI;
  const double a2 = radius * radius;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z[i];
    double pr = 0.0, pa = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      const double g = -log(a2 - ((xi * x[j] + yi * y[j]) + zi * z[j])) / four_pi;
      pr = pr + (g * relvort[j]) * area[j];
      pa = pa + (g * absvort[j]) * area[j];
    }
    psi_rel[i] = pr;
    psi_abs[i] = pa;
  }
}

/* SetStreamFunctionOnMesh, src/PlanarIncompressible.f90:470-505:
 * G = log(sqrt((xi-xj)^2 + (yi-yj)^2)) / (2 pi). */
void lpmo_plane_stream(int64_t n, const double* x, const double* y,
                       const double* omega, const double* area, const int32_t* active,
                       int64_t ib, int64_t ie, double* psi, int nthreads)
{
  const double two_pi = 2.0 * PI;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i];
    double p = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      const double dx = xi - x[j], dy = yi - y[j];
      const double g = log(sqrt(dx * dx + dy * dy)) / two_pi;
      p = p + (g * omega[j]) * area[j];
    }
    psi[i] = p;
  }
}

/*
 * timestepPrivate, src/SphereBVESolver.f90:219-353, without the stream-function call
 * at :352 (its result is not part of the RK4 state).
 */
void lpmo_bve_timestep(int64_t n, double* x, double* y, double* z, double* zeta,
                       const double* area, const int32_t* active, double* u, double* v,
                       double* w, double radius, double omega, double dt, int nsteps,
                       int nthreads)
{
  const size_t bytes = (size_t)n * sizeof(double);
  double* buf = (double*)malloc(bytes * 20);
  double *x1 = buf, *y1 = buf + n, *z1 = buf + 2 * n, *q1 = buf + 3 * n;
  double *x2 = buf + 4 * n, *y2 = buf + 5 * n, *z2 = buf + 6 * n, *q2 = buf + 7 * n;
  double *x3 = buf + 8 * n, *y3 = buf + 9 * n, *z3 = buf + 10 * n, *q3 = buf + 11 * n;
  double *x4 = buf + 12 * n, *y4 = buf + 13 * n, *z4 = buf + 14 * n, *q4 = buf + 15 * n;
  double *xin = buf + 16 * n, *yin = buf + 17 * n, *zin = buf + 18 * n, *qin = buf + 19 * n;
  for (int s = 0; s < nsteps; ++s) {
    /* stage 1 (:238-244): k1 = dt * u_prev */
    for (int64_t i = 0; i < n; ++i) {
      x1[i] = dt * u[i];
      y1[i] = dt * v[i];
      z1[i] = dt * w[i];
      q1[i] = -((((dt * 2.0) * omega) * w[i]) / radius);
    }
    /* stages 2-4 (:249-313) */
    double* ks[3][4] = {{x1, y1, z1, q1}, {x2, y2, z2, q2}, {x3, y3, z3, q3}};
    double* kout[3][4] = {{x2, y2, z2, q2}, {x3, y3, z3, q3}, {x4, y4, z4, q4}};
    for (int st = 0; st < 3; ++st) {
      double** kp = ks[st];
      double** ko = kout[st];
      for (int64_t i = 0; i < n; ++i) {
        if (st < 2) {
          xin[i] = x[i] + 0.5 * kp[0][i];
          yin[i] = y[i] + 0.5 * kp[1][i];
          zin[i] = z[i] + 0.5 * kp[2][i];
          qin[i] = zeta[i] + 0.5 * kp[3][i];
        } else {
          xin[i] = x[i] + kp[0][i];
          yin[i] = y[i] + kp[1][i];
          zin[i] = z[i] + kp[2][i];
          qin[i] = zeta[i] + kp[3][i];
        }
      }
      lpmo_bve_velocity(n, xin, yin, zin, qin, area, active, radius, LPMO_ASSOC_SOLVER, 0, n,
                        ko[0], ko[1], ko[2], nthreads);
      for (int64_t i = 0; i < n; ++i) {
        ko[3][i] = -((((dt * 2.0) * omega) * ko[2][i]) / radius);
        ko[0][i] = dt * ko[0][i];
        ko[1][i] = dt * ko[1][i];
        ko[2][i] = dt * ko[2][i];
      }
    }
    /* RK4 update (:319-329) */
    for (int64_t i = 0; i < n; ++i) {
      x[i] = (((x[i] + x1[i] / 6.0) + x2[i] / 3.0) + x3[i] / 3.0) + x4[i] / 6.0;
      y[i] = (((y[i] + y1[i] / 6.0) + y2[i] / 3.0) + y3[i] / 3.0) + y4[i] / 6.0;
      z[i] = (((z[i] + z1[i] / 6.0) + z2[i] / 3.0) + z3[i] / 3.0) + z4[i] / 6.0;
      zeta[i] = (((zeta[i] + q1[i] / 6.0) + q2[i] / 3.0) + q3[i] / 3.0) + q4[i] / 6.0;
    }
    /* velocity at the new positions (:345-350) */
    lpmo_bve_velocity(n, x, y, z, zeta, area, active, radius, LPMO_ASSOC_SOLVER, 0, n, u, v,
                      w, nthreads);
  }
  free(buf);
}

/* timestepPrivate, src/PlaneIncompressibleSolver.f90:171-259 (without the stream function). */
void lpmo_plane_timestep(int64_t n, double* x, double* y, const double* omega,
                         const double* area, const int32_t* active, double* u, double* v,
                         double delta, double dt, int nsteps, int nthreads)
{
  const size_t bytes = (size_t)n * sizeof(double);
  double* buf = (double*)malloc(bytes * 10);
  double *x1 = buf, *y1 = buf + n, *x2 = buf + 2 * n, *y2 = buf + 3 * n;
  double *x3 = buf + 4 * n, *y3 = buf + 5 * n, *x4 = buf + 6 * n, *y4 = buf + 7 * n;
  double *xin = buf + 8 * n, *yin = buf + 9 * n;
  for (int s = 0; s < nsteps; ++s) {
    for (int64_t i = 0; i < n; ++i) {
      x1[i] = dt * u[i];
      y1[i] = dt * v[i];
    }
    double* kp[3][2] = {{x1, y1}, {x2, y2}, {x3, y3}};
    double* ko[3][2] = {{x2, y2}, {x3, y3}, {x4, y4}};
    for (int st = 0; st < 3; ++st) {
      for (int64_t i = 0; i < n; ++i) {
        if (st < 2) {
          xin[i] = x[i] + 0.5 * kp[st][0][i];
          yin[i] = y[i] + 0.5 * kp[st][1][i];
        } else {
          xin[i] = x[i] + kp[st][0][i];
          yin[i] = y[i] + kp[st][1][i];
        }
      }
      lpmo_plane_velocity(n, xin, yin, omega, area, active, delta, 0, n, ko[st][0], ko[st][1],
                          nthreads);
      for (int64_t i = 0; i < n; ++i) {
        ko[st][0][i] = dt * ko[st][0][i];
        ko[st][1][i] = dt * ko[st][1][i];
      }
    }
    for (int64_t i = 0; i < n; ++i) {
      x[i] = (((x[i] + x1[i] / 6.0) + x2[i] / 3.0) + x3[i] / 3.0) + x4[i] / 6.0;
      y[i] = (((y[i] + y1[i] / 6.0) + y2[i] / 3.0) + y3[i] / 3.0) + y4[i] / 6.0;
    }
    lpmo_plane_velocity(n, x, y, omega, area, active, delta, 0, n, u, v, nthreads);
  }
  free(buf);
}

/* TotalKE / TotalEnstrophy, src/SphereBVE.f90:410-441; circulation = sum zeta A over
 * active particles (SetGaussConst numerator, examples/BVESingleGaussianVortex.f90:350). */
void lpmo_bve_diagnostics(int64_t n, const double* u, const double* v, const double* w,
                          const double* zeta, const double* area, const int32_t* active,
                          double* ke, double* enstrophy, double* circulation)
{
  double k = 0.0, e = 0.0, c = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    if (!active[i]) continue;
    const double m2 = (u[i] * u[i] + v[i] * v[i]) + (w ? w[i] * w[i] : 0.0);
    k = k + m2 * area[i];
    e = e + (zeta[i] * zeta[i]) * area[i];
    c = c + zeta[i] * area[i];
  }
  *ke = 0.5 * k;
  *enstrophy = 0.5 * e;
  *circulation = c;
}

/* bivariateDeltaKernel8, src/PSEDirectSum.f90:611-616, with the power chain of lpmo_k8. */
double lpmo_kdelta8(double r)
{
  const double r2 = r * r;
  const double r3 = r * r2;
  const double r4 = r2 * r2;
  const double r6 = r3 * r3;
  return (((4.0 - 6.0 * r2) + 2.0 * r4) - r6 / 6.0) * exp(-(r * r)) / PI;
}

/*
 * PSEPlaneGradientAtParticles, src/PSEDirectSum.f90:180-217 (planar particles, z = 0): for
 * every active j
 *   grad += (f_j + f_i) (x_i - x_j) K1(ChordDistance(x_i, x_j)/eps) / eps**3 * A_j
 * and the field is multiplied by 1/eps.
 */
void lpmo_pse_plane_gradient(int64_t n, const double* x, const double* y, const double* f,
                             const double* area, const int32_t* active, double eps, int64_t ib,
                             int64_t ie, double* gx, double* gy, int nthreads)
{
  const double eps3 = eps * (eps * eps);
  const double scale = 1.0 / eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double ax = 0.0, ay = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double kin = chord_distance(x[i], y[i], 0.0, x[j], y[j], 0.0) / eps;
      const double k1 = lpmo_k1(kin);
      const double fs = f[j] + f[i];
      ax = ax + (((fs * (x[i] - x[j])) * k1) / eps3) * area[j];
      ay = ay + (((fs * (y[i] - y[j])) * k1) / eps3) * area[j];
    }
    gx[i] = scale * ax;
    gy[i] = scale * ay;
  }
}

/* The four planar first-derivative sums shared by the second partials and the double dot
 * product, src/PSEDirectSum.f90:286-301 and :339-354:
 *   s_ab += (a_j + a_i) (x_b,i - x_b,j) / eps * K1(chord/eps) / eps**2 * A_j. */
static void plane_d4(int64_t n, const double* x, const double* y, const double* a, const double* b,
                     const double* area, const int32_t* active, double eps, int64_t i, double s[4])
{
  const double eps2 = eps * eps;
  double ax = 0.0, ay = 0.0, bx = 0.0, by = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    if (!active[j]) continue;
    const double kin = chord_distance(x[i], y[i], 0.0, x[j], y[j], 0.0) / eps;
    const double kout = lpmo_k1(kin) / eps2;
    const double dx = x[i] - x[j], dy = y[i] - y[j];
    ax = ax + ((((a[j] + a[i]) * dx) / eps) * kout) * area[j];
    ay = ay + ((((a[j] + a[i]) * dy) / eps) * kout) * area[j];
    bx = bx + ((((b[j] + b[i]) * dx) / eps) * kout) * area[j];
    by = by + ((((b[j] + b[i]) * dy) / eps) * kout) * area[j];
  }
  s[0] = ax;
  s[1] = ay;
  s[2] = bx;
  s[3] = by;
}

/*
 * PSEPlaneSecondPartialsAtParticles, src/PSEDirectSum.f90:269-320, from the gradient field
 * (gx, gy): xx = dxx, xy = 0.5 (dxy + dyx), yy = dyy, each multiplied by 1/eps.
 */
void lpmo_pse_plane_second_partials(int64_t n, const double* x, const double* y, const double* gx,
                                    const double* gy, const double* area, const int32_t* active,
                                    double eps, int64_t ib, int64_t ie, double* dxx, double* dxy,
                                    double* dyy, int nthreads)
{
  const double scale = 1.0 / eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double s[4];
    plane_d4(n, x, y, gx, gy, area, active, eps, i, s);
    dxx[i] = scale * s[0];
    dxy[i] = scale * (0.5 * (s[1] + s[2]));
    dyy[i] = scale * s[3];
  }
}

/* PSEPlaneDoubleDotProductAtParticles, src/PSEDirectSum.f90:322-365:
 * (ux ux + 2 uy vx + vy vy) / eps**2 of the velocity (u, v). */
void lpmo_pse_plane_double_dot(int64_t n, const double* x, const double* y, const double* u,
                               const double* v, const double* area, const int32_t* active, double eps,
                               int64_t ib, int64_t ie, double* ddot, int nthreads)
{
  const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double s[4];
    plane_d4(n, x, y, u, v, area, active, eps, i, s);
    ddot[i] = ((s[0] * s[0] + (2.0 * s[1]) * s[2]) + s[3] * s[3]) / eps2;
  }
}

/*
 * PSESphereDoubleDotProductAtParticles, src/PSEDirectSum.f90:367-418: nine first-derivative
 * sums with K1(SphereDistance(x_i, x_j)/eps) / eps**2.  As in the reference, the third row
 * pairs w_j with v_i: (w_j + v_i) (:399-404).  Result (ux ux + vy vy + wz wz + 2 (uy vx +
 * uz wx + vz wy)) / eps**2.
 */
void lpmo_pse_sphere_double_dot(int64_t n, const double* x, const double* y, const double* z,
                                const double* u, const double* v, const double* w, const double* area,
                                const int32_t* active, double eps, double radius, int64_t ib, int64_t ie,
                                double* ddot, int nthreads)
{
  const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double ux = 0.0, uy = 0.0, uz = 0.0, vx = 0.0, vy = 0.0, vz = 0.0, wx = 0.0, wy = 0.0, wz = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double kin = sphere_distance(x[i], y[i], z[i], x[j], y[j], z[j], radius) / eps;
      const double kout = lpmo_k1(kin) / eps2;
      const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
      const double su = u[j] + u[i], sv = v[j] + v[i], sw = w[j] + v[i];
      ux = ux + (((su * dx) / eps) * kout) * area[j];
      uy = uy + (((su * dy) / eps) * kout) * area[j];
      uz = uz + (((su * dz) / eps) * kout) * area[j];
      vx = vx + (((sv * dx) / eps) * kout) * area[j];
      vy = vy + (((sv * dy) / eps) * kout) * area[j];
      vz = vz + (((sv * dz) / eps) * kout) * area[j];
      wx = wx + (((sw * dx) / eps) * kout) * area[j];
      wy = wy + (((sw * dy) / eps) * kout) * area[j];
      wz = wz + (((sw * dz) / eps) * kout) * area[j];
    }
    ddot[i] = (((ux * ux + vy * vy) + wz * wz) + 2.0 * ((uy * vx + uz * wx) + vz * wy)) / eps2;
  }
}

/*
 * PSEPlaneInterpolateScalar / PSESphereInterpolateScalar, src/PSEDirectSum.f90:128-168, at m
 * query points q: sum over active j of f_j A_j Kdelta8(dist(q, x_j)/eps) / eps**2, with the
 * chord distance (geometry 0) or the great-circle distance times radius (geometry 1).
 */
void lpmo_pse_interpolate(int64_t n, const double* x, const double* y, const double* z, const double* f,
                          const double* area, const int32_t* active, double eps, double radius, int geometry,
                          int64_t m, const double* qx, const double* qy, const double* qz, double* out,
                          int nthreads)
{
  const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t k = 0; k < m; ++k) {
    const double q0 = qx[k], q1 = qy[k], q2 = qz ? qz[k] : 0.0;
    double s = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double zj = z ? z[j] : 0.0;
      const double d = geometry == 1 ? sphere_distance(x[j], y[j], zj, q0, q1, q2, radius)
                                     : chord_distance(q0, q1, q2, x[j], y[j], zj);
      s = s + ((f[j] * area[j]) * lpmo_kdelta8(d / eps)) / eps2;
    }
    out[k] = s;
  }
}

/*
 * SWEPlaneRHSIntegrals, src/SWEPlaneSolver.f90:457-571, with the surface height
 * sh = h + topoFn(x, y) evaluated by the caller.  Per active j:
 *   lapSurf += K8(r/eps)/eps**2 (sh_j - sh_i) A_j      (j = i included: a zero term)
 * and for j != i, with r^2 = dx^2 + dy^2, denom = 2 pi r^2, denom2 = pi r^4,
 *   rot = vort_j A_j / denom, pot = div_j A_j / denom,
 *   u += -dy rot + dx pot,  v += dx rot + dy pot,
 *   ux += pot - dx (dx div_j - dy vort_j) A_j / denom2,  uy += -rot - dy (dx div_j - dy vort_j) A_j / denom2,
 *   vx += rot - dx (dy div_j + dx vort_j) A_j / denom2,  vy += pot - dy (dy div_j + dx vort_j) A_j / denom2;
 * then lapSurf /= eps**2 and doubleDot = ux ux + 2 uy vx + vy vy.
 */
void lpmo_swe_plane_rhs(int64_t n, const double* x, const double* y, const double* vort, const double* div,
                        const double* sh, const double* area, const int32_t* active, double eps, int64_t ib,
                        int64_t ie, double* u, double* v, double* ddot, double* lap, int nthreads)
{
  const double eps2 = eps * eps;
  const double two_pi = 2.0 * PI;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double ui = 0.0, vi = 0.0, li = 0.0, ux = 0.0, uy = 0.0, vx = 0.0, vy = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double dx = x[i] - x[j], dy = y[i] - y[j];
      const double sq = dx * dx + dy * dy;
      const double denom = two_pi * sq;
      const double denom2 = (PI * sq) * sq;
      const double rot = (vort[j] * area[j]) / denom;
      const double pot = (div[j] * area[j]) / denom;
      const double lk = lpmo_k8(sqrt(sq) / eps) / eps2;
      li = li + (lk * (sh[j] - sh[i])) * area[j];
      if (j == i) continue;
      ui = (ui - dy * rot) + dx * pot;
      vi = (vi + dx * rot) + dy * pot;
      const double cu = dx * div[j] - dy * vort[j];
      const double cv = dy * div[j] + dx * vort[j];
      ux = (ux + pot) - ((dx * cu) * area[j]) / denom2;
      uy = (uy - rot) - ((dy * cu) * area[j]) / denom2;
      vx = (vx + rot) - ((dx * cv) * area[j]) / denom2;
      vy = (vy + pot) - ((dy * cv) * area[j]) / denom2;
    }
    u[i] = ui;
    v[i] = vi;
    lap[i] = li / eps2;
    ddot[i] = (ux * ux + (2.0 * uy) * vx) + vy * vy;
  }
}

/*
 * SWESphereRHSIntegrals, src/SphereSWESolver.f90:299-372, with sh = h + topoFn(x, y, z) from
 * the caller.  Per active j:
 *   lapSurf += K8(SphereDistance(x_i, x_j)/eps)/eps**2 (sh_j - sh_i) A_j   (j = i included)
 * (SphereDistance scales by the module's SphereRadius, `sphere_radius` here), and for j != i,
 * with denom = 4 pi a^2 (a^2 - x_i.x_j):
 *   rot = zeta_j A_j / denom, pot = a div_j A_j / denom,
 *   u -= (y_i z_j - z_i y_j) rot + x_j pot (and cyclically for v, w).
 * As in the reference, doubleDot stays 0 and lapSurf is not divided again by eps**2.
 */
void lpmo_swe_sphere_rhs(int64_t n, const double* x, const double* y, const double* z, const double* relvort,
                         const double* div, const double* sh, const double* area, const int32_t* active,
                         double radius, double sphere_radius, double eps, int64_t ib, int64_t ie, double* u,
                         double* v, double* w, double* ddot, double* lap, int nthreads)
{
  const double eps2 = eps * eps;
  const double four_pi_r2 = ((4.0 * PI) * radius) * radius;
  const double a2 = radius * radius;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    const double xi = x[i], yi = y[i], zi = z[i];
    double ui = 0.0, vi = 0.0, wi = 0.0, li = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (!active[j]) continue;
      const double kin = sphere_distance(xi, yi, zi, x[j], y[j], z[j], sphere_radius) / eps;
      const double lk = lpmo_k8(kin) / eps2;
      li = li + (lk * (sh[j] - sh[i])) * area[j];
      if (j == i) continue;
      const double dp = (xi * x[j] + yi * y[j]) + zi * z[j];
      const double denom = four_pi_r2 * (a2 - dp);
      const double rot = (relvort[j] * area[j]) / denom;
      const double pot = ((radius * div[j]) * area[j]) / denom;
      ui = (ui - (yi * z[j] - zi * y[j]) * rot) - x[j] * pot;
      vi = (vi - (zi * x[j] - xi * z[j]) * rot) - y[j] * pot;
      wi = (wi - (xi * y[j] - yi * x[j]) * rot) - z[j] * pot;
    }
    u[i] = ui;
    v[i] = vi;
    w[i] = wi;
    lap[i] = li;
    ddot[i] = 0.0;
  }
}

/*
 * BetaPlaneVelocity, src/BetaPlaneSolver.f90:227-268 (and the same sum in
 * setVelocityFromVorticity, src/BetaPlane.f90:359-397): the x-periodic (period 1) point-vortex
 * kernel.  Per active j != i, in ascending j:
 *   strength = 0.5 zeta_j A_j / (cosh(2 pi dy) - cos(2 pi dx)),
 *   u -= sinh(2 pi dy) strength,  v += sin(2 pi dx) strength,   dx = x_i - x_j, dy = y_i - y_j.
 */
void lpmo_beta_plane_velocity(int64_t n, const double* x, const double* y, const double* zeta,
                              const double* area, const int32_t* active, int64_t ib, int64_t ie, double* u,
                              double* v, int nthreads)
{
  const double two_pi = 2.0 * PI;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double ui = 0.0, vi = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      const double ay = two_pi * (y[i] - y[j]), ax = two_pi * (x[i] - x[j]);
      const double s = ((0.5 * zeta[j]) * area[j]) / (cosh(ay) - cos(ax));
      ui = ui - sinh(ay) * s;
      vi = vi + sin(ax) * s;
    }
    u[i] = ui;
    v[i] = vi;
  }
}

/*
 * SetStreamFunctionsOnMesh of the beta plane, src/BetaPlane.f90:399-442:
 *   G = log(cosh(2 pi dy) - cos(2 pi dx)) / (4 pi),  psi_rel += G zeta_rel_j A_j,
 *   psi_abs += G zeta_abs_j A_j,  j != i, active.
 */
void lpmo_beta_plane_stream(int64_t n, const double* x, const double* y, const double* relvort,
                            const double* absvort, const double* area, const int32_t* active, int64_t ib,
                            int64_t ie, double* psi_rel, double* psi_abs, int nthreads)
{
  const double two_pi = 2.0 * PI, four_pi = 4.0 * PI;
#pragma omp parallel for schedule(dynamic, 16) num_threads(pick_threads(nthreads))
  for (int64_t i = ib; i < ie; ++i) {
    double pr = 0.0, pa = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i || !active[j]) continue;
      const double g = log(cosh(two_pi * (y[i] - y[j])) - cos(two_pi * (x[i] - x[j]))) / four_pi;
      pr = pr + (g * relvort[j]) * area[j];
      pa = pa + (g * absvort[j]) * area[j];
    }
    psi_rel[i] = pr;
    psi_abs[i] = pa;
  }
}
