// ops.cuh -- pair operators of the direct sums, FP64 (reference association) and FP32C.
//
// The FP32C pieces here (BveF32's target split, BetaF32's direct pair form) are called by
// the group-relative sweeps (bve_rel.cuh, stream_rel.cuh, beta_rel.cuh), whose prep kernels
// build the records from the particle arrays.  Each FP64 operator restates one Fortran loop body with explicit round-to-nearest intrinsics so
// that nvcc cannot fuse a multiply into an add: every intermediate rounds exactly where
// the Fortran rounds it.
#pragma once

#include "lpm_common.cuh"

namespace lpm {

// hi/lo split of a double: hi = fl32(v), lo = fl32(v - hi); hi + lo carries ~48 bits.
__device__ __forceinline__ void split2(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - static_cast<double>(hi));
}

// ============================================================ sphere BVE velocity
// Reference: BVESphereVelocity, src/SphereBVESolver.f90:395-420.
//
// FP32C form.  With unit-scaled positions p = x/a, d = p_i - p_j and c = |p|^2 - 1,
//   a^2 - x_i.x_j = a^2 (|d|^2 - c_i - c_j) / 2      (exact identity, no cancellation)
//   x_i x x_j     = a^2 (d x p_i)
// so u_i = [ sum_j S_j d / (|d|^2 - c_i - c_j) ] x p_i with S_j = -zeta_j A_j / (2 pi a).
// The cross product leaves the sum.  BveF32 holds the target side of the FP32C sweeps
// (bve_rel.cuh, and bve_x2.cuh for the allocation-free entry point).
struct BveF32 {
  static constexpr int NC = 3;
  struct __align__(16) Rec {
    float4 a;  // p_hi.x, p_hi.y, p_hi.z, -c
    float4 b;  // S, p_lo.x, p_lo.y, p_lo.z
  };
  struct Tgt {
    float xh, yh, zh, xl, yl, zl, nc;
  };
  struct Params {
    const double *x, *y, *z;
    double inv_a;
  };
  // -c_i is offset by 2^-100 so that a self pair (d = 0) on an exactly normalised particle
  // gives a finite weight times d = 0 instead of inf * 0.  |c| is either 0 or >= 2^-54, so
  // the offset never changes a nonzero c.
  __device__ static Tgt load_target(const Params& p, int64_t i) {
    Tgt t;
    const double px = p.x[i] * p.inv_a, py = p.y[i] * p.inv_a, pz = p.z[i] * p.inv_a;
    split2(px, t.xh, t.xl);
    split2(py, t.yh, t.yl);
    split2(pz, t.zh, t.zl);
    const double c = fma(px, px, fma(py, py, fma(pz, pz, -1.0)));
    t.nc = __double2float_rn(-c) + 7.888609052210118e-31f;  // + 2^-100
    return t;
  }
};

// FP64 source record shared by the sphere sums: position, q = zeta*A (or f and A for PSE)
struct __align__(16) Rec64 {
  double x, y, z, q;
  double r;       // second scalar (area for PSE, absolute vorticity for the stream function)
  long long idx;  // particle index (self-interaction test)
};

struct BveF64Params {
  const double *x, *y, *z;
  double a2, kden;  // a*a and fl(fl(4 pi) a)
  double *u, *v, *w;
};

// ASSOC 0: ((a^2 - xi xj) - yi yj) - zi zj   (SphereBVESolver.f90:403-404)
// ASSOC 1: a^2 - ((xi xj + yi yj) + zi zj)   (SphereBVE.f90:509, sum(xi*xj))
template <int ASSOC>
struct BveF64 {
  struct Tgt {
    double x, y, z;
  };
  struct Acc {
    double u, v, w;
  };
  __device__ static Tgt load(const BveF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.z[i]}; }
  __device__ static __forceinline__ void interact(const BveF64Params& p, const Tgt& t,
                                                  const Rec64& r, Acc& a) {
    double den;
    if (ASSOC == 0) {
      den = __dsub_rn(__dsub_rn(__dsub_rn(p.a2, __dmul_rn(t.x, r.x)), __dmul_rn(t.y, r.y)),
                      __dmul_rn(t.z, r.z));
    } else {
      den = __dsub_rn(p.a2, __dadd_rn(__dadd_rn(__dmul_rn(t.x, r.x), __dmul_rn(t.y, r.y)),
                                      __dmul_rn(t.z, r.z)));
    }
    const double s = -__ddiv_rn(r.q, __dmul_rn(p.kden, den));
    a.u = __dadd_rn(a.u, __dmul_rn(__dsub_rn(__dmul_rn(t.y, r.z), __dmul_rn(t.z, r.y)), s));
    a.v = __dadd_rn(a.v, __dmul_rn(__dsub_rn(__dmul_rn(t.z, r.x), __dmul_rn(t.x, r.z)), s));
    a.w = __dadd_rn(a.w, __dmul_rn(__dsub_rn(__dmul_rn(t.x, r.y), __dmul_rn(t.y, r.x)), s));
  }
  __device__ static void store(const BveF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.u[il] = a.u;
    p.v[il] = a.v;
    p.w[il] = a.w;
  }
  static constexpr bool kSkipSelf = true;
};

// ============================================================ planar velocity
// Reference: planarIncompressibleVelocity, src/PlaneIncompressibleSolver.f90:291-308.
// (The FP32C form is plane_rel.cuh.)
struct __align__(16) RecPlane64 {
  double x, y, q;
  long long idx;
};

struct PlaneF64Params {
  const double *x, *y;
  double two_pi, d2;
  double *u, *v;
};

struct PlaneF64 {
  struct Tgt {
    double x, y;
  };
  struct Acc {
    double u, v;
  };
  __device__ static Tgt load(const PlaneF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i]}; }
  __device__ static __forceinline__ void interact(const PlaneF64Params& p, const Tgt& t,
                                                  const RecPlane64& r, Acc& a) {
    const double dx = __dsub_rn(t.x, r.x);
    const double dy = __dsub_rn(t.y, r.y);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), p.d2);
    const double s = __ddiv_rn(r.q, __dmul_rn(p.two_pi, r2));
    a.u = __dsub_rn(a.u, __dmul_rn(dy, s));
    a.v = __dadd_rn(a.v, __dmul_rn(dx, s));
  }
  __device__ static void store(const PlaneF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.u[il] = a.u;
    p.v[il] = a.v;
  }
  static constexpr bool kSkipSelf = true;
};

// ============================================================ PSE Laplacian
// Reference: PSESphereLaplacianAtParticles / PSEPlaneLaplacianAtParticles,
// src/PSEDirectSum.f90:467-535, kernel bivariateLaplacianKernel8 (:622-627).
// KIND 0: K8 of the great-circle distance (SphereDistance, SphereGeometry.f90:107-125)
// KIND 1: Gaussian 4 exp(-r^2)/pi of the chord distance
// KIND 2: K8 of the chord distance (ChordDistance, SphereGeometry.f90:67-73)
// (FP64 forms below; the FP32C forms are pse_rel.cuh on the sphere and plane_rel.cuh in
// the plane.)
enum { kPseK8Geodesic = 0, kPseGaussChord = 1, kPseK8Chord = 2 };

// FP64 K8, bivariateLaplacianKernel8 with gfortran's integer-power chain
// (r^2 = r r, r^4 = r^2 r^2, r^6 = r^3 r^3 with r^3 = r r^2).
__device__ __forceinline__ double k8_f64(double r) {
  const double r2 = __dmul_rn(r, r);
  const double r3 = __dmul_rn(r, r2);
  const double r4 = __dmul_rn(r2, r2);
  const double r6 = __dmul_rn(r3, r3);
  const double poly = __dsub_rn(__dadd_rn(__dsub_rn(40.0, __dmul_rn(40.0, r2)), __dmul_rn(10.0, r4)),
                                __ddiv_rn(__dmul_rn(2.0, r6), 3.0));
  return __ddiv_rn(__dmul_rn(poly, exp(-__dmul_rn(r, r))), 3.1415926535897932384626433832795027975);
}

struct PseF64Params {
  const double *x, *y, *z, *f;
  double eps, eps2, scale, radius;
  double* lap;
};

template <int KIND>
struct PseF64 {
  struct Tgt {
    double x, y, z, f;
  };
  struct Acc {
    double l;
  };
  __device__ static Tgt load(const PseF64Params& p, int64_t i) {
    return Tgt{p.x[i], p.y[i], p.z ? p.z[i] : 0.0, p.f[i]};
  }
  __device__ static __forceinline__ void interact(const PseF64Params& p, const Tgt& t,
                                                  const Rec64& r, Acc& a) {
    double k;
    if (KIND == kPseK8Geodesic) {
      const double c1 = __dsub_rn(__dmul_rn(t.y, r.z), __dmul_rn(r.y, t.z));
      const double c2 = __dsub_rn(__dmul_rn(r.x, t.z), __dmul_rn(t.x, r.z));
      const double c3 = __dsub_rn(__dmul_rn(t.x, r.y), __dmul_rn(r.x, t.y));
      const double cn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(c1, c1), __dmul_rn(c2, c2)), __dmul_rn(c3, c3)));
      const double dp = __dadd_rn(__dadd_rn(__dmul_rn(t.x, r.x), __dmul_rn(t.y, r.y)), __dmul_rn(t.z, r.z));
      const double kin = __ddiv_rn(__dmul_rn(atan2(cn, dp), p.radius), p.eps);
      k = k8_f64(kin);
    } else {
      const double d1 = __dsub_rn(r.x, t.x), d2 = __dsub_rn(r.y, t.y), d3 = __dsub_rn(r.z, t.z);
      const double kin = __ddiv_rn(
          __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d1, d1), __dmul_rn(d2, d2)), __dmul_rn(d3, d3))), p.eps);
      if (KIND == kPseGaussChord) {
        k = __ddiv_rn(__dmul_rn(4.0, exp(-__dmul_rn(kin, kin))), 3.1415926535897932384626433832795027975);
      } else {
        k = k8_f64(kin);
      }
    }
    a.l = __dadd_rn(a.l, __dmul_rn(__ddiv_rn(__dmul_rn(__dsub_rn(r.q, t.f), k), p.eps2), r.r));
  }
  __device__ static void store(const PseF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.lap[il] = __dmul_rn(a.l, p.scale);
  }
  static constexpr bool kSkipSelf = false;
};

// ============================================================ PSE gradient / divergence (FP64)
// PSESphereGradientAtParticles, src/PSEDirectSum.f90:220-267, and
// PSESphereDivergenceAtParticles, :537-579, with bivariateFirstDerivativeKernel8 (:629-634) in
// gfortran's power chain and MATMUL(SphereProjection(x_i), .) (SphereGeometry.f90:578-590)
// summed row by row left to right.
__device__ __forceinline__ double k1_f64(double r) {
  const double r2 = __dmul_rn(r, r);
  const double r3 = __dmul_rn(r, r2);
  const double r4 = __dmul_rn(r2, r2);
  const double r6 = __dmul_rn(r3, r3);
  const double poly = __dadd_rn(__dsub_rn(__dadd_rn(-20.0, __dmul_rn(20.0, r2)), __dmul_rn(5.0, r4)),
                                __ddiv_rn(r6, 3.0));
  return __ddiv_rn(__dmul_rn(poly, exp(-__dmul_rn(r, r))), 3.1415926535897932384626433832795027975);
}

// atan2(|x_j x x_i|, x_j . x_i): SphereDistance(x_j, x_i) / SphereRadius
__device__ __forceinline__ double sphere_angle_f64(double ax, double ay, double az, double bx, double by, double bz) {
  const double c1 = __dsub_rn(__dmul_rn(ay, bz), __dmul_rn(by, az));
  const double c2 = __dsub_rn(__dmul_rn(bx, az), __dmul_rn(ax, bz));
  const double c3 = __dsub_rn(__dmul_rn(ax, by), __dmul_rn(bx, ay));
  const double cn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(c1, c1), __dmul_rn(c2, c2)), __dmul_rn(c3, c3)));
  const double dp = __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
  return atan2(cn, dp);
}

// (I - x x^T) g, rows summed left to right
__device__ __forceinline__ void sphere_project_f64(double x, double y, double z, double g0, double g1, double g2,
                                                   double& o0, double& o1, double& o2) {
  const double p11 = __dsub_rn(1.0, __dmul_rn(x, x)), p12 = -__dmul_rn(x, y), p13 = -__dmul_rn(x, z);
  const double p21 = -__dmul_rn(y, x), p22 = __dsub_rn(1.0, __dmul_rn(y, y)), p23 = -__dmul_rn(y, z);
  const double p31 = -__dmul_rn(z, x), p32 = -__dmul_rn(z, y), p33 = __dsub_rn(1.0, __dmul_rn(z, z));
  o0 = __dadd_rn(__dadd_rn(__dmul_rn(p11, g0), __dmul_rn(p12, g1)), __dmul_rn(p13, g2));
  o1 = __dadd_rn(__dadd_rn(__dmul_rn(p21, g0), __dmul_rn(p22, g1)), __dmul_rn(p23, g2));
  o2 = __dadd_rn(__dadd_rn(__dmul_rn(p31, g0), __dmul_rn(p32, g1)), __dmul_rn(p33, g2));
}

struct __align__(16) RecVec64 {
  double x, y, z, vx, vy, vz, area;
  long long idx;
};

struct PseVecF64Params {
  const double *x, *y, *z, *f, *vx, *vy, *vz;
  double eps, eps2, denom, radius, scale;  // eps**2, eps**3, 1/eps**2 (gradient) or 1/eps
  double *o0, *o1, *o2;
};

// grad_i += (f_j + f_i) (x_i - x_j) K1(d/eps) / eps**2 A_j; then projected and scaled
struct PseGradF64 {
  struct Tgt {
    double x, y, z, f;
  };
  struct Acc {
    double g0, g1, g2;
  };
  __device__ static Tgt load(const PseVecF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.z[i], p.f[i]}; }
  __device__ static __forceinline__ void interact(const PseVecF64Params& p, const Tgt& t, const Rec64& r, Acc& a) {
    const double kin = __ddiv_rn(__dmul_rn(sphere_angle_f64(r.x, r.y, r.z, t.x, t.y, t.z), p.radius), p.eps);
    const double kout = __ddiv_rn(k1_f64(kin), p.eps2);
    const double fs = __dadd_rn(r.q, t.f);
    a.g0 = __dadd_rn(a.g0, __dmul_rn(__dmul_rn(__dmul_rn(fs, __dsub_rn(t.x, r.x)), kout), r.r));
    a.g1 = __dadd_rn(a.g1, __dmul_rn(__dmul_rn(__dmul_rn(fs, __dsub_rn(t.y, r.y)), kout), r.r));
    a.g2 = __dadd_rn(a.g2, __dmul_rn(__dmul_rn(__dmul_rn(fs, __dsub_rn(t.z, r.z)), kout), r.r));
  }
  __device__ static void store(const PseVecF64Params& p, int64_t i, int64_t il, const Acc& a) {
    double o0, o1, o2;
    sphere_project_f64(p.x[i], p.y[i], p.z[i], a.g0, a.g1, a.g2, o0, o1, o2);
    p.o0[il] = __dmul_rn(o0, p.scale);
    p.o1[il] = __dmul_rn(o1, p.scale);
    p.o2[il] = __dmul_rn(o2, p.scale);
  }
  static constexpr bool kSkipSelf = false;
};

// div_i += (P_i ((x_i - x_j) K1(d/eps) / eps**3)) . (V_j + V_i) A_j; then scaled by 1/eps
struct PseDivF64 {
  struct Tgt {
    double x, y, z, vx, vy, vz;
  };
  struct Acc {
    double d;
  };
  __device__ static Tgt load(const PseVecF64Params& p, int64_t i) {
    return Tgt{p.x[i], p.y[i], p.z[i], p.vx[i], p.vy[i], p.vz[i]};
  }
  __device__ static __forceinline__ void interact(const PseVecF64Params& p, const Tgt& t, const RecVec64& r,
                                                  Acc& a) {
    const double kin = __ddiv_rn(__dmul_rn(sphere_angle_f64(r.x, r.y, r.z, t.x, t.y, t.z), p.radius), p.eps);
    const double k1 = k1_f64(kin);
    const double g0 = __ddiv_rn(__dmul_rn(__dsub_rn(t.x, r.x), k1), p.denom);
    const double g1 = __ddiv_rn(__dmul_rn(__dsub_rn(t.y, r.y), k1), p.denom);
    const double g2 = __ddiv_rn(__dmul_rn(__dsub_rn(t.z, r.z), k1), p.denom);
    double h0, h1, h2;
    sphere_project_f64(t.x, t.y, t.z, g0, g1, g2, h0, h1, h2);
    const double dot = __dadd_rn(__dadd_rn(__dmul_rn(h0, __dadd_rn(r.vx, t.vx)), __dmul_rn(h1, __dadd_rn(r.vy, t.vy))),
                                 __dmul_rn(h2, __dadd_rn(r.vz, t.vz)));
    a.d = __dadd_rn(a.d, __dmul_rn(dot, r.area));
  }
  __device__ static void store(const PseVecF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = __dmul_rn(a.d, p.scale);
  }
  static constexpr bool kSkipSelf = false;
};

// ============================================================ stream functions (FP64)
// SetStreamFunctionsOnMesh, src/SphereBVE.f90:445-485 and SetStreamFunctionOnMesh,
// src/PlanarIncompressible.f90:470-505.  Both skip j = i.
struct __align__(16) RecStream64 {
  double x, y, z, qr, qa, area;
  long long idx;
  long long pad;
};

struct StreamF64Params {
  const double *x, *y, *z;
  double a2, four_pi, two_pi;
  double *psi_rel, *psi_abs;
};

// G = -log(a^2 - sum(xi*xj)) / (4 pi); psi_rel += (G zeta_rel) A, psi_abs += (G zeta_abs) A
struct SphereStreamF64 {
  struct Tgt {
    double x, y, z;
  };
  struct Acc {
    double r, a;
  };
  __device__ static Tgt load(const StreamF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.z[i]}; }
  __device__ static __forceinline__ void interact(const StreamF64Params& p, const Tgt& t,
                                                  const RecStream64& r, Acc& a) {
    const double dot = __dadd_rn(__dadd_rn(__dmul_rn(t.x, r.x), __dmul_rn(t.y, r.y)), __dmul_rn(t.z, r.z));
    const double g = -__ddiv_rn(log(__dsub_rn(p.a2, dot)), p.four_pi);
    a.r = __dadd_rn(a.r, __dmul_rn(__dmul_rn(g, r.qr), r.area));
    a.a = __dadd_rn(a.a, __dmul_rn(__dmul_rn(g, r.qa), r.area));
  }
  __device__ static void store(const StreamF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.psi_rel[il] = a.r;
    p.psi_abs[il] = a.a;
  }
  static constexpr bool kSkipSelf = true;
};

// G = log(sqrt((xi-xj)^2 + (yi-yj)^2)) / (2 pi); psi += (G omega) A
struct PlaneStreamF64 {
  struct Tgt {
    double x, y, z;
  };
  struct Acc {
    double r;
  };
  __device__ static Tgt load(const StreamF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], 0.0}; }
  __device__ static __forceinline__ void interact(const StreamF64Params& p, const Tgt& t,
                                                  const RecStream64& r, Acc& a) {
    const double dx = __dsub_rn(t.x, r.x), dy = __dsub_rn(t.y, r.y);
    const double g = __ddiv_rn(log(__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)))), p.two_pi);
    a.r = __dadd_rn(a.r, __dmul_rn(__dmul_rn(g, r.qr), r.area));
  }
  __device__ static void store(const StreamF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.psi_rel[il] = a.r;
  }
  static constexpr bool kSkipSelf = true;
};

// ============================================================ more PSE operators, SWE integrals (FP64)
// Each restates its Fortran loop body with explicit roundings, like the operators above.

// bivariateDeltaKernel8, src/PSEDirectSum.f90:611-616, with the power chain of k8_f64
__device__ __forceinline__ double kdelta8_f64(double r) {
  const double r2 = __dmul_rn(r, r);
  const double r3 = __dmul_rn(r, r2);
  const double r4 = __dmul_rn(r2, r2);
  const double r6 = __dmul_rn(r3, r3);
  const double poly = __dsub_rn(__dadd_rn(__dsub_rn(4.0, __dmul_rn(6.0, r2)), __dmul_rn(2.0, r4)), __ddiv_rn(r6, 6.0));
  return __ddiv_rn(__dmul_rn(poly, exp(-__dmul_rn(r, r))), 3.1415926535897932384626433832795027975);
}

// ChordDistance of two planar particles (z = 0 on both): sqrt((dx^2 + dy^2) + 0)
__device__ __forceinline__ double plane_chord_f64(double ax, double ay, double bx, double by) {
  const double d1 = __dsub_rn(bx, ax), d2 = __dsub_rn(by, ay);
  return __dsqrt_rn(__dadd_rn(__dmul_rn(d1, d1), __dmul_rn(d2, d2)));
}

struct PseExtF64Params {
  const double *x, *y, *z, *s1, *s2, *s3;  // positions and the target-side fields
  double eps, eps2, eps3, radius, radius2, k0, scale;
  double *o0, *o1, *o2, *o3;
};

// PSEPlaneGradientAtParticles, src/PSEDirectSum.f90:180-217 (Rec64: q = f_j, r = A_j):
// g += (((f_j + f_i) (x_i - x_j)) K1) / eps**3 * A_j, then multiplied by 1/eps
struct PsePlaneGradF64 {
  struct Tgt {
    double x, y, f;
  };
  struct Acc {
    double gx, gy;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.s1[i]}; }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const Rec64& r, Acc& a) {
    const double k1 = k1_f64(__ddiv_rn(plane_chord_f64(t.x, t.y, r.x, r.y), p.eps));
    const double fs = __dadd_rn(r.q, t.f);
    a.gx = __dadd_rn(a.gx, __dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(fs, __dsub_rn(t.x, r.x)), k1), p.eps3), r.r));
    a.gy = __dadd_rn(a.gy, __dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(fs, __dsub_rn(t.y, r.y)), k1), p.eps3), r.r));
  }
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = __dmul_rn(p.scale, a.gx);
    p.o1[il] = __dmul_rn(p.scale, a.gy);
  }
  static constexpr bool kSkipSelf = false;
};

// The four planar sums of PSEPlaneSecondPartialsAtParticles (:286-301) and
// PSEPlaneDoubleDotProductAtParticles (:339-354) (RecVec64: vx = a_j, vy = b_j):
// s_ab += (((a_j + a_i) (x_b,i - x_b,j)) / eps) K1 / eps**2 * A_j
struct PlaneD4F64 {
  struct Tgt {
    double x, y, a, b;
  };
  struct Acc {
    double ax, ay, bx, by;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.s1[i], p.s2[i]}; }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const RecVec64& r,
                                                  Acc& a) {
    const double kout = __ddiv_rn(k1_f64(__ddiv_rn(plane_chord_f64(t.x, t.y, r.x, r.y), p.eps)), p.eps2);
    const double dx = __dsub_rn(t.x, r.x), dy = __dsub_rn(t.y, r.y);
    const double sa = __dadd_rn(r.vx, t.a), sb = __dadd_rn(r.vy, t.b);
    a.ax = __dadd_rn(a.ax, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(sa, dx), p.eps), kout), r.area));
    a.ay = __dadd_rn(a.ay, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(sa, dy), p.eps), kout), r.area));
    a.bx = __dadd_rn(a.bx, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(sb, dx), p.eps), kout), r.area));
    a.by = __dadd_rn(a.by, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(sb, dy), p.eps), kout), r.area));
  }
  static constexpr bool kSkipSelf = false;
};

// PSEPlaneSecondPartialsAtParticles: xx = dxx, xy = 0.5 (dxy + dyx), yy = dyy, times 1/eps
struct PsePlaneSecondF64 : PlaneD4F64 {
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = __dmul_rn(p.scale, a.ax);
    p.o1[il] = __dmul_rn(p.scale, __dmul_rn(0.5, __dadd_rn(a.ay, a.bx)));
    p.o2[il] = __dmul_rn(p.scale, a.by);
  }
};

// PSEPlaneDoubleDotProductAtParticles: (ux ux + 2 uy vx + vy vy) / eps**2
struct PsePlaneDdotF64 : PlaneD4F64 {
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(a.ax, a.ax), __dmul_rn(__dmul_rn(2.0, a.ay), a.bx)),
                               __dmul_rn(a.by, a.by));
    p.o0[il] = __ddiv_rn(s, p.eps2);
  }
};

// PSESphereDoubleDotProductAtParticles, src/PSEDirectSum.f90:367-418 (RecVec64: u, v, w of
// j).  The third row pairs w_j with v_i, as the reference does (:399-404).
struct PseSphereDdotF64 {
  struct Tgt {
    double x, y, z, u, v;
  };
  struct Acc {
    double ux, uy, uz, vx, vy, vz, wx, wy, wz;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) {
    return Tgt{p.x[i], p.y[i], p.z[i], p.s1[i], p.s2[i]};
  }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const RecVec64& r,
                                                  Acc& a) {
    const double kin = __ddiv_rn(__dmul_rn(sphere_angle_f64(t.x, t.y, t.z, r.x, r.y, r.z), p.radius), p.eps);
    const double kout = __ddiv_rn(k1_f64(kin), p.eps2);
    const double dx = __dsub_rn(t.x, r.x), dy = __dsub_rn(t.y, r.y), dz = __dsub_rn(t.z, r.z);
    const double su = __dadd_rn(r.vx, t.u), sv = __dadd_rn(r.vy, t.v), sw = __dadd_rn(r.vz, t.v);
#define LPM_DD(acc, s, d) acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(s, d), p.eps), kout), r.area))
    LPM_DD(a.ux, su, dx);
    LPM_DD(a.uy, su, dy);
    LPM_DD(a.uz, su, dz);
    LPM_DD(a.vx, sv, dx);
    LPM_DD(a.vy, sv, dy);
    LPM_DD(a.vz, sv, dz);
    LPM_DD(a.wx, sw, dx);
    LPM_DD(a.wy, sw, dy);
    LPM_DD(a.wz, sw, dz);
#undef LPM_DD
  }
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    const double d = __dadd_rn(__dadd_rn(__dmul_rn(a.ux, a.ux), __dmul_rn(a.vy, a.vy)), __dmul_rn(a.wz, a.wz));
    const double c = __dadd_rn(__dadd_rn(__dmul_rn(a.uy, a.vx), __dmul_rn(a.uz, a.wx)), __dmul_rn(a.vz, a.wy));
    p.o0[il] = __ddiv_rn(__dadd_rn(d, __dmul_rn(2.0, c)), p.eps2);
  }
  static constexpr bool kSkipSelf = false;
};

// PSEPlaneInterpolateScalar / PSESphereInterpolateScalar, src/PSEDirectSum.f90:128-168, at
// query points (the targets; Rec64: q = f_j, r = A_j): s += ((f_j A_j) Kdelta8) / eps**2
template <bool SPHERE>
struct PseInterpF64 {
  struct Tgt {
    double x, y, z;
  };
  struct Acc {
    double s;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) {
    return Tgt{p.x[i], p.y[i], p.z ? p.z[i] : 0.0};
  }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const Rec64& r, Acc& a) {
    double d;
    if (SPHERE) {
      d = __dmul_rn(sphere_angle_f64(r.x, r.y, r.z, t.x, t.y, t.z), p.radius);
    } else {
      const double d1 = __dsub_rn(r.x, t.x), d2 = __dsub_rn(r.y, t.y), d3 = __dsub_rn(r.z, t.z);
      d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d1, d1), __dmul_rn(d2, d2)), __dmul_rn(d3, d3)));
    }
    a.s = __dadd_rn(a.s, __ddiv_rn(__dmul_rn(__dmul_rn(r.q, r.r), kdelta8_f64(__ddiv_rn(d, p.eps))), p.eps2));
  }
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) { p.o0[il] = a.s; }
  static constexpr bool kSkipSelf = false;
};

// SWEPlaneRHSIntegrals, src/SWEPlaneSolver.f90:457-571 (RecVec64: vx = vort_j, vy = div_j,
// vz = sh_j, the surface height h + topoFn).  The Laplacian term includes j = i (a zero
// term); the rest skips it, as the reference's `cycle` does.
struct SwePlaneF64 {
  struct Tgt {
    double x, y, sh;
    int64_t i;
  };
  struct Acc {
    double u, v, l, ux, uy, vx, vy;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i], p.s3[i], i}; }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const RecVec64& r,
                                                  Acc& a) {
    const double dx = __dsub_rn(t.x, r.x), dy = __dsub_rn(t.y, r.y);
    const double sq = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    const double lk = __ddiv_rn(k8_f64(__ddiv_rn(__dsqrt_rn(sq), p.eps)), p.eps2);
    a.l = __dadd_rn(a.l, __dmul_rn(__dmul_rn(lk, __dsub_rn(r.vz, t.sh)), r.area));
    if (r.idx == t.i) return;
    const double denom = __dmul_rn(p.k0, sq);  // (2 pi) r^2
    const double denom2 = __dmul_rn(__dmul_rn(3.1415926535897932384626433832795027975, sq), sq);
    const double rot = __ddiv_rn(__dmul_rn(r.vx, r.area), denom);
    const double pot = __ddiv_rn(__dmul_rn(r.vy, r.area), denom);
    a.u = __dadd_rn(__dsub_rn(a.u, __dmul_rn(dy, rot)), __dmul_rn(dx, pot));
    a.v = __dadd_rn(__dadd_rn(a.v, __dmul_rn(dx, rot)), __dmul_rn(dy, pot));
    const double cu = __dsub_rn(__dmul_rn(dx, r.vy), __dmul_rn(dy, r.vx));
    const double cv = __dadd_rn(__dmul_rn(dy, r.vy), __dmul_rn(dx, r.vx));
    a.ux = __dsub_rn(__dadd_rn(a.ux, pot), __ddiv_rn(__dmul_rn(__dmul_rn(dx, cu), r.area), denom2));
    a.uy = __dsub_rn(__dsub_rn(a.uy, rot), __ddiv_rn(__dmul_rn(__dmul_rn(dy, cu), r.area), denom2));
    a.vx = __dsub_rn(__dadd_rn(a.vx, rot), __ddiv_rn(__dmul_rn(__dmul_rn(dx, cv), r.area), denom2));
    a.vy = __dsub_rn(__dadd_rn(a.vy, pot), __ddiv_rn(__dmul_rn(__dmul_rn(dy, cv), r.area), denom2));
  }
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = a.u;
    p.o1[il] = a.v;
    p.o2[il] = __dadd_rn(__dadd_rn(__dmul_rn(a.ux, a.ux), __dmul_rn(__dmul_rn(2.0, a.uy), a.vx)), __dmul_rn(a.vy, a.vy));
    p.o3[il] = __ddiv_rn(a.l, p.eps2);
  }
  static constexpr bool kSkipSelf = false;
};

// SWESphereRHSIntegrals, src/SphereSWESolver.f90:299-372 (RecVec64: vx = zeta_j, vy = div_j,
// vz = sh_j).  k0 = 4 pi a^2, radius = a, radius2 = the SphereRadius of SphereDistance.  As in
// the reference, lapSurf keeps the 1/eps**2 inside the kernel only and doubleDot is 0.
struct SweSphereF64 {
  struct Tgt {
    double x, y, z, sh;
    int64_t i;
  };
  struct Acc {
    double u, v, w, l;
  };
  __device__ static Tgt load(const PseExtF64Params& p, int64_t i) {
    return Tgt{p.x[i], p.y[i], p.z[i], p.s3[i], i};
  }
  __device__ static __forceinline__ void interact(const PseExtF64Params& p, const Tgt& t, const RecVec64& r,
                                                  Acc& a) {
    const double kin = __ddiv_rn(__dmul_rn(sphere_angle_f64(t.x, t.y, t.z, r.x, r.y, r.z), p.radius2), p.eps);
    const double lk = __ddiv_rn(k8_f64(kin), p.eps2);
    a.l = __dadd_rn(a.l, __dmul_rn(__dmul_rn(lk, __dsub_rn(r.vz, t.sh)), r.area));
    if (r.idx == t.i) return;
    const double dp = __dadd_rn(__dadd_rn(__dmul_rn(t.x, r.x), __dmul_rn(t.y, r.y)), __dmul_rn(t.z, r.z));
    const double denom = __dmul_rn(p.k0, __dsub_rn(__dmul_rn(p.radius, p.radius), dp));
    const double rot = __ddiv_rn(__dmul_rn(r.vx, r.area), denom);
    const double pot = __ddiv_rn(__dmul_rn(__dmul_rn(p.radius, r.vy), r.area), denom);
    a.u = __dsub_rn(__dsub_rn(a.u, __dmul_rn(__dsub_rn(__dmul_rn(t.y, r.z), __dmul_rn(t.z, r.y)), rot)),
                    __dmul_rn(r.x, pot));
    a.v = __dsub_rn(__dsub_rn(a.v, __dmul_rn(__dsub_rn(__dmul_rn(t.z, r.x), __dmul_rn(t.x, r.z)), rot)),
                    __dmul_rn(r.y, pot));
    a.w = __dsub_rn(__dsub_rn(a.w, __dmul_rn(__dsub_rn(__dmul_rn(t.x, r.y), __dmul_rn(t.y, r.x)), rot)),
                    __dmul_rn(r.z, pot));
  }
  __device__ static void store(const PseExtF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = a.u;
    p.o1[il] = a.v;
    p.o2[il] = a.w;
    p.o3[il] = a.l;
  }
  static constexpr bool kSkipSelf = false;
};

// BetaPlaneVelocity, src/BetaPlaneSolver.f90:227-268 (RecStream64: qr = zeta_j, area): the
// x-periodic kernel, strength = ((0.5 zeta_j) A_j) / (cosh(2 pi dy) - cos(2 pi dx)),
// u -= sinh(2 pi dy) strength, v += sin(2 pi dx) strength; j = i skipped.
struct BetaF64Params {
  const double *x, *y;
  double two_pi, four_pi;
  double *o0, *o1;
};

struct BetaVelF64 {
  struct Tgt {
    double x, y;
  };
  struct Acc {
    double u, v;
  };
  __device__ static Tgt load(const BetaF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i]}; }
  __device__ static __forceinline__ void interact(const BetaF64Params& p, const Tgt& t, const RecStream64& r,
                                                  Acc& a) {
    const double ay = __dmul_rn(p.two_pi, __dsub_rn(t.y, r.y)), ax = __dmul_rn(p.two_pi, __dsub_rn(t.x, r.x));
    const double s = __ddiv_rn(__dmul_rn(__dmul_rn(0.5, r.qr), r.area), __dsub_rn(cosh(ay), cos(ax)));
    a.u = __dsub_rn(a.u, __dmul_rn(sinh(ay), s));
    a.v = __dadd_rn(a.v, __dmul_rn(sin(ax), s));
  }
  __device__ static void store(const BetaF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = a.u;
    p.o1[il] = a.v;
  }
  static constexpr bool kSkipSelf = true;
};

// SetStreamFunctionsOnMesh of the beta plane, src/BetaPlane.f90:399-442 (RecStream64: qr, qa
// = relative and absolute vorticity): G = log(cosh(2 pi dy) - cos(2 pi dx)) / (4 pi),
// psi += (G zeta_j) A_j; j = i skipped.
struct BetaStreamF64 {
  struct Tgt {
    double x, y;
  };
  struct Acc {
    double r, a;
  };
  __device__ static Tgt load(const BetaF64Params& p, int64_t i) { return Tgt{p.x[i], p.y[i]}; }
  __device__ static __forceinline__ void interact(const BetaF64Params& p, const Tgt& t, const RecStream64& r,
                                                  Acc& a) {
    const double g = __ddiv_rn(log(__dsub_rn(cosh(__dmul_rn(p.two_pi, __dsub_rn(t.y, r.y))),
                                             cos(__dmul_rn(p.two_pi, __dsub_rn(t.x, r.x))))),
                               p.four_pi);
    a.r = __dadd_rn(a.r, __dmul_rn(__dmul_rn(g, r.qr), r.area));
    a.a = __dadd_rn(a.a, __dmul_rn(__dmul_rn(g, r.qa), r.area));
  }
  __device__ static void store(const BetaF64Params& p, int64_t i, int64_t il, const Acc& a) {
    p.o0[il] = a.r;
    p.o1[il] = a.a;
  }
  static constexpr bool kSkipSelf = true;
};

// ============================================================ beta-plane velocity (FP32C)
// BetaPlaneVelocity, src/BetaPlaneSolver.f90:227-268, in FP32 with a form that does not
// cancel: cosh(2a) - cos(2b) = 2 (sinh^2 a + sin^2 b), sinh 2a = 2 sinh a cosh a and
// sin 2b = 2 sin b cos b with a = pi dy, b = pi dx, so per pair
//   u -= S sh ch / (sh^2 + sn^2),  v += S sn cs / (sh^2 + sn^2),  S = zeta_j A_j / 2.
// dx is reduced to t = dx - rint(dx) in [-1/2, 1/2] (the kernel has period 1 in x) with the
// rounding of x_i - x_j kept (TwoSum), so that neighbours across the periodic boundary keep
// full precision; sin(pi t), cos(pi t) are Taylor polynomials (|error| <= 6e-8 on the
// interval).  sinh and cosh of a = pi |dy| use a = k ln 2 + r, |r| <= ln2/2, polynomials in
// r, and sinh a = 2^(k-1) ((1 - 4^-k) cosh r + (1 + 4^-k) sinh r) (cosh alike); the common
// factor 2^(k-1) is divided out of every term (sn, cs scaled by 2^(1-k)), so nothing
// overflows for any dy.  The self pair (d = 0) has zero numerators and a denominator of
// 2^-100, a zero term.
// Shared pieces of the x-periodic kernels, two targets at a time.  A record holds
// (x_hi, y_hi, x_lo, y_lo) of the source in its first float4.
struct BetaTgt {
  float xh, yh, xl, yl;
};

__device__ __forceinline__ float2 bits_abs(float2 v) {
  return make_float2(__uint_as_float(__float_as_uint(v.x) & 0x7fffffffu),
                     __uint_as_float(__float_as_uint(v.y) & 0x7fffffffu));
}

// t = (x_i - x_j) - rint(x_i - x_j) in [-1/2, 1/2] keeping the rounding of the hi difference
// (TwoSum), and dy = (y_i - y_j) from the hi/lo parts.
__device__ __forceinline__ void beta_deltas2(const BetaTgt& t0, const BetaTgt& t1, float4 ra, float2& tt, float2& dy) {
  const float2 kM = make_float2(12582912.0f, 12582912.0f), kNM = make_float2(-12582912.0f, -12582912.0f);
  const float2 nxh = make_float2(-ra.x, -ra.x);
  const float2 txh = make_float2(t0.xh, t1.xh);
  const float2 dh = __fadd2_rn(txh, nxh);
  const float2 bb = __fadd2_rn(dh, make_float2(-txh.x, -txh.y));
  const float2 dv = __fadd2_rn(dh, make_float2(-bb.x, -bb.y));
  const float2 e = __fadd2_rn(__fadd2_rn(txh, make_float2(-dv.x, -dv.y)), __fadd2_rn(nxh, make_float2(-bb.x, -bb.y)));
  const float2 nn = __fadd2_rn(__fadd2_rn(dh, kM), kNM);
  const float2 lo = __fadd2_rn(e, __fadd2_rn(make_float2(t0.xl, t1.xl), make_float2(-ra.z, -ra.z)));
  tt = __fadd2_rn(__fadd2_rn(dh, make_float2(-nn.x, -nn.y)), lo);
  dy = __fadd2_rn(__fadd2_rn(make_float2(t0.yh, t1.yh), make_float2(-ra.y, -ra.y)),
                  __fadd2_rn(make_float2(t0.yl, t1.yl), make_float2(-ra.w, -ra.w)));
}

// sin(pi t) and cos(pi t), |t| <= 1/2, Taylor polynomials in t^2 (|error| <= 6e-8)
__device__ __forceinline__ float2 sinpi2(float2 tt, float2 t2) {
  float2 ps = __ffma2_rn(make_float2(-0.00737043097615242f, -0.00737043097615242f), t2,
                         make_float2(0.08214588463306427f, 0.08214588463306427f));
  ps = __ffma2_rn(ps, t2, make_float2(-0.5992645025253296f, -0.5992645025253296f));
  ps = __ffma2_rn(ps, t2, make_float2(2.550163984298706f, 2.550163984298706f));
  ps = __ffma2_rn(ps, t2, make_float2(-5.167712688446045f, -5.167712688446045f));
  ps = __ffma2_rn(ps, t2, make_float2(3.1415927410125732f, 3.1415927410125732f));
  return __fmul2_rn(ps, tt);
}
__device__ __forceinline__ float2 cospi2(float2 t2) {
  float2 pc = __ffma2_rn(make_float2(0.001929574296809733f, 0.001929574296809733f), t2,
                         make_float2(-0.025806890800595284f, -0.025806890800595284f));
  pc = __ffma2_rn(pc, t2, make_float2(0.23533062636852264f, 0.23533062636852264f));
  pc = __ffma2_rn(pc, t2, make_float2(-1.3352627754211426f, -1.3352627754211426f));
  pc = __ffma2_rn(pc, t2, make_float2(4.058712005615234f, 4.058712005615234f));
  pc = __ffma2_rn(pc, t2, make_float2(-4.934802055358887f, -4.934802055358887f));
  return __ffma2_rn(pc, t2, make_float2(1.0f, 1.0f));
}

// a = k ln 2 + r, |r| <= ln 2 / 2: sinh r, cosh r (Taylor), and kb = 1.5 2^23 + k (its bits
// minus those of 1.5 2^23 are k), for a >= 0 below 2^22 ln 2.
__device__ __forceinline__ void sinh_cosh_reduced2(float2 a, float2& shr, float2& chr, float2& kb) {
  kb = __ffma2_rn(a, make_float2(1.442695f, 1.442695f), make_float2(12582912.0f, 12582912.0f));
  const float2 kf = __fadd2_rn(kb, make_float2(-12582912.0f, -12582912.0f));
  float2 rr = __ffma2_rn(make_float2(-kf.x, -kf.y), make_float2(0.69314575f, 0.69314575f), a);
  rr = __ffma2_rn(make_float2(-kf.x, -kf.y), make_float2(1.4286068e-06f, 1.4286068e-06f), rr);
  const float2 r2 = __fmul2_rn(rr, rr);
  shr = __ffma2_rn(
      __fmul2_rn(rr, r2),
      __ffma2_rn(__ffma2_rn(r2, make_float2(1.9841270e-4f, 1.9841270e-4f), make_float2(8.3333333e-3f, 8.3333333e-3f)),
                 r2, make_float2(0.16666667f, 0.16666667f)),
      rr);
  chr = __ffma2_rn(
      __ffma2_rn(__ffma2_rn(__ffma2_rn(r2, make_float2(2.4801587e-5f, 2.4801587e-5f),
                                       make_float2(1.3888889e-3f, 1.3888889e-3f)),
                            r2, make_float2(4.1666667e-2f, 4.1666667e-2f)),
                 r2, make_float2(0.5f, 0.5f)),
      r2, make_float2(1.0f, 1.0f));
}

struct BetaF32 {
  struct __align__(16) Rec {
    float4 a;  // x_hi, y_hi, x_lo, y_lo
    float4 b;  // S = zeta A / 2, 0, 0, 0
  };
  using Tgt = BetaTgt;
  // Two targets at once in packed FP32x2 arithmetic.  2^-k comes from the bits of the
  // magic-number sum that rounds a / ln 2 (a clamped to 87 < 126 ln 2: beyond it the terms
  // have reached their limits, u -> S sign(dy), v -> 0); 2^(1-k) = 2^-k + 2^-k and
  // 4^-k = (2^-k)^2, which underflows to 0 for k > 63 as it should.
  __device__ static __forceinline__ void interact2(const Tgt& t0, const Tgt& t1, const Rec& r, float (&a0)[2],
                                                   float (&a1)[2]) {
    float2 tt, dy;
    beta_deltas2(t0, t1, r.a, tt, dy);
    const float2 t2 = __fmul2_rn(tt, tt);
    const float2 sn = sinpi2(tt, t2), cs = cospi2(t2);
    float2 a = __fmul2_rn(make_float2(3.1415927f, 3.1415927f), bits_abs(dy));
    a = make_float2(fminf(a.x, 87.0f), fminf(a.y, 87.0f));
    float2 shr, chr, kb;
    sinh_cosh_reduced2(a, shr, chr, kb);
    // 2^-k: 0x3f800000 - (k << 23) with k = bits(kb) - bits(kM) (bits(kM) << 23 vanishes mod 2^32)
    const float2 pk = make_float2(__uint_as_float(0x3f800000u - (__float_as_uint(kb.x) << 23)),
                                  __uint_as_float(0x3f800000u - (__float_as_uint(kb.y) << 23)));
    const float2 sc = __fadd2_rn(pk, pk);
    const float2 q = __fmul2_rn(pk, pk);
    const float2 om = __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-q.x, -q.y));
    const float2 op = __fadd2_rn(make_float2(1.0f, 1.0f), q);
    float2 shp = __ffma2_rn(om, chr, __fmul2_rn(op, shr));
    shp = make_float2(copysignf(shp.x, dy.x), copysignf(shp.y, dy.y));
    const float2 chp = __ffma2_rn(op, chr, __fmul2_rn(om, shr));
    const float2 snp = __fmul2_rn(sn, sc), csp = __fmul2_rn(cs, sc);
    const float2 den = __ffma2_rn(shp, shp, __ffma2_rn(snp, snp, make_float2(7.888609052210118e-31f, 7.888609052210118e-31f)));
    const float2 w = __fmul2_rn(make_float2(r.b.x, r.b.x), make_float2(rcp_approx(den.x), rcp_approx(den.y)));
    const float2 wsh = __fmul2_rn(w, shp), wsn = __fmul2_rn(w, snp);
    const float2 au = __ffma2_rn(make_float2(-wsh.x, -wsh.y), chp, make_float2(a0[0], a1[0]));
    const float2 av = __ffma2_rn(wsn, csp, make_float2(a0[1], a1[1]));
    a0[0] = au.x;
    a1[0] = au.y;
    a0[1] = av.x;
    a1[1] = av.y;
  }
};

// ============================================================ stream functions (FP32C)
// Both stream functions (stream_rel.cuh) sum S_j ln(q_ij) with ln from ln_q2, accurate to
// about 1 ulp.  A pair with d = 0 (the self pair) is skipped by giving it q = 1, as the
// reference's j /= i skips it; q is otherwise clamped to >= 2^-126 so that a degenerate pair
// stays finite.  The sums are over many terms of both signs that cancel to a much smaller
// psi, so the FP32 partials are flushed into the compensated accumulators every 32 sources.
constexpr float kLogFloor = 1.1754943508222875e-38f;  // 2^-126
constexpr double kInv4Pi = 0.079577471545947667884;   // 1 / (4 pi)

}  // namespace lpm
