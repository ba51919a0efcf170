"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the test suite, the smoke check and the benchmark's CPU-baseline leg use this module.
It restates the reference Fortran loops in FP64 (see lpm_oracle.h for the citations and
for what pins each routine); the shipped library never imports it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build  # noqa: F401  (package-relative when imported as oracle.oracle)

_LIB = None

ASSOC_SOLVER = 0
ASSOC_MESH = 1
PSE_K8_GEODESIC = 0
PSE_GAUSS_CHORD = 1
PSE_K8_CHORD = 2

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_i64 = ctypes.c_int64


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        L.lpmo_bve_velocity.argtypes = [_i64, _D, _D, _D, _D, _D, _I, ctypes.c_double, ctypes.c_int,
                                        _i64, _i64, _D, _D, _D, ctypes.c_int]
        L.lpmo_plane_velocity.argtypes = [_i64, _D, _D, _D, _D, _I, ctypes.c_double, _i64, _i64, _D, _D,
                                          ctypes.c_int]
        L.lpmo_pse_laplacian.argtypes = [_i64, _D, _D, _D, _D, _D, _I, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, _i64, _i64, _D, ctypes.c_int]
        L.lpmo_bve_stream.argtypes = [_i64, _D, _D, _D, _D, _D, _D, _I, ctypes.c_double, _i64, _i64, _D, _D,
                                      ctypes.c_int]
        L.lpmo_plane_stream.argtypes = [_i64, _D, _D, _D, _D, _I, _i64, _i64, _D, ctypes.c_int]
        L.lpmo_bve_timestep.argtypes = [_i64, _D, _D, _D, _D, _D, _I, _D, _D, _D, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.lpmo_plane_timestep.argtypes = [_i64, _D, _D, _D, _D, _I, _D, _D, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int]
        L.lpmo_bve_diagnostics.argtypes = [_i64, _D, _D, _D, _D, _D, _I, _D, _D, _D]
        L.lpmo_pse_sphere_gradient.argtypes = [_i64, _D, _D, _D, _D, _D, _I, ctypes.c_double, ctypes.c_double,
                                               _i64, _i64, _D, _D, _D, ctypes.c_int]
        L.lpmo_pse_sphere_divergence.argtypes = [_i64, _D, _D, _D, _D, _D, _D, _D, _I, ctypes.c_double,
                                                 ctypes.c_double, _i64, _i64, _D, ctypes.c_int]
        c_d, c_i = ctypes.c_double, ctypes.c_int
        L.lpmo_pse_plane_gradient.argtypes = [_i64, _D, _D, _D, _D, _I, c_d, _i64, _i64, _D, _D, c_i]
        L.lpmo_pse_plane_second_partials.argtypes = [_i64, _D, _D, _D, _D, _D, _I, c_d, _i64, _i64, _D, _D, _D,
                                                     c_i]
        L.lpmo_pse_plane_double_dot.argtypes = [_i64, _D, _D, _D, _D, _D, _I, c_d, _i64, _i64, _D, c_i]
        L.lpmo_pse_sphere_double_dot.argtypes = [_i64, _D, _D, _D, _D, _D, _D, _D, _I, c_d, c_d, _i64, _i64, _D,
                                                 c_i]
        L.lpmo_pse_interpolate.argtypes = [_i64, _D, _D, _D, _D, _D, _I, c_d, c_d, c_i, _i64, _D, _D, _D, _D, c_i]
        L.lpmo_swe_plane_rhs.argtypes = [_i64, _D, _D, _D, _D, _D, _D, _I, c_d, _i64, _i64, _D, _D, _D, _D, c_i]
        L.lpmo_swe_sphere_rhs.argtypes = [_i64, _D, _D, _D, _D, _D, _D, _D, _I, c_d, c_d, c_d, _i64, _i64, _D, _D,
                                          _D, _D, _D, c_i]
        L.lpmo_beta_plane_velocity.argtypes = [_i64, _D, _D, _D, _D, _I, _i64, _i64, _D, _D, c_i]
        L.lpmo_beta_plane_stream.argtypes = [_i64, _D, _D, _D, _D, _D, _I, _i64, _i64, _D, _D, c_i]
        L.lpmo_kdelta8.argtypes = [ctypes.c_double]
        L.lpmo_kdelta8.restype = ctypes.c_double
        L.lpmo_k8.argtypes = [ctypes.c_double]
        L.lpmo_k1.argtypes = [ctypes.c_double]
        L.lpmo_k1.restype = ctypes.c_double
        L.lpmo_k8.restype = ctypes.c_double
        _LIB = L
    return _LIB


def _d(a):
    if a is None:
        return None
    return a.ctypes.data_as(_D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _range(n, ib, ie):
    ib = 0 if ib is None else int(ib)
    ie = n if ie is None else int(ie)
    return ib, ie


def bve_velocity(x, y, z, zeta, area, active, radius=1.0, assoc=ASSOC_SOLVER, ib=None, ie=None, threads=0):
    """BVESphereVelocity / setVelocityFromVorticity for targets [ib, ie) (0-based)."""
    x, y, z, zeta, area = (_f64(a) for a in (x, y, z, zeta, area))
    active = _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    u = np.zeros(n)
    v = np.zeros(n)
    w = np.zeros(n)
    lib().lpmo_bve_velocity(n, _d(x), _d(y), _d(z), _d(zeta), _d(area), active.ctypes.data_as(_I), radius,
                            assoc, ib, ie, _d(u), _d(v), _d(w), threads)
    return u[ib:ie], v[ib:ie], w[ib:ie]


def plane_velocity(x, y, omega, area, active, delta=0.0, ib=None, ie=None, threads=0):
    x, y, omega, area, active = _f64(x), _f64(y), _f64(omega), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    u = np.zeros(n)
    v = np.zeros(n)
    lib().lpmo_plane_velocity(n, _d(x), _d(y), _d(omega), _d(area), active.ctypes.data_as(_I), delta, ib, ie,
                              _d(u), _d(v), threads)
    return u[ib:ie], v[ib:ie]


def pse_laplacian(x, y, z, f, area, active, eps, radius=1.0, kernel=PSE_K8_GEODESIC, ib=None, ie=None,
                  threads=0):
    x, y, f, area, active = _f64(x), _f64(y), _f64(f), _f64(area), _i32(active)
    z = None if z is None else _f64(z)
    n = x.size
    ib, ie = _range(n, ib, ie)
    lap = np.zeros(n)
    lib().lpmo_pse_laplacian(n, _d(x), _d(y), _d(z), _d(f), _d(area), active.ctypes.data_as(_I), eps, radius,
                             kernel, ib, ie, _d(lap), threads)
    return lap[ib:ie]


def pse_sphere_gradient(x, y, z, f, area, active, eps, radius=1.0, ib=None, ie=None, threads=0):
    """PSESphereGradientAtParticles (src/PSEDirectSum.f90:220-267); returns (gx, gy, gz) of the block."""
    x, y, z, f, area, active = _f64(x), _f64(y), _f64(z), _f64(f), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    g = [np.zeros(n) for _ in range(3)]
    lib().lpmo_pse_sphere_gradient(n, _d(x), _d(y), _d(z), _d(f), _d(area), active.ctypes.data_as(_I), eps, radius,
                                   ib, ie, _d(g[0]), _d(g[1]), _d(g[2]), threads)
    return tuple(a[ib:ie] for a in g)


def pse_sphere_divergence(x, y, z, vx, vy, vz, area, active, eps, radius=1.0, ib=None, ie=None, threads=0):
    """PSESphereDivergenceAtParticles (src/PSEDirectSum.f90:537-579); returns div of the block."""
    x, y, z, vx, vy, vz, area, active = (_f64(x), _f64(y), _f64(z), _f64(vx), _f64(vy), _f64(vz), _f64(area),
                                         _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    d = np.zeros(n)
    lib().lpmo_pse_sphere_divergence(n, _d(x), _d(y), _d(z), _d(vx), _d(vy), _d(vz), _d(area),
                                     active.ctypes.data_as(_I), eps, radius, ib, ie, _d(d), threads)
    return d[ib:ie]


def pse_plane_gradient(x, y, f, area, active, eps, ib=None, ie=None, threads=0):
    """PSEPlaneGradientAtParticles (src/PSEDirectSum.f90:180-217); returns (gx, gy) of the block."""
    x, y, f, area, active = _f64(x), _f64(y), _f64(f), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    g = [np.zeros(n) for _ in range(2)]
    lib().lpmo_pse_plane_gradient(n, _d(x), _d(y), _d(f), _d(area), active.ctypes.data_as(_I), eps, ib, ie,
                                  _d(g[0]), _d(g[1]), threads)
    return tuple(a[ib:ie] for a in g)


def pse_plane_second_partials(x, y, gx, gy, area, active, eps, ib=None, ie=None, threads=0):
    """PSEPlaneSecondPartialsAtParticles (src/PSEDirectSum.f90:269-320); returns (xx, xy, yy)."""
    x, y, gx, gy, area, active = _f64(x), _f64(y), _f64(gx), _f64(gy), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    o = [np.zeros(n) for _ in range(3)]
    lib().lpmo_pse_plane_second_partials(n, _d(x), _d(y), _d(gx), _d(gy), _d(area), active.ctypes.data_as(_I),
                                         eps, ib, ie, _d(o[0]), _d(o[1]), _d(o[2]), threads)
    return tuple(a[ib:ie] for a in o)


def pse_plane_double_dot(x, y, u, v, area, active, eps, ib=None, ie=None, threads=0):
    """PSEPlaneDoubleDotProductAtParticles (src/PSEDirectSum.f90:322-365)."""
    x, y, u, v, area, active = _f64(x), _f64(y), _f64(u), _f64(v), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    o = np.zeros(n)
    lib().lpmo_pse_plane_double_dot(n, _d(x), _d(y), _d(u), _d(v), _d(area), active.ctypes.data_as(_I), eps,
                                    ib, ie, _d(o), threads)
    return o[ib:ie]


def pse_sphere_double_dot(x, y, z, u, v, w, area, active, eps, radius=1.0, ib=None, ie=None, threads=0):
    """PSESphereDoubleDotProductAtParticles (src/PSEDirectSum.f90:367-418)."""
    x, y, z, u, v, w, area, active = (_f64(x), _f64(y), _f64(z), _f64(u), _f64(v), _f64(w), _f64(area),
                                      _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    o = np.zeros(n)
    lib().lpmo_pse_sphere_double_dot(n, _d(x), _d(y), _d(z), _d(u), _d(v), _d(w), _d(area),
                                     active.ctypes.data_as(_I), eps, radius, ib, ie, _d(o), threads)
    return o[ib:ie]


def pse_interpolate(x, y, z, f, area, active, eps, qx, qy, qz, geometry, radius=1.0, threads=0):
    """PSEPlaneInterpolateScalar (geometry 0) / PSESphereInterpolateScalar (geometry 1),
    src/PSEDirectSum.f90:128-168, at the query points (qx, qy, qz)."""
    x, y, f, area, active = _f64(x), _f64(y), _f64(f), _f64(area), _i32(active)
    z = np.zeros_like(x) if z is None else _f64(z)
    qx, qy = _f64(qx), _f64(qy)
    qz = np.zeros_like(qx) if qz is None else _f64(qz)
    o = np.zeros(qx.size)
    lib().lpmo_pse_interpolate(x.size, _d(x), _d(y), _d(z), _d(f), _d(area), active.ctypes.data_as(_I), eps,
                               radius, geometry, qx.size, _d(qx), _d(qy), _d(qz), _d(o), threads)
    return o


def swe_plane_rhs(x, y, vort, div, sh, area, active, eps, ib=None, ie=None, threads=0):
    """SWEPlaneRHSIntegrals (src/SWEPlaneSolver.f90:457-571); returns (u, v, doubleDot, lapSurf)."""
    x, y, vort, div, sh, area, active = (_f64(x), _f64(y), _f64(vort), _f64(div), _f64(sh), _f64(area),
                                         _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    o = [np.zeros(n) for _ in range(4)]
    lib().lpmo_swe_plane_rhs(n, _d(x), _d(y), _d(vort), _d(div), _d(sh), _d(area), active.ctypes.data_as(_I), eps,
                             ib, ie, _d(o[0]), _d(o[1]), _d(o[2]), _d(o[3]), threads)
    return tuple(a[ib:ie] for a in o)


def swe_sphere_rhs(x, y, z, relvort, div, sh, area, active, radius, sphere_radius, eps, ib=None, ie=None,
                   threads=0):
    """SWESphereRHSIntegrals (src/SphereSWESolver.f90:299-372); returns (u, v, w, doubleDot, lapSurf)."""
    x, y, z, relvort, div, sh, area, active = (_f64(x), _f64(y), _f64(z), _f64(relvort), _f64(div), _f64(sh),
                                               _f64(area), _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    o = [np.zeros(n) for _ in range(5)]
    lib().lpmo_swe_sphere_rhs(n, _d(x), _d(y), _d(z), _d(relvort), _d(div), _d(sh), _d(area),
                              active.ctypes.data_as(_I), radius, sphere_radius, eps, ib, ie, _d(o[0]), _d(o[1]),
                              _d(o[2]), _d(o[3]), _d(o[4]), threads)
    return tuple(a[ib:ie] for a in o)


def beta_plane_velocity(x, y, zeta, area, active, ib=None, ie=None, threads=0):
    """BetaPlaneVelocity (src/BetaPlaneSolver.f90:227-268); returns (u, v) of the block."""
    x, y, zeta, area, active = _f64(x), _f64(y), _f64(zeta), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    u, v = np.zeros(n), np.zeros(n)
    lib().lpmo_beta_plane_velocity(n, _d(x), _d(y), _d(zeta), _d(area), active.ctypes.data_as(_I), ib, ie, _d(u),
                                   _d(v), threads)
    return u[ib:ie], v[ib:ie]


def beta_plane_stream(x, y, relvort, absvort, area, active, ib=None, ie=None, threads=0):
    """SetStreamFunctionsOnMesh of the beta plane (src/BetaPlane.f90:399-442); returns (psi_rel, psi_abs)."""
    x, y, relvort, absvort, area, active = (_f64(x), _f64(y), _f64(relvort), _f64(absvort), _f64(area),
                                            _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    pr, pa = np.zeros(n), np.zeros(n)
    lib().lpmo_beta_plane_stream(n, _d(x), _d(y), _d(relvort), _d(absvort), _d(area), active.ctypes.data_as(_I), ib,
                                 ie, _d(pr), _d(pa), threads)
    return pr[ib:ie], pa[ib:ie]


def kdelta8(r):
    return lib().lpmo_kdelta8(float(r))


def bve_stream(x, y, z, relvort, absvort, area, active, radius=1.0, ib=None, ie=None, threads=0):
    x, y, z, relvort, absvort, area, active = (_f64(x), _f64(y), _f64(z), _f64(relvort), _f64(absvort),
                                               _f64(area), _i32(active))
    n = x.size
    ib, ie = _range(n, ib, ie)
    pr = np.zeros(n)
    pa = np.zeros(n)
    lib().lpmo_bve_stream(n, _d(x), _d(y), _d(z), _d(relvort), _d(absvort), _d(area), active.ctypes.data_as(_I),
                          radius, ib, ie, _d(pr), _d(pa), threads)
    return pr[ib:ie], pa[ib:ie]


def plane_stream(x, y, omega, area, active, ib=None, ie=None, threads=0):
    x, y, omega, area, active = _f64(x), _f64(y), _f64(omega), _f64(area), _i32(active)
    n = x.size
    ib, ie = _range(n, ib, ie)
    p = np.zeros(n)
    lib().lpmo_plane_stream(n, _d(x), _d(y), _d(omega), _d(area), active.ctypes.data_as(_I), ib, ie, _d(p),
                            threads)
    return p[ib:ie]


def bve_timestep(x, y, z, zeta, area, active, u, v, w, radius, omega, dt, nsteps, threads=0):
    """Advances copies of the state; returns (x, y, z, zeta, u, v, w)."""
    x, y, z, zeta, u, v, w = (_f64(a).copy() for a in (x, y, z, zeta, u, v, w))
    area, active = _f64(area), _i32(active)
    lib().lpmo_bve_timestep(x.size, _d(x), _d(y), _d(z), _d(zeta), _d(area), active.ctypes.data_as(_I), _d(u),
                            _d(v), _d(w), radius, omega, dt, nsteps, threads)
    return x, y, z, zeta, u, v, w


def plane_timestep(x, y, omega, area, active, u, v, delta, dt, nsteps, threads=0):
    x, y, u, v = (_f64(a).copy() for a in (x, y, u, v))
    omega, area, active = _f64(omega), _f64(area), _i32(active)
    lib().lpmo_plane_timestep(x.size, _d(x), _d(y), _d(omega), _d(area), active.ctypes.data_as(_I), _d(u),
                              _d(v), delta, dt, nsteps, threads)
    return x, y, u, v


def bve_diagnostics(u, v, w, zeta, area, active):
    u, v, zeta, area, active = _f64(u), _f64(v), _f64(zeta), _f64(area), _i32(active)
    w = None if w is None else _f64(w)
    ke = ctypes.c_double()
    en = ctypes.c_double()
    ci = ctypes.c_double()
    lib().lpmo_bve_diagnostics(u.size, _d(u), _d(v), _d(w), _d(zeta), _d(area), active.ctypes.data_as(_I),
                               ctypes.byref(ke), ctypes.byref(en), ctypes.byref(ci))
    return ke.value, en.value, ci.value


def k8(r: float) -> float:
    return lib().lpmo_k8(r)


LIB_PATH: Path = _build.LIB_PATH
