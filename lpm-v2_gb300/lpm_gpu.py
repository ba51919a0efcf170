"""Python binding of liblpm_gpu.so (the GB300 direct-sum library) through its C ABI.

The functions mirror the lpm-v2 routines they replace -- same names (snake_case), same
argument meaning, 1-based inclusive target ranges -- so a test reads like the reference's
own code.  Every call goes through the C ABI declared in include/lpm_gpu.h; there is no
CPU fallback: if the library cannot be loaded, or a call fails, LpmError is raised.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "liblpm_gpu.so"

MODE_FP64 = 0
MODE_FP32C = 1
FLAG_CHECK_FINITE = 0x100
PSE_K8_GEODESIC = 0
PSE_GAUSS_CHORD = 1
PSE_K8_CHORD = 2

QUAD_RECT_SEED = 202
ICOS_TRI_SPHERE_SEED = 205
CUBED_SPHERE_SEED = 206

ERRORS = {
    0: "LPM_OK",
    -1: "LPM_ERR_ARG",
    -2: "LPM_ERR_CUDA",
    -3: "LPM_ERR_TIMEOUT",
    -4: "LPM_ERR_NONFINITE",
    -5: "LPM_ERR_ALLOC",
    -6: "LPM_ERR_NO_DEVICE",
    -7: "LPM_ERR_STATE",
}


class LpmError(RuntimeError):
    """A liblpm_gpu call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_L = ctypes.POINTER(ctypes.c_int64)
_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_int = ctypes.c_int
_vp = ctypes.c_void_p
_pvp = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes (restype int unless listed in _RESTYPES)
_SIGNATURES = {
    "lpm_last_error_string": [],
    "lpm_version": [],
    "lpm_bve_velocity": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _D, _int],
    "lpm_bve_set_velocity_from_vorticity": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _D, _int],
    "lpm_plane_velocity": [_i64, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _int],
    "lpm_pse_sphere_laplacian": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _int, _i64, _i64, _D, _int],
    "lpm_pse_plane_laplacian": [_i64, _D, _D, _D, _D, _I, _dbl, _int, _i64, _i64, _D, _int],
    "lpm_bve_stream_functions": [_i64, _D, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _int],
    "lpm_pse_sphere_gradient": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _i64, _i64, _D, _D, _D, _int],
    "lpm_pse_sphere_divergence": [_i64, _D, _D, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _i64, _i64, _D, _int],
    "lpm_plane_stream_function": [_i64, _D, _D, _D, _D, _I, _i64, _i64, _D, _int],
    "lpm_beta_plane_velocity": [_i64, _D, _D, _D, _D, _I, _i64, _i64, _D, _D, _int],
    "lpm_beta_plane_stream_functions": [_i64, _D, _D, _D, _D, _D, _I, _i64, _i64, _D, _D, _int],
    "lpm_pse_plane_gradient": [_i64, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _int],
    "lpm_pse_plane_second_partials": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _D, _int],
    "lpm_pse_plane_double_dot": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _int],
    "lpm_pse_sphere_double_dot": [_i64, _D, _D, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _i64, _i64, _D, _int],
    "lpm_pse_interpolate_scalar": [_i64, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _int, _i64, _D, _D, _D, _D, _int],
    "lpm_swe_plane_rhs_integrals": [_i64, _D, _D, _D, _D, _D, _D, _I, _dbl, _i64, _i64, _D, _D, _D, _D, _int],
    "lpm_swe_sphere_rhs_integrals": [_i64, _D, _D, _D, _D, _D, _D, _D, _I, _dbl, _dbl, _dbl, _i64, _i64, _D, _D, _D,
                                     _D, _D, _int],
    "lpm_bve_solver_create": [_pvp, _i64, _D, _D, _D, _D, _D, _I, _D, _D, _D, _dbl, _dbl, _int],
    "lpm_bve_timestep": [_vp, _dbl, _int, _int],
    "lpm_bve_get_state": [_vp, _D, _D, _D, _D, _D, _D, _D],
    "lpm_bve_set_state": [_vp, _D, _D, _D, _D, _D, _D, _D],
    "lpm_bve_solver_remesh": [_vp, _i64, _D, _D, _D, _D, _D, _I, _D, _D, _D],
    "lpm_bve_diagnostics": [_vp, _D, _D, _D],
    "lpm_bve_kernel_timing": [_vp, _D, _L],
    "lpm_bve_solver_set_stream": [_vp, _vp],
    "lpm_bve_solver_stream_functions": [_vp, _D, _D, _D],
    "lpm_bve_solver_set_timing": [_vp, _int],
    "lpm_bve_solver_destroy": [_vp],
    "lpm_measure_fp32_peak": [_dbl, _D],
    "lpm_plane_solver_create": [_pvp, _i64, _D, _D, _D, _D, _I, _D, _D, _dbl, _int],
    "lpm_plane_solver_remesh": [_vp, _i64, _D, _D, _D, _D, _I, _D, _D],
    "lpm_plane_timestep": [_vp, _dbl, _int],
    "lpm_plane_get_state": [_vp, _D, _D, _D, _D],
    "lpm_plane_diagnostics": [_vp, _D, _D, _D],
    "lpm_plane_solver_destroy": [_vp],
    "lpm_ensemble_create": [_pvp, _int, _L, _D, _D, _D, _D, _D, _I, _D, _D, _int],
    "lpm_ensemble_timestep": [_vp, _dbl, _int, _int],
    "lpm_ensemble_velocity": [_vp],
    "lpm_ensemble_get_state": [_vp, _D, _D, _D, _D, _D, _D, _D],
    "lpm_ensemble_kernel_timing": [_vp, _D, _L],
    "lpm_ensemble_sweep_shape": [_vp, _I, _I, _I, _I],
    "lpm_ensemble_select_sweep": [_vp, _int, _int, _int],
    "lpm_ensemble_destroy": [_vp],
    "lpm_mesh_create": [_pvp, _int, _int, _dbl],
    "lpm_mesh_destroy": [_vp],
    "lpm_mesh_n_particles": [_vp],
    "lpm_mesh_n_active": [_vp],
    "lpm_mesh_n_faces": [_vp],
    "lpm_mesh_n_edges": [_vp],
    "lpm_mesh_n_leaf_edges": [_vp],
    "lpm_mesh_is_spherical": [_vp],
    "lpm_mesh_get_particles": [_vp, _D, _D, _D, _D, _I],
    "lpm_mesh_max_edge_length": [_vp],
    "lpm_mesh_avg_edge_length": [_vp],
    "lpm_release_workspace": [],
    "lpm_debug_fail_device_alloc": [_i64],
    "lpm_debug_inject_wait_timeout": [_i64, _i64],
}
_RESTYPES = {
    "lpm_last_error_string": ctypes.c_char_p,
    "lpm_version": ctypes.c_char_p,
    "lpm_mesh_destroy": None,
    "lpm_mesh_n_particles": _i64,
    "lpm_mesh_n_active": _i64,
    "lpm_mesh_n_faces": _i64,
    "lpm_mesh_n_edges": _i64,
    "lpm_mesh_n_leaf_edges": _i64,
    "lpm_mesh_max_edge_length": _dbl,
    "lpm_mesh_avg_edge_length": _dbl,
}

_LIB = None


def lib() -> ctypes.CDLL:
    """Loads liblpm_gpu.so (built by build.py).  Raises if it is missing: no fallback."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("LPM_GPU_LIB", LIB_PATH))
        if not path.exists():
            raise LpmError(-6, f"{path} is missing: build it with __graft_entry__.build() (no CPU fallback)")
        L = ctypes.CDLL(str(path))
        for name, args in _SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _LIB = L
    return _LIB


def version() -> str:
    return lib().lpm_version().decode()


def _check(rc: int) -> None:
    if rc != 0:
        msg = lib().lpm_last_error_string().decode(errors="replace")
        raise LpmError(rc, msg)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(np.asarray(a).astype(np.int32, copy=False))


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def _mode(mode) -> int:
    if isinstance(mode, str):
        return {"fp64": MODE_FP64, "fp32c": MODE_FP32C}[mode.lower()]
    return int(mode)


def _range(n, i_begin, i_end):
    ib = 1 if i_begin is None else int(i_begin)
    ie = n if i_end is None else int(i_end)
    return ib, ie


# ------------------------------------------------------------------ direct sums
def bve_sphere_velocity(x, y, z, rel_vort, area, active_mask, sphere_radius=1.0, i_begin=None, i_end=None,
                        mode="fp64", out=None):
    """BVESphereVelocity (src/SphereBVESolver.f90:377).  Returns (u, v, w) of length n; only
    entries i_begin..i_end (1-based, inclusive) are written."""
    x, y, z, rel_vort, area = (_f64(a) for a in (x, y, z, rel_vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    u, v, w = out if out is not None else (np.zeros(n), np.zeros(n), np.zeros(n))
    _check(lib().lpm_bve_velocity(n, _dp(x), _dp(y), _dp(z), _dp(rel_vort), _dp(area), _ip(act),
                                  float(sphere_radius), ib, ie, _dp(u), _dp(v), _dp(w), _mode(mode)))
    return u, v, w


def set_velocity_from_vorticity(x, y, z, rel_vort, area, active_mask, sphere_radius=1.0, i_begin=None,
                                i_end=None, mode="fp64"):
    """setVelocityFromVorticity (src/SphereBVE.f90:489)."""
    x, y, z, rel_vort, area = (_f64(a) for a in (x, y, z, rel_vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    u, v, w = np.zeros(n), np.zeros(n), np.zeros(n)
    _check(lib().lpm_bve_set_velocity_from_vorticity(n, _dp(x), _dp(y), _dp(z), _dp(rel_vort), _dp(area),
                                                     _ip(act), float(sphere_radius), ib, ie, _dp(u), _dp(v),
                                                     _dp(w), _mode(mode)))
    return u, v, w


def planar_incompressible_velocity(x, y, vort, area, active_mask, delta=0.0, i_begin=None, i_end=None,
                                   mode="fp64"):
    """planarIncompressibleVelocity (src/PlaneIncompressibleSolver.f90:278); delta = 0 is the
    reference kernel."""
    x, y, vort, area = (_f64(a) for a in (x, y, vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    u, v = np.zeros(n), np.zeros(n)
    _check(lib().lpm_plane_velocity(n, _dp(x), _dp(y), _dp(vort), _dp(area), _ip(act), float(delta), ib, ie,
                                    _dp(u), _dp(v), _mode(mode)))
    return u, v


def pse_sphere_laplacian_at_particles(x, y, z, f, area, active_mask, eps, sphere_radius=1.0,
                                      kernel=PSE_K8_GEODESIC, i_begin=None, i_end=None, mode="fp64"):
    """PSESphereLaplacianAtParticles (src/PSEDirectSum.f90:502)."""
    x, y, z, f, area = (_f64(a) for a in (x, y, z, f, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    lap = np.zeros(n)
    _check(lib().lpm_pse_sphere_laplacian(n, _dp(x), _dp(y), _dp(z), _dp(f), _dp(area), _ip(act), float(eps),
                                          float(sphere_radius), int(kernel), ib, ie, _dp(lap), _mode(mode)))
    return lap


def pse_plane_laplacian_at_particles(x, y, f, area, active_mask, eps, kernel=PSE_K8_CHORD, i_begin=None,
                                     i_end=None, mode="fp64"):
    """PSEPlaneLaplacianAtParticles (src/PSEDirectSum.f90:467)."""
    x, y, f, area = (_f64(a) for a in (x, y, f, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    lap = np.zeros(n)
    _check(lib().lpm_pse_plane_laplacian(n, _dp(x), _dp(y), _dp(f), _dp(area), _ip(act), float(eps), int(kernel),
                                         ib, ie, _dp(lap), _mode(mode)))
    return lap


def pse_sphere_gradient_at_particles(x, y, z, f, area, active_mask, eps, sphere_radius=1.0, i_begin=None,
                                     i_end=None, mode="fp64"):
    """PSESphereGradientAtParticles (src/PSEDirectSum.f90:220).  Returns (gx, gy, gz)."""
    x, y, z, f, area = (_f64(a) for a in (x, y, z, f, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    g = [np.zeros(n) for _ in range(3)]
    _check(lib().lpm_pse_sphere_gradient(n, _dp(x), _dp(y), _dp(z), _dp(f), _dp(area), _ip(act), float(eps),
                                         float(sphere_radius), ib, ie, *(_dp(a) for a in g), _mode(mode)))
    return tuple(g)


def pse_sphere_divergence_at_particles(x, y, z, vx, vy, vz, area, active_mask, eps, sphere_radius=1.0, i_begin=None,
                                       i_end=None, mode="fp64"):
    """PSESphereDivergenceAtParticles (src/PSEDirectSum.f90:537)."""
    x, y, z, vx, vy, vz, area = (_f64(a) for a in (x, y, z, vx, vy, vz, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    d = np.zeros(n)
    _check(lib().lpm_pse_sphere_divergence(n, _dp(x), _dp(y), _dp(z), _dp(vx), _dp(vy), _dp(vz), _dp(area),
                                           _ip(act), float(eps), float(sphere_radius), ib, ie, _dp(d), _mode(mode)))
    return d


def beta_plane_velocity(x, y, rel_vort, area, active_mask, i_begin=None, i_end=None, mode="fp64"):
    """BetaPlaneVelocity (src/BetaPlaneSolver.f90:227), the x-periodic sum.  Returns (u, v)."""
    x, y, rel_vort, area = (_f64(a) for a in (x, y, rel_vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    u, v = np.zeros(n), np.zeros(n)
    _check(lib().lpm_beta_plane_velocity(n, _dp(x), _dp(y), _dp(rel_vort), _dp(area), _ip(act), ib, ie, _dp(u),
                                         _dp(v), _mode(mode)))
    return u, v


def beta_plane_stream_functions(x, y, rel_vort, abs_vort, area, active_mask, i_begin=None, i_end=None, mode="fp64"):
    """The beta plane's SetStreamFunctionsOnMesh (src/BetaPlane.f90:399).  Returns (psi_rel, psi_abs)."""
    x, y, rel_vort, abs_vort, area = (_f64(a) for a in (x, y, rel_vort, abs_vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    pr, pa = np.zeros(n), np.zeros(n)
    _check(lib().lpm_beta_plane_stream_functions(n, _dp(x), _dp(y), _dp(rel_vort), _dp(abs_vort), _dp(area),
                                                 _ip(act), ib, ie, _dp(pr), _dp(pa), _mode(mode)))
    return pr, pa


def pse_plane_gradient_at_particles(x, y, f, area, active_mask, eps, i_begin=None, i_end=None, mode="fp64"):
    """PSEPlaneGradientAtParticles (src/PSEDirectSum.f90:180).  Returns (gx, gy)."""
    x, y, f, area = (_f64(a) for a in (x, y, f, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    gx, gy = np.zeros(n), np.zeros(n)
    _check(lib().lpm_pse_plane_gradient(n, _dp(x), _dp(y), _dp(f), _dp(area), _ip(act), float(eps), ib, ie, _dp(gx),
                                        _dp(gy), _mode(mode)))
    return gx, gy


def pse_plane_second_partials_at_particles(x, y, gx, gy, area, active_mask, eps, i_begin=None, i_end=None,
                                           mode="fp64"):
    """PSEPlaneSecondPartialsAtParticles (src/PSEDirectSum.f90:269).  Returns (dxx, dxy, dyy)."""
    x, y, gx, gy, area = (_f64(a) for a in (x, y, gx, gy, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    o = [np.zeros(n) for _ in range(3)]
    _check(lib().lpm_pse_plane_second_partials(n, _dp(x), _dp(y), _dp(gx), _dp(gy), _dp(area), _ip(act), float(eps),
                                               ib, ie, _dp(o[0]), _dp(o[1]), _dp(o[2]), _mode(mode)))
    return tuple(o)


def pse_plane_double_dot_product_at_particles(x, y, u, v, area, active_mask, eps, i_begin=None, i_end=None,
                                              mode="fp64"):
    """PSEPlaneDoubleDotProductAtParticles (src/PSEDirectSum.f90:322)."""
    x, y, u, v, area = (_f64(a) for a in (x, y, u, v, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    d = np.zeros(n)
    _check(lib().lpm_pse_plane_double_dot(n, _dp(x), _dp(y), _dp(u), _dp(v), _dp(area), _ip(act), float(eps), ib, ie,
                                          _dp(d), _mode(mode)))
    return d


def pse_sphere_double_dot_product_at_particles(x, y, z, u, v, w, area, active_mask, eps, sphere_radius=1.0,
                                               i_begin=None, i_end=None, mode="fp64"):
    """PSESphereDoubleDotProductAtParticles (src/PSEDirectSum.f90:367)."""
    x, y, z, u, v, w, area = (_f64(a) for a in (x, y, z, u, v, w, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    d = np.zeros(n)
    _check(lib().lpm_pse_sphere_double_dot(n, _dp(x), _dp(y), _dp(z), _dp(u), _dp(v), _dp(w), _dp(area), _ip(act),
                                           float(eps), float(sphere_radius), ib, ie, _dp(d), _mode(mode)))
    return d


GEOMETRY_PLANE = 0
GEOMETRY_SPHERE = 1


def pse_interpolate_scalar(x, y, z, f, area, active_mask, eps, qx, qy, qz=None, geometry=GEOMETRY_PLANE,
                           sphere_radius=1.0, mode="fp64"):
    """PSEPlaneInterpolateScalar / PSESphereInterpolateScalar (src/PSEDirectSum.f90:128-168) at
    every query point (qx, qy, qz) at once."""
    x, y, f, area = (_f64(a) for a in (x, y, f, area))
    act = _i32(active_mask)
    qx, qy = _f64(qx), _f64(qy)
    zp = None if z is None else _f64(z)
    qzp = None if qz is None else _f64(qz)
    out = np.zeros(qx.size)
    _check(lib().lpm_pse_interpolate_scalar(x.size, _dp(x), _dp(y), None if zp is None else _dp(zp), _dp(f),
                                            _dp(area), _ip(act), float(eps), float(sphere_radius), int(geometry),
                                            qx.size, _dp(qx), _dp(qy), None if qzp is None else _dp(qzp), _dp(out),
                                            _mode(mode)))
    return out


def swe_plane_rhs_integrals(x, y, vort, div, surf_height, area, active_mask, eps, i_begin=None, i_end=None,
                            mode="fp64"):
    """SWEPlaneRHSIntegrals (src/SWEPlaneSolver.f90:457), with surf_height = h + topoFn(x, y).
    Returns (u, v, doubleDot, lapSurf)."""
    x, y, vort, div, sh, area = (_f64(a) for a in (x, y, vort, div, surf_height, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    o = [np.zeros(n) for _ in range(4)]
    _check(lib().lpm_swe_plane_rhs_integrals(n, _dp(x), _dp(y), _dp(vort), _dp(div), _dp(sh), _dp(area), _ip(act),
                                             float(eps), ib, ie, _dp(o[0]), _dp(o[1]), _dp(o[2]), _dp(o[3]),
                                             _mode(mode)))
    return tuple(o)


def swe_sphere_rhs_integrals(x, y, z, rel_vort, div, surf_height, area, active_mask, radius, pse_eps,
                             sphere_radius=1.0, i_begin=None, i_end=None, mode="fp64"):
    """SWESphereRHSIntegrals (src/SphereSWESolver.f90:299), with surf_height = h + topoFn(x, y, z)
    and sphere_radius the SphereRadius of SphereDistance.  Returns (u, v, w, doubleDot, lapSurf)."""
    x, y, z, rel_vort, div, sh, area = (_f64(a) for a in (x, y, z, rel_vort, div, surf_height, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    o = [np.zeros(n) for _ in range(5)]
    _check(lib().lpm_swe_sphere_rhs_integrals(n, _dp(x), _dp(y), _dp(z), _dp(rel_vort), _dp(div), _dp(sh), _dp(area),
                                              _ip(act), float(radius), float(sphere_radius), float(pse_eps), ib, ie,
                                              _dp(o[0]), _dp(o[1]), _dp(o[2]), _dp(o[3]), _dp(o[4]), _mode(mode)))
    return tuple(o)


def set_stream_functions_on_mesh(x, y, z, rel_vort, abs_vort, area, active_mask, sphere_radius=1.0, i_begin=None,
                                 i_end=None, mode="fp64"):
    """SetStreamFunctionsOnMesh (src/SphereBVE.f90:445).  Returns (psi_rel, psi_abs)."""
    x, y, z, rel_vort, abs_vort, area = (_f64(a) for a in (x, y, z, rel_vort, abs_vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    pr, pa = np.zeros(n), np.zeros(n)
    _check(lib().lpm_bve_stream_functions(n, _dp(x), _dp(y), _dp(z), _dp(rel_vort), _dp(abs_vort), _dp(area),
                                          _ip(act), float(sphere_radius), ib, ie, _dp(pr), _dp(pa), _mode(mode)))
    return pr, pa


def set_stream_function_on_mesh(x, y, vort, area, active_mask, i_begin=None, i_end=None, mode="fp64"):
    """SetStreamFunctionOnMesh (src/PlanarIncompressible.f90:470)."""
    x, y, vort, area = (_f64(a) for a in (x, y, vort, area))
    act = _i32(active_mask)
    n = x.size
    ib, ie = _range(n, i_begin, i_end)
    p = np.zeros(n)
    _check(lib().lpm_plane_stream_function(n, _dp(x), _dp(y), _dp(vort), _dp(area), _ip(act), ib, ie, _dp(p),
                                           _mode(mode)))
    return p


# ------------------------------------------------------------------ solvers
class BVESolver:
    """Device-resident BVESolver (src/SphereBVESolver.f90:38-353)."""

    def __init__(self, x, y, z, rel_vort, area, active_mask, radius=1.0, rotation_rate=0.0, u=None, v=None, w=None,
                 mode="fp64"):
        arrs = [_f64(a) for a in (x, y, z, rel_vort, area)]
        self.n = arrs[0].size
        self._keep = arrs
        act = _i32(active_mask)
        uvw = [None if a is None else _f64(a) for a in (u, v, w)]
        h = ctypes.c_void_p()
        _check(lib().lpm_bve_solver_create(ctypes.byref(h), self.n, *(_dp(a) for a in arrs), _ip(act),
                                           *(_dp(a) for a in uvw), float(radius), float(rotation_rate), _mode(mode)))
        self._h = h

    def timestep(self, dt, n_steps=1, renormalize=False):
        _check(lib().lpm_bve_timestep(self._h, float(dt), int(n_steps), 1 if renormalize else 0))

    def get_state(self):
        out = [np.empty(self.n) for _ in range(7)]
        _check(lib().lpm_bve_get_state(self._h, *(_dp(a) for a in out)))
        return dict(zip(("x", "y", "z", "rel_vort", "u", "v", "w"), out))

    def set_state(self, x, y, z, rel_vort, u, v, w):
        arrs = [_f64(a) for a in (x, y, z, rel_vort, u, v, w)]
        _check(lib().lpm_bve_set_state(self._h, *(_dp(a) for a in arrs)))

    def remesh(self, x, y, z, rel_vort, area, active_mask, u=None, v=None, w=None):
        """Loads a remeshed particle set in place of Delete(solver) + New(solver, sphere)."""
        arrs = [_f64(a) for a in (x, y, z, rel_vort, area)]
        act = _i32(active_mask)
        uvw = [None if a is None else _f64(a) for a in (u, v, w)]
        _check(lib().lpm_bve_solver_remesh(self._h, arrs[0].size, *(_dp(a) for a in arrs), _ip(act),
                                           *(_dp(a) for a in uvw)))
        self.n = arrs[0].size
        self._keep = arrs

    def diagnostics(self):
        ke, en, ci = _dbl(), _dbl(), _dbl()
        _check(lib().lpm_bve_diagnostics(self._h, ctypes.byref(ke), ctypes.byref(en), ctypes.byref(ci)))
        return {"kinetic_energy": ke.value, "enstrophy": en.value, "circulation": ci.value}

    def stream_functions(self, abs_vort=None):
        """SetStreamFunctionsOnMesh (src/SphereBVE.f90:445) at the current state, as the
        reference's Timestep calls it after each step.  Returns (psi_rel, psi_abs)."""
        pr, pa = np.empty(self.n), np.empty(self.n)
        av = None if abs_vort is None else _f64(abs_vort)
        _check(lib().lpm_bve_solver_stream_functions(self._h, None if av is None else _dp(av), _dp(pr), _dp(pa)))
        return pr, pa

    def kernel_timing(self):
        ms, n = _dbl(), _i64()
        _check(lib().lpm_bve_kernel_timing(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_timing(self, enable: bool):
        """True (default): synchronise after each step to accumulate kernel timing."""
        _check(lib().lpm_bve_solver_set_timing(self._h, 1 if enable else 0))

    def set_stream(self, stream_handle: int | None):
        """Enqueue the solver's work on a caller's cudaStream_t (an integer handle)."""
        _check(lib().lpm_bve_solver_set_stream(self._h, ctypes.c_void_p(stream_handle or None)))

    def close(self):
        if getattr(self, "_h", None):
            lib().lpm_bve_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlaneSolver:
    """Device-resident PlaneSolver (src/PlaneIncompressibleSolver.f90:103-259)."""

    def __init__(self, x, y, vort, area, active_mask, u=None, v=None, delta=0.0, mode="fp64"):
        arrs = [_f64(a) for a in (x, y, vort, area)]
        self.n = arrs[0].size
        self._keep = arrs
        act = _i32(active_mask)
        uv = [None if a is None else _f64(a) for a in (u, v)]
        h = ctypes.c_void_p()
        _check(lib().lpm_plane_solver_create(ctypes.byref(h), self.n, *(_dp(a) for a in arrs), _ip(act),
                                             *(_dp(a) for a in uv), float(delta), _mode(mode)))
        self._h = h

    def timestep(self, dt, n_steps=1):
        _check(lib().lpm_plane_timestep(self._h, float(dt), int(n_steps)))

    def get_state(self):
        out = [np.empty(self.n) for _ in range(4)]
        _check(lib().lpm_plane_get_state(self._h, *(_dp(a) for a in out)))
        return dict(zip(("x", "y", "u", "v"), out))

    def remesh(self, x, y, vort, area, active_mask, u=None, v=None):
        """Loads a remeshed particle set in place of Delete(solver) + New(solver, plane)."""
        arrs = [_f64(a) for a in (x, y, vort, area)]
        act = _i32(active_mask)
        uv = [None if a is None else _f64(a) for a in (u, v)]
        _check(lib().lpm_plane_solver_remesh(self._h, arrs[0].size, *(_dp(a) for a in arrs), _ip(act),
                                             *(_dp(a) for a in uv)))
        self.n = arrs[0].size
        self._keep = arrs

    def diagnostics(self):
        ke, en, ci = _dbl(), _dbl(), _dbl()
        _check(lib().lpm_plane_diagnostics(self._h, ctypes.byref(ke), ctypes.byref(en), ctypes.byref(ci)))
        return {"kinetic_energy": ke.value, "enstrophy": en.value, "circulation": ci.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().lpm_plane_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Batched independent sphere-BVE instances (one persistent launch per RK4 stage)."""

    def __init__(self, instances, mode="fp32c"):
        """instances: list of dicts with x, y, z, rel_vort, area, active, radius, rotation_rate."""
        self.sizes = [int(np.asarray(d["x"]).size) for d in instances]
        offs = np.zeros(len(instances) + 1, dtype=np.int64)
        offs[1:] = np.cumsum(self.sizes)
        self.offsets = offs
        cat = {k: _f64(np.concatenate([np.asarray(d[k], dtype=np.float64) for d in instances]))
               for k in ("x", "y", "z", "rel_vort", "area")}
        act = _i32(np.concatenate([np.asarray(d["active"]) for d in instances]))
        radius = _f64([d.get("radius", 1.0) for d in instances])
        rot = _f64([d.get("rotation_rate", 0.0) for d in instances])
        self._keep = (cat, act, radius, rot)
        h = ctypes.c_void_p()
        _check(lib().lpm_ensemble_create(ctypes.byref(h), len(instances), offs.ctypes.data_as(_L), _dp(cat["x"]),
                                         _dp(cat["y"]), _dp(cat["z"]), _dp(cat["rel_vort"]), _dp(cat["area"]),
                                         _ip(act), _dp(radius), _dp(rot), _mode(mode)))
        self._h = h
        self.n = int(offs[-1])

    def timestep(self, dt, n_steps=1, renormalize=False):
        _check(lib().lpm_ensemble_timestep(self._h, float(dt), int(n_steps), 1 if renormalize else 0))

    def velocity(self):
        _check(lib().lpm_ensemble_velocity(self._h))

    def get_state(self):
        out = [np.empty(self.n) for _ in range(7)]
        _check(lib().lpm_ensemble_get_state(self._h, *(_dp(a) for a in out)))
        return dict(zip(("x", "y", "z", "rel_vort", "u", "v", "w"), out))

    def kernel_timing(self):
        ms, n = _dbl(), _i64()
        _check(lib().lpm_ensemble_kernel_timing(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def sweep_shape(self):
        """(threads, targets per thread, CTAs per SM, items per CTA slot) the tuner chose."""
        v = [ctypes.c_int32() for _ in range(4)]
        _check(lib().lpm_ensemble_sweep_shape(self._h, *(ctypes.byref(q) for q in v)))
        return tuple(q.value for q in v)

    def select_sweep(self, threads, targets_per_thread, items_per_slot):
        """Replaces the autotuner's choice of the persistent sweep's configuration."""
        _check(lib().lpm_ensemble_select_sweep(self._h, int(threads), int(targets_per_thread), int(items_per_slot)))

    def close(self):
        if getattr(self, "_h", None):
            lib().lpm_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def release_workspace() -> None:
    """Frees the device workspace the host-buffer calls keep between calls."""
    _check(lib().lpm_release_workspace())


def debug_fail_device_alloc(k: int) -> None:
    """Test hook: the k-th device allocation from now on fails (0 disarms)."""
    _check(lib().lpm_debug_fail_device_alloc(int(k)))


def debug_inject_wait_timeout(skip_tile: int, budget_ns: int) -> None:
    """Test hook: the next host-buffer sphere-BVE or sphere PSE FP32C sum skips the copy of one
    source tile and bounds its waits by budget_ns, so it returns LPM_ERR_TIMEOUT (one-shot)."""
    _check(lib().lpm_debug_inject_wait_timeout(int(skip_tile), int(budget_ns)))


def measure_fp32_peak(ms_target: float = 200.0) -> float:
    """Measured FP32 FMA throughput of the current GPU in TFLOP/s."""
    t = _dbl()
    _check(lib().lpm_measure_fp32_peak(float(ms_target), ctypes.byref(t)))
    return t.value


# ------------------------------------------------------------------ meshes
class PolyMesh2d:
    """Uniformly refined lpm-v2 mesh (New(PolyMesh2d, seed, initNest, ...), src/PolyMesh2d.f90:135)."""

    def __init__(self, mesh_seed: int, init_nest: int, amp_factor: float = 1.0):
        h = ctypes.c_void_p()
        _check(lib().lpm_mesh_create(ctypes.byref(h), int(mesh_seed), int(init_nest), float(amp_factor)))
        self._h = h
        L = lib()
        self.n = int(L.lpm_mesh_n_particles(h))
        self.spherical = bool(L.lpm_mesh_is_spherical(h))
        self.x = np.empty(self.n)
        self.y = np.empty(self.n)
        self.z = np.zeros(self.n)
        self.area = np.empty(self.n)
        self.active = np.empty(self.n, dtype=np.int32)
        _check(L.lpm_mesh_get_particles(h, _dp(self.x), _dp(self.y), _dp(self.z) if self.spherical else None,
                                        _dp(self.area), _ip(self.active)))
        self.n_active = int(L.lpm_mesh_n_active(h))
        self.n_faces = int(L.lpm_mesh_n_faces(h))
        self.n_edges = int(L.lpm_mesh_n_edges(h))
        self.n_leaf_edges = int(L.lpm_mesh_n_leaf_edges(h))
        self.max_edge_length = float(L.lpm_mesh_max_edge_length(h))
        self.avg_edge_length = float(L.lpm_mesh_avg_edge_length(h))
        L.lpm_mesh_destroy(h)
        self._h = None
