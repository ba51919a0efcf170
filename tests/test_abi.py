"""CPU tests of the C ABI: the library loads, exports every function include/*.h declares,
and rejects bad arguments before touching a GPU; without a GPU a valid call fails loudly."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions():
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(lpm_[a-z0-9_]+)\s*\(", text):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("lpm_bve_velocity", "lpm_plane_velocity", "lpm_pse_sphere_laplacian", "lpm_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(str(built_lib.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_version(built_lib):
    assert "sm_103a" in built_lib.version()


def _tiny():
    x = np.array([1.0, 0.0, 0.0])
    y = np.array([0.0, 1.0, 0.0])
    z = np.array([0.0, 0.0, 1.0])
    return x, y, z, np.ones(3), np.full(3, 0.1), np.array([1, 1, 0], dtype=np.int32)


@pytest.mark.parametrize("kw", [dict(i_begin=0), dict(i_end=4), dict(i_begin=3, i_end=2), dict(mode=7),
                                dict(mode=0x1000), dict(sphere_radius=0.0)])
def test_bad_arguments_rejected(built_lib, kw):
    x, y, z, zeta, area, act = _tiny()
    with pytest.raises(built_lib.LpmError) as e:
        built_lib.bve_sphere_velocity(x, y, z, zeta, area, act, **kw)
    assert e.value.code == -1


def test_empty_input_rejected(built_lib):
    e = np.zeros(0)
    with pytest.raises(built_lib.LpmError) as ex:
        built_lib.bve_sphere_velocity(e, e, e, e, e, np.zeros(0, np.int32))
    assert ex.value.code == -1


def test_plane_negative_delta_rejected(built_lib):
    x, y, _, w, a, act = _tiny()
    with pytest.raises(built_lib.LpmError) as e:
        built_lib.planar_incompressible_velocity(x, y, w, a, act, delta=-1.0)
    assert e.value.code == -1


def test_pse_bad_kernel_rejected(built_lib):
    x, y, z, f, a, act = _tiny()
    with pytest.raises(built_lib.LpmError):
        built_lib.pse_sphere_laplacian_at_particles(x, y, z, f, a, act, 0.1, kernel=9)
    with pytest.raises(built_lib.LpmError):
        built_lib.pse_plane_laplacian_at_particles(x, y, f, a, act, 0.1, kernel=0)


def test_stream_bad_radius_rejected(built_lib):
    x, y, z, f, a, act = _tiny()
    with pytest.raises(built_lib.LpmError) as e:
        built_lib.set_stream_functions_on_mesh(x, y, z, f, f, a, act, sphere_radius=0.0, mode="fp32c")
    assert e.value.code == -1


def test_no_gpu_fails_loudly(built_lib):
    """Without a GPU a valid call returns LPM_ERR_NO_DEVICE (or CUDA error): no CPU fallback."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    x, y, z, zeta, area, act = _tiny()
    with pytest.raises(built_lib.LpmError) as e:
        built_lib.bve_sphere_velocity(x, y, z, zeta, area, act)
    assert e.value.code in (-6, -2)


@pytest.mark.parametrize("call", ["pse_plane_grad", "pse_plane_second", "pse_plane_ddot", "pse_sphere_ddot",
                                  "pse_sphere_grad", "pse_sphere_div", "swe_plane", "swe_sphere", "beta",
                                  "beta_stream", "interp_geometry", "interp_sphere_no_z", "interp_no_points"])
def test_operator_argument_checks(built_lib, call):
    """Bad eps, radius, block or geometry arguments of the PSE, SWE and beta-plane entry points
    fail with LPM_ERR_ARG before any device work (so they also fail this way without a GPU)."""
    lg = built_lib
    x, y, z, f, a, act = _tiny()
    fn = {
        "pse_plane_grad": lambda: lg.pse_plane_gradient_at_particles(x, y, f, a, act, 0.0),
        "pse_plane_second": lambda: lg.pse_plane_second_partials_at_particles(x, y, f, f, a, act, -1.0),
        "pse_plane_ddot": lambda: lg.pse_plane_double_dot_product_at_particles(x, y, f, f, a, act, 0.1, i_end=5),
        "pse_sphere_ddot": lambda: lg.pse_sphere_double_dot_product_at_particles(x, y, z, f, f, f, a, act, 0.1,
                                                                                  sphere_radius=0.0),
        "pse_sphere_grad": lambda: lg.pse_sphere_gradient_at_particles(x, y, z, f, a, act, 0.0),
        "pse_sphere_div": lambda: lg.pse_sphere_divergence_at_particles(x, y, z, f, f, f, a, act, 0.1, i_begin=0),
        "swe_plane": lambda: lg.swe_plane_rhs_integrals(x, y, f, f, f, a, act, 0.0),
        "swe_sphere": lambda: lg.swe_sphere_rhs_integrals(x, y, z, f, f, f, a, act, 1.0, 0.1, sphere_radius=-1.0),
        "beta": lambda: lg.beta_plane_velocity(x, y, f, a, act, i_begin=2, i_end=1),
        "beta_stream": lambda: lg.beta_plane_stream_functions(x, y, f, f, a, act, mode="fp16"),
        "interp_geometry": lambda: lg.pse_interpolate_scalar(x, y, None, f, a, act, 0.1, x[:1], y[:1], geometry=3),
        "interp_sphere_no_z": lambda: lg.pse_interpolate_scalar(x, y, None, f, a, act, 0.1, x[:1], y[:1],
                                                                geometry=lg.GEOMETRY_SPHERE),
        "interp_no_points": lambda: lg.pse_interpolate_scalar(x, y, None, f, a, act, 0.1, x[:0], y[:0]),
    }[call]
    with pytest.raises((lg.LpmError, ValueError, KeyError)) as e:
        fn()
    if isinstance(e.value, lg.LpmError):
        assert e.value.code == -1


def test_particle_count_above_32_bit_indices_rejected(built_lib):
    """n above 2^31 - 1 is refused before any array is read or any device is touched: the
    source lists, sort values and curve orders hold 32-bit particle indices."""
    L = built_lib.lib()
    dp, ip = built_lib._dp, built_lib._ip
    x, y, z, zeta, area, act = _tiny()
    out = np.zeros(3)
    big = 2 ** 31
    rc = L.lpm_bve_velocity(big, dp(x), dp(y), dp(z), dp(zeta), dp(area), ip(act), 1.0, 1, 1, dp(out), dp(out),
                            dp(out), 0)
    assert rc == -1 and "32-bit" in L.lpm_last_error_string().decode()
    rc = L.lpm_plane_velocity(big, dp(x), dp(y), dp(zeta), dp(area), ip(act), 0.0, 1, 1, dp(out), dp(out), 0)
    assert rc == -1
    h = ctypes.c_void_p()
    rc = L.lpm_bve_solver_create(ctypes.byref(h), big, dp(x), dp(y), dp(z), dp(zeta), dp(area), ip(act), None, None,
                                 None, 1.0, 0.0, 0)
    assert rc == -1 and not h.value
    rc = L.lpm_plane_solver_create(ctypes.byref(h), big, dp(x), dp(y), dp(zeta), dp(area), ip(act), None, None, 0.0,
                                   0)
    assert rc == -1 and not h.value
    rc = L.lpm_pse_interpolate_scalar(3, dp(x), dp(y), dp(z), dp(zeta), dp(area), ip(act), 0.1, 1.0, 1, big - 2,
                                      dp(x), dp(y), dp(z), dp(out), 0)
    assert rc == -1


def _c_prototypes():
    """name -> (return type, [(base type, pointer depth)]) for every function include/*.h declares."""
    out = {}
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", " ", h.read_text(), flags=re.S)
        text = re.sub(r"^\s*#.*$", " ", text, flags=re.M)
        for m in re.finditer(r"([\w\s\*]+?)\b(lpm_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
            params = m.group(3).strip()
            plist = []
            if params not in ("", "void"):
                for p in params.split(","):
                    p = p.replace("const", " ").strip()
                    plist.append((p.replace("*", " ").split()[0], p.count("*")))
            ret = " ".join(m.group(1).split()[-2:]) if "*" in m.group(1) else m.group(1).split()[-1]
            out[m.group(2)] = (ret.replace("const", "").strip(), plist)
    return out


def test_ctypes_signatures_match_the_headers(built_lib):
    """The Python binding's argtypes and restypes against the C prototypes, parameter by
    parameter: int64_t <-> c_int64, int <-> c_int, double <-> c_double, double* / int32_t* /
    int64_t* <-> POINTER of the same, a handle or void* <-> c_void_p, a handle** <->
    POINTER(c_void_p).  ctypes converts whatever it is told, so a wrong entry here would pass
    a wrong value rather than fail."""
    lg = built_lib
    scalar = {"int64_t": ctypes.c_int64, "int": ctypes.c_int, "double": ctypes.c_double}
    pointee = {"double": ctypes.c_double, "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "int": ctypes.c_int}
    protos = _c_prototypes()
    assert set(lg._SIGNATURES) <= set(protos), set(lg._SIGNATURES) - set(protos)
    checked = 0
    for name, argtypes in lg._SIGNATURES.items():
        ret, params = protos[name]
        assert len(argtypes) == len(params), name
        for k, (t, (base, depth)) in enumerate(zip(argtypes, params)):
            if depth == 0:
                want = scalar[base]
            elif depth == 1 and (base.startswith("lpm_") or base == "void"):
                want = ctypes.c_void_p
            elif depth == 1:
                want = ctypes.POINTER(pointee[base])
            else:
                want = ctypes.POINTER(ctypes.c_void_p)
            assert t is want, f"{name} argument {k + 1}: {t} for C {base}{'*' * depth}"
            checked += 1
        rt = lg._RESTYPES.get(name, ctypes.c_int)
        want_rt = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "double": ctypes.c_double, "void": None,
                   "char*": ctypes.c_char_p}[ret.replace(" ", "")]
        assert rt is want_rt, f"{name} returns {ret}, bound as {rt}"
    assert checked > 300
