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
