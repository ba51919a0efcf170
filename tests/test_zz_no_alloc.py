"""GPU test of lpm_bve_velocity_noalloc, the allocation-free sphere-BVE entry point.

That entry point is for callers that cannot allocate device memory while they run -- for
example a host code whose own pool allocator already owns the GPU's memory, or a time loop
that must not pay the device-wide synchronisation of cudaMalloc/cudaFree.  They own all
inputs and outputs; the library keeps its scratch in one fixed device array.

The test allocates the device arrays itself (with torch, as such a caller would with its own
allocator) and calls the entry point through the C ABI twice in a row -- a larger problem,
then a smaller one on a sub-block of targets, so the shared scratch array holds the first
call's contents when the second call starts.  Each result is checked against the oracle
(the reference's BVESphereVelocity loop restated on the CPU) and against the allocating entry
point lpm_bve_velocity in LPM_MODE_FP32C, to the FP32C tolerance used throughout the tests,
1e-6 relative L-infinity.  A warm call must leave the device's free
memory unchanged, and the largest accepted problem (LPM_NOALLOC_MAX_PARTICLES particles, every
one a target) must fit the fixed scratch.  The file is collected last, so a run that stops at
the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32C_TOL = 1e-6
MAX_PARTICLES = 262144  # LPM_NOALLOC_MAX_PARTICLES in include/lpm_gpu.h
_D = ctypes.c_void_p


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


def _noalloc(lg):
    fn = lg.lib().lpm_bve_velocity_noalloc
    fn.argtypes = [ctypes.c_int64, _D, _D, _D, _D, _D, _D, ctypes.c_double, ctypes.c_int64, ctypes.c_int64, _D, _D, _D,
                   _D]
    fn.restype = ctypes.c_int
    return fn


def _device_inputs(torch, c):
    dev = {k: torch.from_numpy(np.ascontiguousarray(c[k], dtype=np.float64)).cuda() for k in ("x", "y", "z", "zeta",
                                                                                              "area")}
    dev["active"] = torch.from_numpy(np.ascontiguousarray(c["active"], dtype=np.int32)).cuda()
    return dev


def _call(lg, torch, c, i_begin, i_end, free_before_after=None):
    n = c["x"].size
    dev = _device_inputs(torch, c)
    out = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(3)]
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = _noalloc(lg)(n, dev["x"].data_ptr(), dev["y"].data_ptr(), dev["z"].data_ptr(), dev["zeta"].data_ptr(),
                      dev["area"].data_ptr(), dev["active"].data_ptr(), c["radius"], i_begin, i_end,
                      out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), stream)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert rc == 0, lg.lib().lpm_last_error_string().decode()
    if free_before_after is not None:
        free_before_after.append((free0, free1))
    return [o.cpu().numpy() for o in out]


def _oracle_block(oracle_mod, c, ib, ie):
    """The oracle's velocity for 1-based targets ib..ie."""
    return oracle_mod.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], c["radius"],
                                   ib=ib - 1, ie=ie)


def test_noalloc_matches_oracle_and_entry_point_twice(lg, oracle_mod):
    torch = pytest.importorskip("torch")
    import workloads as wl
    cases = [(wl.config_rh54_icos(5, seed=2), None), (wl.config_gauss_vortex_icos(4), (1001, 5500))]
    mem = []
    for c, block in cases:
        n = c["x"].size
        ib, ie = block if block else (1, n)
        got = _call(lg, torch, c, ib, ie, mem)
        g = np.stack([a[ib - 1:ie] for a in got])
        # against the oracle (FP64) ...
        r = np.stack(_oracle_block(oracle_mod, c, ib, ie))
        assert np.abs(g - r).max() / np.abs(r).max() <= FP32C_TOL
        # ... and against the allocating entry point lpm_bve_velocity in LPM_MODE_FP32C
        e = lg.bve_sphere_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], c["radius"],
                                   i_begin=ib, i_end=ie, mode="fp32c")
        e = np.stack([a[ib - 1:ie] for a in e])
        assert np.abs(g - e).max() / np.abs(e).max() <= FP32C_TOL
        for a in got:  # entries outside the block are left as they were
            assert np.all(a[:ib - 1] == 7.0) and np.all(a[ie:] == 7.0)
    # the second call came after the first had loaded the module and reserved the scratch:
    # it allocated nothing on the device
    assert mem[1][0] == mem[1][1], mem


def test_noalloc_largest_problem(lg, oracle_mod):
    """n = LPM_NOALLOC_MAX_PARTICLES with every particle a target: the records and the FP64
    partial sums fit the fixed scratch, and a block of the result matches the oracle."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    n = MAX_PARTICLES
    p = rng.normal(size=(3, n))
    p /= np.linalg.norm(p, axis=0)
    active = (rng.random(n) < 0.66).astype(np.int32)
    zeta = 2.0 * p[2] + np.cos(3.0 * p[0]) * p[1]
    area = np.where(active == 1, 4.0 * np.pi / active.sum(), 0.0)
    c = dict(x=p[0], y=p[1], z=p[2], zeta=zeta, area=area, active=active, radius=1.0)
    got = _call(lg, torch, c, 1, n)
    for ib in (1, n // 2, n - 2047):
        ie = ib + 2047
        ref = np.stack(_oracle_block(oracle_mod, c, ib, ie))
        g = np.stack([a[ib - 1:ie] for a in got])
        assert np.abs(g - ref).max() / np.abs(ref).max() <= FP32C_TOL


def test_noalloc_rejects_oversized_problem(lg):
    n = MAX_PARTICLES + 1
    rc = _noalloc(lg)(n, 1, 1, 1, 1, 1, 1, 1.0, 1, n, 1, 1, 1, None)
    assert rc == -1
    assert "at most" in lg.lib().lpm_last_error_string().decode()
