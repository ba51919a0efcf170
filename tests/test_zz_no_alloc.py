"""GPU test of lpm_bve_velocity_noalloc, the allocation-free sphere-BVE entry point.

That entry point is for callers that cannot allocate device memory while they run -- for
example a host code whose own pool allocator already owns the GPU's memory, or a time loop
that must not pay the device-wide synchronisation of cudaMalloc/cudaFree.  They own all
inputs and outputs; the library keeps its scratch in one array reserved at load time.

The test allocates the device arrays itself (with torch, as such a caller would with its own
allocator), calls the entry point through the C ABI twice in a row -- a larger problem, then
a smaller one on a sub-block of targets, so the shared scratch array holds the first call's
contents when the second call starts -- and checks each result against lpm_bve_velocity in
LPM_MODE_FP32C to the FP32C tolerance used throughout the tests (1e-6 relative L-infinity).
It is collected last, so a run that stops at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32C_TOL = 1e-6
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


def _call(lg, torch, c, i_begin, i_end):
    n = c["x"].size
    dev = {k: torch.from_numpy(np.ascontiguousarray(c[k], dtype=np.float64)).cuda() for k in ("x", "y", "z", "zeta",
                                                                                              "area")}
    act = torch.from_numpy(np.ascontiguousarray(c["active"], dtype=np.int32)).cuda()
    out = [torch.full((n,), 7.0, dtype=torch.float64, device="cuda") for _ in range(3)]
    stream = torch.cuda.current_stream().cuda_stream
    rc = _noalloc(lg)(n, dev["x"].data_ptr(), dev["y"].data_ptr(), dev["z"].data_ptr(), dev["zeta"].data_ptr(),
                      dev["area"].data_ptr(), act.data_ptr(), c["radius"], i_begin, i_end, out[0].data_ptr(),
                      out[1].data_ptr(), out[2].data_ptr(), stream)
    assert rc == 0, lg.lib().lpm_last_error_string().decode()
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in out]


def test_noalloc_matches_fp32c_entry_point_twice(lg):
    torch = pytest.importorskip("torch")
    import workloads as wl
    cases = [(wl.config_rh54_icos(5, seed=2), None), (wl.config_gauss_vortex_icos(4), (1001, 5500))]
    for c, block in cases:
        n = c["x"].size
        ib, ie = block if block else (1, n)
        got = _call(lg, torch, c, ib, ie)
        ref = lg.bve_sphere_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], c["radius"],
                                     i_begin=ib, i_end=ie, mode="fp32c")
        g = np.stack([a[ib - 1:ie] for a in got])
        r = np.stack([a[ib - 1:ie] for a in ref])
        assert np.abs(g - r).max() / np.abs(r).max() <= FP32C_TOL
        for a in got:  # entries outside the block are left as they were
            assert np.all(a[:ib - 1] == 7.0) and np.all(a[ie:] == 7.0)


def test_noalloc_rejects_oversized_problem(lg):
    n = 262144 + 1
    rc = _noalloc(lg)(n, 1, 1, 1, 1, 1, 1, 1.0, 1, n, 1, 1, 1, None)
    assert rc == -1
    assert "at most" in lg.lib().lpm_last_error_string().decode()
