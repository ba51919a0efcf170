"""GPU tests of the error paths, with failures made on purpose but no GPU fault.

The reference reports failures through its logger (LogMessage at ERROR_LOGGING_LEVEL,
src/Logger.f90:159), which the Fortran shim calls on any non-zero status.  These tests make
the library's two kinds of failure happen without faulting, trapping or hanging a GPU:

* A bounded device wait that runs out: lpm_debug_inject_wait_timeout makes the next
  host-buffer sphere-BVE or sphere PSE FP32C sum (the block-synchronous and the
  warp-decoupled tile pipelines) skip the copy of one source tile and bounds its waits by
  1 ms.  The waits for that tile give up, the call returns LPM_ERR_TIMEOUT with the caller's
  outputs untouched, and the next call on the same context is correct.  No copy is ever in
  flight for the skipped tile, so nothing is left to land after the CTA has gone.
* A device allocation that fails: lpm_debug_fail_device_alloc makes the k-th allocation of
  the library fail as if cudaMalloc had run out of memory.  For every k up to the number of
  allocations an entry point makes, the call returns LPM_ERR_ALLOC with a message, leaks no
  device memory, and the next call succeeds with correct results.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LPM_ERR_TIMEOUT = -3
LPM_ERR_ALLOC = -5
LPM_MODE_FP32C = 1
FP32C_TOL = 1e-6


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def wl(built_lib):
    import workloads
    return workloads


def _rel_linf(got, ref):
    got, ref = np.stack(got), np.stack(ref)
    return float(np.abs(got - ref).max() / np.abs(ref).max())


def test_bounded_wait_runs_out_and_context_survives(lg, wl, oracle_mod):
    c = wl.config_gauss_vortex_icos(4)  # 5,120 sources: 20 tiles of 256
    a = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    ref = oracle_mod.bve_velocity(*a, 1.0)
    lg.bve_sphere_velocity(*a, 1.0, mode="fp32c")  # the autotuner times this size class first
    n = c["x"].size
    x, y, z, zeta, area = (np.ascontiguousarray(q, dtype=np.float64) for q in a[:5])
    act = np.ascontiguousarray(c["active"], dtype=np.int32)
    out = [np.full(n, 7.0) for _ in range(3)]
    P = ctypes.POINTER(ctypes.c_double)
    lg.debug_inject_wait_timeout(3, 1_000_000)
    rc = lg.lib().lpm_bve_velocity(n, *(q.ctypes.data_as(P) for q in (x, y, z, zeta, area)),
                                   act.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 1.0, 1, n,
                                   *(q.ctypes.data_as(P) for q in out), LPM_MODE_FP32C)
    assert rc == LPM_ERR_TIMEOUT, lg.lib().lpm_last_error_string().decode()
    assert "wait" in lg.lib().lpm_last_error_string().decode()
    for q in out:
        assert np.all(q == 7.0)  # an error return leaves the outputs as they were
    # the same context, the next call: correct
    got = lg.bve_sphere_velocity(*a, 1.0, mode="fp32c")
    assert _rel_linf(got, ref) <= FP32C_TOL
    got64 = lg.bve_sphere_velocity(*a, 1.0, mode="fp64")
    for g, r in zip(got64, ref):
        assert np.array_equal(g, r)


@pytest.mark.parametrize("skip_tile", [0, 3])
def test_bounded_wait_runs_out_warp_decoupled_pipeline(lg, wl, oracle_mod, skip_tile):
    """The same on the warp-decoupled pipeline of the PSE sweeps: every warp of the CTAs that
    own the skipped tile gives up on it, thread 0's bounded waits for the stages end, the copies
    of the other stages are waited for, and the call returns LPM_ERR_TIMEOUT with the output
    untouched; the next call is within the PSE FP32C bound of the oracle."""
    c = wl.config_pse_cubed(4)
    a = (c["x"], c["y"], c["z"], c["f"], c["area"], c["active"])
    ref = oracle_mod.pse_laplacian(*a, c["eps_k8"], 1.0, oracle_mod.PSE_K8_GEODESIC)
    lg.pse_sphere_laplacian_at_particles(*a, c["eps_k8"], 1.0, lg.PSE_K8_GEODESIC, mode="fp32c")
    n = c["x"].size
    x, y, z, f, area = (np.ascontiguousarray(q, dtype=np.float64) for q in a[:5])
    act = np.ascontiguousarray(c["active"], dtype=np.int32)
    out = np.full(n, 7.0)
    P = ctypes.POINTER(ctypes.c_double)
    lg.debug_inject_wait_timeout(skip_tile, 1_000_000)
    rc = lg.lib().lpm_pse_sphere_laplacian(n, *(q.ctypes.data_as(P) for q in (x, y, z, f, area)),
                                           act.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), c["eps_k8"], 1.0,
                                           lg.PSE_K8_GEODESIC, 1, n, out.ctypes.data_as(P), LPM_MODE_FP32C)
    assert rc == LPM_ERR_TIMEOUT, lg.lib().lpm_last_error_string().decode()
    assert np.all(out == 7.0)
    got = lg.pse_sphere_laplacian_at_particles(*a, c["eps_k8"], 1.0, lg.PSE_K8_GEODESIC, mode="fp32c")
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_inject_wait_timeout_rejects_bad_arguments(lg):
    with pytest.raises(lg.LpmError):
        lg.debug_inject_wait_timeout(-1, 1000)
    with pytest.raises(lg.LpmError):
        lg.debug_inject_wait_timeout(0, 0)


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _fail_each_allocation(lg, call, check, max_allocs=64):
    """Runs call() with its k-th device allocation failing, k = 1, 2, ... until it makes no
    k-th allocation (and succeeds).  Every failing call must raise LPM_ERR_ALLOC with the
    injected message; after each, the call must succeed with correct results and the free
    device memory must come back (workspace released).  Returns the number of failures."""
    lg.release_workspace()
    base = _free_bytes()
    failures = 0
    for k in range(1, max_allocs + 1):
        lg.release_workspace()
        lg.debug_fail_device_alloc(k)
        try:
            res = call()
        except lg.LpmError as e:
            assert e.code == LPM_ERR_ALLOC, (k, e)
            assert "injected" in str(e), (k, e)
            failures += 1
            lg.debug_fail_device_alloc(0)
            check(call())
            continue
        lg.debug_fail_device_alloc(0)
        check(res)
        break
    else:
        pytest.fail(f"the call made more than {max_allocs} allocations")
    lg.release_workspace()
    # nothing held: the free memory is back to the baseline (a few MiB of runtime slack)
    assert _free_bytes() >= base - (8 << 20)
    return failures


def test_alloc_failures_host_buffer_sums(lg, wl, oracle_mod):
    pytest.importorskip("torch")
    c = wl.config_gauss_vortex_icos(4)
    a = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    ref = oracle_mod.bve_velocity(*a, 1.0)
    for mode in ("fp32c", "fp64"):
        def call():
            return lg.bve_sphere_velocity(*a, 1.0, mode=mode)

        def check(res):
            assert _rel_linf(res, ref) <= FP32C_TOL

        assert _fail_each_allocation(lg, call, check) >= 3
    p = wl.config_colliding_dipoles(4)
    pa = (p["x"], p["y"], p["omega"], p["area"], p["active"])
    pref = oracle_mod.plane_velocity(*pa, 0.02)
    assert _fail_each_allocation(lg, lambda: lg.planar_incompressible_velocity(*pa, 0.02, mode="fp32c"),
                                 lambda r: _rel_linf(r, pref) <= FP32C_TOL) >= 3
    q = wl.config_pse_cubed(4)
    qa = (q["x"], q["y"], q["z"], q["f"], q["area"], q["active"])
    qref = oracle_mod.pse_laplacian(*qa, q["eps_k8"], 1.0, oracle_mod.PSE_K8_GEODESIC)

    def pcheck(r):
        assert np.abs(r - qref).max() <= 1e-4 * np.abs(qref).max()

    assert _fail_each_allocation(lg, lambda: lg.pse_sphere_laplacian_at_particles(
        *qa, q["eps_k8"], 1.0, lg.PSE_K8_GEODESIC, mode="fp32c"), pcheck) >= 3


def test_alloc_failures_handles(lg, wl):
    """Solver and ensemble creation: a failed create releases everything it had allocated."""
    pytest.importorskip("torch")
    c = wl.config_gauss_vortex_icos(5)
    a = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"])
    ref_state = {}

    def make_bve():
        s = lg.BVESolver(*a, mode="fp32c")
        s.timestep(0.01, 1)
        st = s.get_state()
        s.close()
        return st

    def check_bve(st):
        if not ref_state:
            ref_state.update(make_bve())
        for k in st:
            assert np.array_equal(st[k], ref_state[k]), k

    make_bve()  # loads the modules once, so the memory baseline is steady
    assert _fail_each_allocation(lg, make_bve, check_bve) >= 5
    p = wl.config_colliding_dipoles(5)
    pa = (p["x"], p["y"], p["omega"], p["area"], p["active"])

    def make_plane():
        s = lg.PlaneSolver(*pa, delta=0.02, mode="fp32c")
        s.timestep(0.005, 1)
        st = s.get_state()
        s.close()
        return st

    plane_ref = make_plane()
    assert _fail_each_allocation(lg, make_plane,
                                 lambda st: all(np.array_equal(st[k], plane_ref[k]) for k in st)) >= 5
    inst = wl.config_ensemble(n_instances=4, seed=3, nests=(2, 3))

    def make_ens():
        e = lg.Ensemble(inst, mode="fp32c")
        e.timestep(0.01, 1)
        st = e.get_state()
        e.close()
        return st

    ens_ref = make_ens()
    assert _fail_each_allocation(lg, make_ens, lambda st: all(np.array_equal(st[k], ens_ref[k]) for k in st)) >= 5
