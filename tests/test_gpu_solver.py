"""GPU tests of the device-resident RK4 solvers through the C ABI."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def wl(built_lib):
    import workloads
    return workloads


def test_bve_rk4_fp64_bit_exact_golden(lg):
    """10 RK4 steps of timestepPrivate (SphereBVESolver.f90:219-353), FP64: bit-identical."""
    g = np.load(GOLDEN / "bve_rk4_icos2.npz")
    s = lg.BVESolver(g["x0"], g["y0"], g["z0"], g["zeta0"], g["area"], g["active"], 1.0, float(g["omega"]),
                     g["u0"], g["v0"], g["w0"], mode="fp64")
    s.timestep(float(g["dt"]), int(g["steps"]))
    st = s.get_state()
    for k, gk in (("x", "x"), ("y", "y"), ("z", "z"), ("rel_vort", "zeta"), ("u", "u"), ("v", "v"), ("w", "w")):
        assert np.array_equal(st[k], g[gk]), k
    s.close()


def test_bve_rk4_100_steps_bit_exact(lg, wl, oracle_mod):
    """The single-Gaussian-vortex run (icos nest 3, dt 0.01, 100 steps, Omega = 2 pi, remesh
    off): FP64 positions and vorticity bit-identical to the oracle after 100 steps."""
    c = wl.config_gauss_vortex_icos(3)
    u, v, w = oracle_mod.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, 1)
    ref = oracle_mod.bve_timestep(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], u, v, w, 1.0,
                                  c["omega"], 0.01, 100)
    s = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"], mode="fp64")
    s.timestep(0.01, 100)
    st = s.get_state()
    for k, a in zip(("x", "y", "z", "rel_vort", "u", "v", "w"), ref):
        assert np.array_equal(st[k], a), k
    s.close()


def test_bve_rk4_fp32c_tracks_fp64(lg, wl):
    c = wl.config_gauss_vortex_icos(4)
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"])
    s64 = lg.BVESolver(*args, mode="fp64")
    s32 = lg.BVESolver(*args, mode="fp32c")
    d0 = s64.diagnostics()
    s64.timestep(0.01, 20)
    s32.timestep(0.01, 20)
    a, b = s64.get_state(), s32.get_state()
    # velocity errors <= 1e-6 relative over 20 steps of dt = 0.01 bound the positions by
    # ~20 dt 1e-6 |u|; in practice they agree to ~1e-8
    pos = np.stack([a["x"] - b["x"], a["y"] - b["y"], a["z"] - b["z"]])
    assert np.abs(pos).max() < 1e-7
    vel = np.stack([a["u"] - b["u"], a["v"] - b["v"], a["w"] - b["w"]])
    assert np.abs(vel).max() / np.abs(np.stack([a["u"], a["v"], a["w"]])).max() < 2e-6
    d1, d2 = s64.diagnostics(), s32.diagnostics()
    # relative vorticity evolves by -2 Omega w / a, so its circulation is not an invariant
    # here; FP32C and FP64 must agree on it and on the kinetic energy
    assert abs(d2["circulation"] - d1["circulation"]) < 1e-9 * max(1.0, abs(d0["enstrophy"]))
    assert abs(d2["kinetic_energy"] - d1["kinetic_energy"]) < 1e-6 * d1["kinetic_energy"]
    ms, launches = s32.kernel_timing()
    assert ms > 0 and launches == 20 * (4 + 4 * 3 + 7)
    s64.close()
    s32.close()


def test_bve_circulation_conserved_without_rotation(lg, wl):
    """With Omega = 0 the relative vorticity is materially conserved: sum(zeta A) is fixed."""
    c = wl.config_gauss_vortex_icos(3)
    s = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, 0.0, mode="fp32c")
    d0 = s.diagnostics()
    s.timestep(0.01, 10)
    d1 = s.diagnostics()
    assert abs(d1["circulation"] - d0["circulation"]) < 1e-13
    assert abs(d1["kinetic_energy"] - d0["kinetic_energy"]) < 1e-3 * d0["kinetic_energy"]
    s.close()


def test_bve_diagnostics_match_oracle(lg, wl, oracle_mod):
    c = wl.config_gauss_vortex_icos(3)
    s = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"], mode="fp64")
    st = s.get_state()
    d = s.diagnostics()
    ke, en, ci = oracle_mod.bve_diagnostics(st["u"], st["v"], st["w"], st["rel_vort"], c["area"], c["active"])
    assert abs(d["kinetic_energy"] - ke) <= 1e-13 * ke
    assert abs(d["enstrophy"] - en) <= 1e-13 * en
    assert abs(d["circulation"] - ci) <= 1e-12
    s.close()


def test_bve_renormalize_keeps_radius(lg, wl):
    c = wl.config_gauss_vortex_icos(3)
    s = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"], mode="fp32c")
    s.timestep(0.01, 10, renormalize=True)
    st = s.get_state()
    r = np.sqrt(st["x"] ** 2 + st["y"] ** 2 + st["z"] ** 2)
    assert np.abs(r - 1.0).max() < 1e-14
    s.close()


def test_plane_rk4_fp64_bit_exact_golden(lg):
    g = np.load(GOLDEN / "plane_quad3.npz")
    s = lg.PlaneSolver(g["x"], g["y"], g["omega"], g["area"], g["active"], g["u0"], g["v0"], 0.0, mode="fp64")
    s.timestep(float(g["dt"]), int(g["steps"]))
    st = s.get_state()
    assert np.array_equal(st["x"], g["xs"]) and np.array_equal(st["y"], g["ys"])
    assert np.array_equal(st["u"], g["us"]) and np.array_equal(st["v"], g["vs"])
    s.close()


def test_plane_fp32c_tracks_fp64(lg, wl):
    c = wl.config_colliding_dipoles(4)
    args = (c["x"], c["y"], c["omega"], c["area"], c["active"])
    s64 = lg.PlaneSolver(*args, delta=0.02, mode="fp64")
    s32 = lg.PlaneSolver(*args, delta=0.02, mode="fp32c")
    s64.timestep(0.005, 20)
    s32.timestep(0.005, 20)
    a, b = s64.get_state(), s32.get_state()
    assert np.abs(np.stack([a["x"] - b["x"], a["y"] - b["y"]])).max() < 1e-7
    d = s64.diagnostics()
    assert d["kinetic_energy"] > 0
    s64.close()
    s32.close()


def test_solver_bad_arguments(lg):
    with pytest.raises(lg.LpmError):
        lg.BVESolver(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0, np.int32))
    with pytest.raises(lg.LpmError):
        lg.BVESolver(np.ones(3), np.ones(3), np.ones(3), np.ones(3), np.ones(3), np.ones(3, np.int32), radius=-1.0)


def test_measure_fp32_peak(lg):
    t = lg.measure_fp32_peak(50.0)
    assert 30.0 < t < 100.0  # 152 SMs x 128 FP32 lanes x 2 flops x clock


@pytest.mark.parametrize("mode", ["fp64", "fp32c"])
def test_solver_stream_functions(lg, wl, mode):
    """The solver's stream functions at its current state equal the host-buffer call on the
    same state (bit for bit in FP64, which sweeps the sources in the same order)."""
    c = wl.config_gauss_vortex_icos(3)
    s = lg.BVESolver(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, c["omega"], mode=mode)
    s.timestep(0.01, 3)
    st = s.get_state()
    absv = st["rel_vort"] + 2.0 * c["omega"] * st["z"]
    pr, pa = s.stream_functions(absv)
    rr, ra = lg.set_stream_functions_on_mesh(st["x"], st["y"], st["z"], st["rel_vort"], absv, c["area"],
                                             c["active"], 1.0, mode=mode)
    if mode == "fp64":
        assert np.array_equal(pr, rr) and np.array_equal(pa, ra)
    else:
        assert np.abs(pr - rr).max() <= 1e-6 * np.abs(rr).max()
        assert np.abs(pa - ra).max() <= 1e-6 * np.abs(ra).max()
    qr, qa = s.stream_functions()  # absolute vorticity from the state
    assert np.abs(qa - pa).max() <= 1e-9 * np.abs(pa).max() and np.array_equal(qr, pr)
    s.close()


@pytest.mark.parametrize("mode", ["fp64", "fp32c"])
def test_bve_remesh_in_place_matches_new_solver(lg, wl, mode):
    """lpm_bve_solver_remesh in place of Delete(solver) + New(solver, sphere): after a remesh to
    a larger set (the buffers grow), to a smaller one (they are reused), and with a velocity
    given, the states, diagnostics and stream functions are those of a newly created solver."""
    a, b, c = (wl.config_gauss_vortex_icos(k) for k in (3, 4, 2))
    s = lg.BVESolver(a["x"], a["y"], a["z"], a["zeta"], a["area"], a["active"], 1.0, a["omega"], mode=mode)
    s.timestep(0.01, 2)
    for cfg, uvw in ((b, None), (c, None), (b, "given")):
        kw = {}
        if uvw:
            kw = dict(zip("uvw", (-0.1 * cfg["y"], 0.1 * cfg["x"], 0.0 * cfg["z"])))  # tangent: solid body
        s.remesh(cfg["x"], cfg["y"], cfg["z"], cfg["zeta"], cfg["area"], cfg["active"], **kw)
        fresh = lg.BVESolver(cfg["x"], cfg["y"], cfg["z"], cfg["zeta"], cfg["area"], cfg["active"], 1.0,
                             a["omega"], mode=mode, **kw)
        s.timestep(0.01, 3)
        fresh.timestep(0.01, 3)
        st, sf = s.get_state(), fresh.get_state()
        for k in st:
            assert np.array_equal(st[k], sf[k]), k
        assert s.diagnostics() == fresh.diagnostics()
        p1, p2 = s.stream_functions(), fresh.stream_functions()
        assert np.array_equal(p1[0], p2[0]) and np.array_equal(p1[1], p2[1])
        fresh.close()
    s.close()


@pytest.mark.parametrize("mode", ["fp64", "fp32c"])
def test_plane_remesh_in_place_matches_new_solver(lg, wl, mode):
    """lpm_plane_solver_remesh through growth and reuse: the state after a remesh and a few
    steps is that of a newly created solver on the same particle set."""
    a, b, c = (wl.config_colliding_dipoles(k) for k in (4, 5, 3))
    s = lg.PlaneSolver(a["x"], a["y"], a["omega"], a["area"], a["active"], mode=mode)
    s.timestep(0.005, 2)
    for cfg in (b, c, b):
        s.remesh(cfg["x"], cfg["y"], cfg["omega"], cfg["area"], cfg["active"])
        fresh = lg.PlaneSolver(cfg["x"], cfg["y"], cfg["omega"], cfg["area"], cfg["active"], mode=mode)
        s.timestep(0.005, 3)
        fresh.timestep(0.005, 3)
        st, sf = s.get_state(), fresh.get_state()
        for k in st:
            assert np.array_equal(st[k], sf[k]), k
        assert s.diagnostics() == fresh.diagnostics()
        fresh.close()
    s.close()
