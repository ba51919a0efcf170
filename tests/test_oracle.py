"""CPU tests: the oracle against the reference's own pins, the mesh generator against the
reference's mesh invariants, and the oracle against the committed golden fixtures."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def wl(built_lib):
    import workloads
    return workloads


# ------------------------------------------------------------------ mesh invariants
@pytest.mark.parametrize("seed,nest,n,nact", [
    (205, 0, 32, 20), (205, 3, 1922, 1280), (205, 4, 7682, 5120),
    (206, 0, 14, 6), (206, 4, 3074, 1536),
    (202, 0, 13, 4), (202, 3, 545, 256),
])
def test_mesh_counts(lg, seed, nest, n, nact):
    """Particle counts of nVerticesInMesh + nFacesInMesh (src/PolyMesh2d.f90:717-766)."""
    m = lg.PolyMesh2d(seed, nest, 4.0 if seed == 202 else 1.0)
    assert m.n == n
    assert m.n_active == nact
    # a particle is never both active and passive, passive particles carry no area
    # (tests/IcosTriMeshTester.f90:72-78, src/Faces.f90:684-685)
    assert np.all(m.area[m.active == 0] == 0.0)
    assert np.all(m.area[m.active == 1] > 0.0)


@pytest.mark.parametrize("nest", [0, 1, 2, 3])
def test_icos_leaf_edges(lg, nest):
    """Leaf-edge count: 30 at nest 0 (tests/IcosTriMeshTester.f90:84-89), x4 per level."""
    m = lg.PolyMesh2d(205, nest, 1.0)
    assert m.n_leaf_edges == 30 * 4 ** nest


@pytest.mark.parametrize("seed,nest,total", [(205, 4, 4 * np.pi), (206, 4, 4 * np.pi), (202, 4, 64.0)])
def test_mesh_total_area(lg, seed, nest, total):
    m = lg.PolyMesh2d(seed, nest, 4.0 if seed == 202 else 1.0)
    assert abs(m.area.sum() - total) < 1e-11 * total


# ------------------------------------------------------------------ reference regression pins
def test_pse_reference_regression_thresholds(lg, wl, oracle_mod):
    """tests/SpherePSEConvTest.f90:373-390 run as in tests/CMakeLists.txt (mpirun -np 4,
    spherePSEDefault.namelist: icos nest 3, psePower 0.6).  Its MPI_Reduce passes array
    constructors as send and receive buffers, so rank 0's norms cover rank 0's block only
    (the first N/4 particles); the Linf norm is global."""
    m = lg.PolyMesh2d(205, 3, 1.0)
    eps = m.max_edge_length ** 0.6
    f = wl.y54(m.x, m.y, m.z)
    exact = -30.0 * f
    lap = oracle_mod.pse_laplacian(m.x, m.y, m.z, f, m.area, m.active, eps)
    err = np.abs(lap - exact)
    linf = err.max() / np.abs(exact).max()
    assert linf <= 0.0175
    blk = slice(0, m.n // 4)
    act = m.active[blk].astype(bool)
    l2 = np.sum(err[blk][act] ** 2 * m.area[blk][act]) / np.sum(exact[blk][act] ** 2 * m.area[blk][act])
    assert l2 <= 1.18e-4
    # the Laplacian of a constant vanishes (<= ZERO_TOL)
    lc = oracle_mod.pse_laplacian(m.x, m.y, m.z, np.full(m.n, 2.0), m.area, m.active, eps)
    assert np.abs(lc).max() <= 1e-10


def test_bve_solid_body_known_answer(lg, oracle_mod):
    """examples/BVESolidBody.f90:231-243: zeta = 2 w z / a gives u = w (-y, x, 0); the direct
    sum converges to it at first order in the mesh size."""
    errs = []
    for nest in (3, 4, 5):
        m = lg.PolyMesh2d(205, nest, 1.0)
        zeta = 2.0 * m.z
        u, v, w = oracle_mod.bve_velocity(m.x, m.y, m.z, zeta, m.area, m.active)
        errs.append(np.sqrt((u + m.y) ** 2 + (v - m.x) ** 2 + w ** 2).max())
    assert errs[-1] < 3e-3
    assert errs[0] / errs[1] > 1.8 and errs[1] / errs[2] > 1.8


def test_bve_rh54_known_answer(lg, wl, oracle_mod):
    """The RH wave-4 vorticity of the reference's example: the direct sum converges at first
    order to the exact velocity of its stream function (errors 2.9e-2, 1.5e-2, 8.1e-3 of
    max|u| at icosahedral nests 3-5)."""
    errs = []
    for nest in (3, 4, 5):
        m = wl.sphere_mesh(lg.ICOS_TRI_SPHERE_SEED, nest)
        u = np.stack(oracle_mod.bve_velocity(m.x, m.y, m.z, wl.rh54_vorticity(m), m.area, m.active))
        ue = np.stack(wl.rh54_velocity(m.x, m.y, m.z))
        errs.append(np.abs(u - ue).max() / np.abs(ue).max())
    assert errs[-1] < 1e-2
    assert errs[0] / errs[1] > 1.8 and errs[1] / errs[2] > 1.8


def test_plane_gaussian_vortex_known_answer(lg, oracle_mod):
    """Planar sum (delta = 0) of the Gaussian vortex omega = exp(-r^2/s^2), s = 0.5, on the quad
    mesh of [-4,4]^2: the exact velocity is azimuthal, v_theta = s^2 (1 - exp(-r^2/s^2)) / (2 r);
    the midpoint-rule sum converges at second order (5.0e-2, 1.3e-2, 3.3e-3 of max|u| at quad
    nests 4-6)."""
    s2 = 0.25
    errs = []
    for nest in (4, 5, 6):
        m = lg.PolyMesh2d(lg.QUAD_RECT_SEED, nest, 4.0)
        x, y = m.x, m.y
        r2 = x * x + y * y
        u, v = oracle_mod.plane_velocity(x, y, np.exp(-r2 / s2), m.area, m.active, 0.0)
        vt = np.where(r2 > 0, s2 * (1.0 - np.exp(-r2 / s2)) / (2.0 * np.where(r2 > 0, r2, 1.0)), 0.0)
        ue, ve = -vt * y, vt * x
        errs.append(max(np.abs(u - ue).max(), np.abs(v - ve).max()) / np.abs(np.stack([ue, ve])).max())
    assert errs[-1] < 5e-3
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5


def test_pse_gradient_divergence_known_answer(lg, wl, oracle_mod):
    """PSE gradient of y54 (tests/SpherePSETest.f90 computes it against HarmGradient) and
    divergence of that gradient (the surface Laplacian, -30 y54) on the cubed sphere with
    eps = h^0.5; the (f_j + f_i) form of the gradient needs eps well above h."""
    eg, ed = [], []
    for nest in (4, 5, 6):
        m = wl.sphere_mesh(lg.CUBED_SPHERE_SEED, nest)
        eps = m.max_edge_length ** 0.5
        f = wl.y54(m.x, m.y, m.z)
        ge = np.stack(wl.y54_surface_gradient(m.x, m.y, m.z))
        blk = slice(0, min(m.n, 4096))
        g = np.stack(oracle_mod.pse_sphere_gradient(m.x, m.y, m.z, f, m.area, m.active, eps, ib=0, ie=blk.stop))
        eg.append(np.sqrt(((g - ge[:, blk]) ** 2).sum(0)).max() / np.sqrt((ge ** 2).sum(0)).max())
        d = oracle_mod.pse_sphere_divergence(m.x, m.y, m.z, ge[0], ge[1], ge[2], m.area, m.active, eps, ib=0,
                                             ie=blk.stop)
        ed.append(np.abs(d + 30.0 * f[blk]).max() / np.abs(30.0 * f).max())
    assert eg[-1] < 1.5e-2 and eg[0] > eg[1] > eg[2]
    assert ed[-1] < 5e-3 and ed[0] > ed[2]


def test_oracle_associations_agree(lg, wl, oracle_mod):
    """The two reference associations of the BVE denominator differ only by rounding."""
    c = wl.config_gauss_vortex_icos(3)
    u0, v0, w0 = oracle_mod.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, 0)
    u1, v1, w1 = oracle_mod.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], 1.0, 1)
    s = np.abs(np.stack([u0, v0, w0])).max()
    assert np.abs(np.stack([u0 - u1, v0 - v1, w0 - w1])).max() <= 1e-12 * s


def test_oracle_target_range_and_threads(lg, wl, oracle_mod):
    """A rank block [ib, ie) reproduces the same entries of the full sum, any thread count."""
    c = wl.config_gauss_vortex_icos(2)
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    full = oracle_mod.bve_velocity(*args, threads=1)
    part = oracle_mod.bve_velocity(*args, ib=37, ie=301, threads=3)
    for a, b in zip(full, part):
        assert np.array_equal(a[37:301], b)


def test_rk4_conserves_circulation(lg, wl, oracle_mod):
    """Circulation sum(zeta A) is conserved and KE drifts little over 5 steps (the reference
    driver's diagnostics, examples/BVESingleGaussianVortex.f90:253-254)."""
    c = wl.config_gauss_vortex_icos(2)
    u, v, w = oracle_mod.bve_velocity(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    ke0, en0, ci0 = oracle_mod.bve_diagnostics(u, v, w, c["zeta"], c["area"], c["active"])
    s = oracle_mod.bve_timestep(c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"], u, v, w, 1.0, 0.0,
                                0.01, 5)
    ke1, en1, ci1 = oracle_mod.bve_diagnostics(s[4], s[5], s[6], s[3], c["area"], c["active"])
    assert abs(ci1 - ci0) < 1e-12
    assert abs(ke1 - ke0) / ke0 < 1e-2


# ------------------------------------------------------------------ golden fixtures
def _load(name):
    return np.load(GOLDEN / name)


def test_golden_bve(oracle_mod):
    g = _load("bve_icos2.npz")
    u, v, w = oracle_mod.bve_velocity(g["x"], g["y"], g["z"], g["zeta"], g["area"], g["active"], 1.0, 0)
    assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"]) and np.array_equal(w, g["w"])
    um, vm, wm = oracle_mod.bve_velocity(g["x"], g["y"], g["z"], g["zeta"], g["area"], g["active"], 1.0, 1)
    assert np.array_equal(um, g["um"]) and np.array_equal(wm, g["wm"])
    uo, vo, wo = oracle_mod.bve_velocity(g["xo"], g["yo"], g["zo"], g["zeta"], g["area"], g["active"], 1.0, 0)
    assert np.array_equal(uo, g["uo"]) and np.array_equal(vo, g["vo"])


def test_golden_stream(oracle_mod):
    g = _load("bve_icos2.npz")
    pr, pa = oracle_mod.bve_stream(g["x"], g["y"], g["z"], g["zeta"], g["absvort"], g["area"], g["active"])
    # log() may differ by an ulp between C libraries: 1e-13 relative
    assert np.abs(pr - g["psi_rel"]).max() <= 1e-13 * np.abs(g["psi_rel"]).max()
    assert np.abs(pa - g["psi_abs"]).max() <= 1e-13 * np.abs(g["psi_abs"]).max()


def test_golden_rk4(oracle_mod):
    g = _load("bve_rk4_icos2.npz")
    s = oracle_mod.bve_timestep(g["x0"], g["y0"], g["z0"], g["zeta0"], g["area"], g["active"], g["u0"], g["v0"],
                                g["w0"], 1.0, float(g["omega"]), float(g["dt"]), int(g["steps"]))
    for k, a in zip(("x", "y", "z", "zeta", "u", "v", "w"), s):
        assert np.array_equal(a, g[k]), k


def test_golden_plane(oracle_mod):
    g = _load("plane_quad3.npz")
    u, v = oracle_mod.plane_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.0)
    assert np.array_equal(u, g["u0"]) and np.array_equal(v, g["v0"])
    u, v = oracle_mod.plane_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.02)
    assert np.array_equal(u, g["u2"]) and np.array_equal(v, g["v2"])
    t = oracle_mod.plane_timestep(g["x"], g["y"], g["omega"], g["area"], g["active"], g["u0"], g["v0"], 0.0,
                                  float(g["dt"]), int(g["steps"]))
    assert np.array_equal(t[0], g["xs"]) and np.array_equal(t[3], g["vs"])


def test_golden_pse(oracle_mod):
    g = _load("pse_small.npz")
    lk = oracle_mod.pse_laplacian(g["x"], g["y"], g["z"], g["f"], g["area"], g["active"], float(g["eps_k8"]), 1.0, 0)
    lgs = oracle_mod.pse_laplacian(g["x"], g["y"], g["z"], g["f"], g["area"], g["active"], float(g["eps_g"]), 1.0, 1)
    lp = oracle_mod.pse_laplacian(g["px"], g["py"], None, g["pf"], g["parea"], g["pactive"], float(g["peps"]), 1.0,
                                  2)
    for a, b in ((lk, g["lap_k8"]), (lgs, g["lap_gauss"]), (lp, g["plap"])):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_golden_operators(oracle_mod):
    """The other PSE operators, the SWE integrals and the beta plane against ops_small.npz
    (1e-13 of each result's max: exp, atan2, log and cosh may differ by an ulp between C
    libraries)."""
    g = _load("ops_small.npz")
    o = oracle_mod
    sx, sy, sz, sa, sact, seps = g["sx"], g["sy"], g["sz"], g["sa"], g["sact"], float(g["seps"])
    px, py, pa, pact, peps = g["px"], g["py"], g["pa"], g["pact"], float(g["peps"])
    pg = o.pse_plane_gradient(px, py, g["pf"], pa, pact, peps)
    got = {
        "grad": np.stack(o.pse_sphere_gradient(sx, sy, sz, g["sf"], sa, sact, seps, 1.0)),
        "div": o.pse_sphere_divergence(sx, sy, sz, g["sgx"], g["sgy"], g["sgz"], sa, sact, seps, 1.0),
        "sddot": o.pse_sphere_double_dot(sx, sy, sz, g["sgx"], g["sgy"], g["sgz"], sa, sact, seps, 1.0),
        "sinterp": o.pse_interpolate(sx, sy, sz, g["sf"], sa, sact, seps, g["sq"][0], g["sq"][1], g["sq"][2], 1, 1.0),
        "sswe": np.stack(o.swe_sphere_rhs(sx, sy, sz, g["szeta"], g["sdivv"], g["ssh"], sa, sact, 1.0, 1.0, 0.25)),
        "pgrad": np.stack(pg),
        "psecond": np.stack(o.pse_plane_second_partials(px, py, pg[0], pg[1], pa, pact, peps)),
        "pddot": o.pse_plane_double_dot(px, py, pg[0], pg[1], pa, pact, peps),
        "pinterp": o.pse_interpolate(px, py, None, g["pf"], pa, pact, peps, g["pq"][0], g["pq"][1], None, 0, 1.0),
        "pswe": np.stack(o.swe_plane_rhs(px, py, g["pvort"], g["pdivv"], g["psh"], pa, pact, peps)),
        "bvel": np.stack(o.beta_plane_velocity(g["bx"], g["by"], g["bzeta"], g["ba"], g["bact"])),
        "bstream": np.stack(o.beta_plane_stream(g["bx"], g["by"], g["bzeta"], g["bzeta"] + 3.0 * g["by"], g["ba"],
                                                g["bact"])),
    }
    for k, v in got.items():
        ref = g[k]
        assert v.shape == ref.shape, k
        assert np.abs(v - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1e-300), k
