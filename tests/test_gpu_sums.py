"""GPU parity tests of the direct sums through the C ABI (liblpm_gpu.so).

FP64 mode restates the reference loops with the reference association and source order, so
the BVE and planar sums must be bit-identical to the oracle.  The PSE and stream-function
sums call exp/atan2/log, whose CUDA and C-library implementations may differ by an ulp:
those are checked to 1e-12 relative to max|result|.  FP32C mode is checked to the velocity
relative L-infinity error bound 1e-6 (relative to max|u| over the targets).
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"

FP32C_TOL = 1e-6


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def wl(built_lib):
    import workloads
    return workloads


def rel_linf(got, ref):
    got = np.stack(got) if isinstance(got, (tuple, list)) else got
    ref = np.stack(ref) if isinstance(ref, (tuple, list)) else ref
    return np.abs(got - ref).max() / np.abs(ref).max()


# ------------------------------------------------------------------ golden fixtures
def test_golden_bve_fp64_bit_exact(lg):
    g = np.load(GOLDEN / "bve_icos2.npz")
    u, v, w = lg.bve_sphere_velocity(g["x"], g["y"], g["z"], g["zeta"], g["area"], g["active"], 1.0)
    assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"]) and np.array_equal(w, g["w"])
    u, v, w = lg.set_velocity_from_vorticity(g["x"], g["y"], g["z"], g["zeta"], g["area"], g["active"], 1.0)
    assert np.array_equal(u, g["um"]) and np.array_equal(v, g["vm"]) and np.array_equal(w, g["wm"])
    u, v, w = lg.bve_sphere_velocity(g["xo"], g["yo"], g["zo"], g["zeta"], g["area"], g["active"], 1.0)
    assert np.array_equal(u, g["uo"]) and np.array_equal(v, g["vo"]) and np.array_equal(w, g["wo"])


def test_golden_bve_fp32c(lg):
    g = np.load(GOLDEN / "bve_icos2.npz")
    got = lg.bve_sphere_velocity(g["x"], g["y"], g["z"], g["zeta"], g["area"], g["active"], 1.0, mode="fp32c")
    assert rel_linf(got, (g["u"], g["v"], g["w"])) <= FP32C_TOL
    got = lg.bve_sphere_velocity(g["xo"], g["yo"], g["zo"], g["zeta"], g["area"], g["active"], 1.0, mode="fp32c")
    assert rel_linf(got, (g["uo"], g["vo"], g["wo"])) <= FP32C_TOL


def test_golden_plane(lg):
    g = np.load(GOLDEN / "plane_quad3.npz")
    u, v = lg.planar_incompressible_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.0)
    assert np.array_equal(u, g["u0"]) and np.array_equal(v, g["v0"])
    u, v = lg.planar_incompressible_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.02)
    assert np.array_equal(u, g["u2"]) and np.array_equal(v, g["v2"])
    got = lg.planar_incompressible_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.02, mode="fp32c")
    assert rel_linf(got, (g["u2"], g["v2"])) <= FP32C_TOL
    got = lg.planar_incompressible_velocity(g["x"], g["y"], g["omega"], g["area"], g["active"], 0.0, mode="fp32c")
    assert rel_linf(got, (g["u0"], g["v0"])) <= FP32C_TOL


def test_golden_pse(lg):
    g = np.load(GOLDEN / "pse_small.npz")
    lk = lg.pse_sphere_laplacian_at_particles(g["x"], g["y"], g["z"], g["f"], g["area"], g["active"],
                                              float(g["eps_k8"]), 1.0, lg.PSE_K8_GEODESIC)
    assert rel_linf(lk, g["lap_k8"]) <= 1e-12
    lgs = lg.pse_sphere_laplacian_at_particles(g["x"], g["y"], g["z"], g["f"], g["area"], g["active"],
                                               float(g["eps_g"]), 1.0, lg.PSE_GAUSS_CHORD)
    assert rel_linf(lgs, g["lap_gauss"]) <= 1e-12
    lp = lg.pse_plane_laplacian_at_particles(g["px"], g["py"], g["pf"], g["parea"], g["pactive"], float(g["peps"]),
                                             lg.PSE_K8_CHORD)
    assert rel_linf(lp, g["plap"]) <= 1e-12


def test_golden_stream(lg):
    g = np.load(GOLDEN / "bve_icos2.npz")
    pr, pa = lg.set_stream_functions_on_mesh(g["x"], g["y"], g["z"], g["zeta"], g["absvort"], g["area"],
                                             g["active"], 1.0)
    assert rel_linf(pr, g["psi_rel"]) <= 1e-12 and rel_linf(pa, g["psi_abs"]) <= 1e-12
    gp = np.load(GOLDEN / "plane_quad3.npz")
    ps = lg.set_stream_function_on_mesh(gp["x"], gp["y"], gp["omega"], gp["area"], gp["active"])
    assert rel_linf(ps, gp["psi"]) <= 1e-12


# ------------------------------------------------------------------ oracle parity at larger sizes
@pytest.mark.parametrize("nest", [3, 4])
def test_bve_fp64_bit_exact_vs_oracle(lg, wl, oracle_mod, nest):
    c = wl.config_gauss_vortex_icos(nest)
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    ref = oracle_mod.bve_velocity(*args)
    got = lg.bve_sphere_velocity(*args, 1.0)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_bve_fp32c_vs_oracle_rh54(lg, wl, oracle_mod):
    c = wl.config_rh54_icos(5, seed=3)
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    ref = oracle_mod.bve_velocity(*args)
    got = lg.bve_sphere_velocity(*args, 1.0, mode="fp32c")
    assert rel_linf(got, ref) <= FP32C_TOL


def test_bve_rh54_known_answer_gpu(lg, wl):
    """The RH wave-4 field at icosahedral nest 6 (122,882 particles): both modes reproduce the
    exact velocity to the discretisation error of the sum (4.1e-3, first order in h), and FP32C
    stays within 1e-6 of FP64."""
    m = wl.sphere_mesh(lg.ICOS_TRI_SPHERE_SEED, 6)
    zeta = wl.rh54_vorticity(m)
    ue = np.stack(wl.rh54_velocity(m.x, m.y, m.z))
    u64 = lg.bve_sphere_velocity(m.x, m.y, m.z, zeta, m.area, m.active, 1.0)
    u32 = lg.bve_sphere_velocity(m.x, m.y, m.z, zeta, m.area, m.active, 1.0, mode="fp32c")
    assert rel_linf(u64, ue) < 5e-3
    assert rel_linf(u32, u64) <= FP32C_TOL


def test_bve_rank_block_range(lg, wl, oracle_mod):
    """i_begin/i_end (1-based, inclusive) write only the rank's block, as MPISetup splits it."""
    c = wl.config_gauss_vortex_icos(3)
    args = (c["x"], c["y"], c["z"], c["zeta"], c["area"], c["active"])
    n = c["x"].size
    ref = oracle_mod.bve_velocity(*args)
    chunk = n // 3
    for r in range(3):
        ib, ie = r * chunk + 1, (n if r == 2 else (r + 1) * chunk)
        sentinel = [np.full(n, 7.0) for _ in range(3)]
        got = lg.bve_sphere_velocity(*args, 1.0, i_begin=ib, i_end=ie, out=sentinel)
        for a, b in zip(got, ref):
            assert np.array_equal(a[ib - 1:ie], b[ib - 1:ie])
            assert np.all(a[:ib - 1] == 7.0) and np.all(a[ie:] == 7.0)
        got32 = lg.bve_sphere_velocity(*args, 1.0, i_begin=ib, i_end=ie, mode="fp32c")
        assert rel_linf([g[ib - 1:ie] for g in got32], [b[ib - 1:ie] for b in ref]) <= FP32C_TOL


@pytest.mark.parametrize("n", [1, 2, 33, 257, 1000])
def test_bve_ragged_sizes(lg, oracle_mod, n):
    """Odd sizes, not multiples of the tile or the CTA width; random activity pattern."""
    rng = np.random.default_rng(n)
    p = rng.normal(size=(3, n))
    p /= np.linalg.norm(p, axis=0)
    zeta = rng.normal(size=n)
    area = rng.uniform(0.5, 1.5, size=n) * 4 * np.pi / n
    act = (rng.random(n) < 0.7).astype(np.int32)
    ref = oracle_mod.bve_velocity(p[0], p[1], p[2], zeta, area, act)
    got = lg.bve_sphere_velocity(p[0], p[1], p[2], zeta, area, act, 1.0)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    if np.abs(np.stack(ref)).max() > 0:
        got32 = lg.bve_sphere_velocity(p[0], p[1], p[2], zeta, area, act, 1.0, mode="fp32c")
        assert rel_linf(got32, ref) <= FP32C_TOL


def test_bve_no_active_sources(lg):
    n = 10
    p = np.eye(3)[:, [0, 1, 2, 0, 1, 2, 0, 1, 2, 0]] * 1.0
    p[:, 3:] += 0.1
    z = np.zeros(n)
    for mode in ("fp64", "fp32c"):
        u, v, w = lg.bve_sphere_velocity(p[0], p[1], p[2], np.ones(n), np.ones(n), np.zeros(n, np.int32), 1.0,
                                         mode=mode)
        assert np.array_equal(u, z) and np.array_equal(v, z) and np.array_equal(w, z)


def test_bve_radius_scaling(lg, wl, oracle_mod):
    """A sphere of radius a != 1 (the Earth-radius case of the drivers)."""
    c = wl.config_gauss_vortex_icos(3)
    a = 6.37122e6
    args = (c["x"] * a, c["y"] * a, c["z"] * a, c["zeta"] * 1e-5, c["area"] * a * a, c["active"])
    ref = oracle_mod.bve_velocity(*args, radius=a)
    got = lg.bve_sphere_velocity(*args, a)
    for g_, r_ in zip(got, ref):
        assert np.array_equal(g_, r_)
    assert rel_linf(lg.bve_sphere_velocity(*args, a, mode="fp32c"), ref) <= FP32C_TOL


@pytest.mark.parametrize("delta", [0.0, 0.02])
def test_plane_vs_oracle(lg, wl, oracle_mod, delta):
    c = wl.config_colliding_dipoles(5)
    args = (c["x"], c["y"], c["omega"], c["area"], c["active"])
    ref = oracle_mod.plane_velocity(*args, delta)
    got = lg.planar_incompressible_velocity(*args, delta)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert rel_linf(lg.planar_incompressible_velocity(*args, delta, mode="fp32c"), ref) <= FP32C_TOL


@pytest.mark.parametrize("n", [1, 2, 33, 257, 1000, 5000])
@pytest.mark.parametrize("delta", [0.0, 0.02])
def test_plane_fp32c_ragged_clustered(lg, oracle_mod, n, delta):
    """Planar FP32C on odd sizes: a uniform scatter plus a tight cluster (spacings down to
    ~1e-7), a smooth vorticity field, random activity, a rank block."""
    rng = np.random.default_rng(7 + n)
    m = n // 2
    x = np.concatenate([rng.uniform(-4, 4, n - m), 1.0 + 1e-4 * rng.normal(size=m)])
    y = np.concatenate([rng.uniform(-4, 4, n - m), -0.5 + 1e-4 * rng.normal(size=m)])
    om = np.exp(-((x - 0.5) ** 2 + y ** 2)) - 0.5 * np.exp(-((x + 1.0) ** 2 + (y - 1.0) ** 2) / 2.0)
    area = rng.uniform(0.5, 1.5, n) * 64.0 / n
    act = (rng.random(n) < 0.7).astype(np.int32)
    ib, ie = (n // 4 + 1, n) if n > 4 else (1, n)
    ref = oracle_mod.plane_velocity(x, y, om, area, act, delta)
    got = lg.planar_incompressible_velocity(x, y, om, area, act, delta, i_begin=ib, i_end=ie, mode="fp32c")
    sl = slice(ib - 1, ie)
    scale = max(np.abs(np.stack(ref)[:, sl]).max(), 1e-300)
    assert np.abs(np.stack(got)[:, sl] - np.stack(ref)[:, sl]).max() <= FP32C_TOL * scale


def bve_chord_reference(p, zeta, area, act):
    """FP64 sphere velocity through the exact chord identity a^2 - x_i.x_j = (|d|^2 - c_i - c_j)/2
    with d = x_i - x_j (no cancellation for close pairs, unlike the reference's 1 - x_i.x_j,
    which loses ~2^-53 / (1 - x_i.x_j) relative and is useless below spacings of ~1e-6)."""
    n = p.shape[1]
    c = (p ** 2).sum(0) - 1.0
    src = np.nonzero(act)[0]
    s = -zeta[src] * area[src] / (4.0 * np.pi)
    u = np.zeros((3, n))
    for i0 in range(0, n, 512):
        i1 = min(n, i0 + 512)
        d = p[:, i0:i1, None] - p[:, None, src]
        den = 0.5 * ((d ** 2).sum(0) - c[i0:i1, None] - c[None, src])
        w = np.where(np.arange(i0, i1)[:, None] == src[None, :], 0.0, s[None, :] / np.where(den == 0, 1.0, den))
        cr = np.cross(p[:, i0:i1, None], p[:, None, src], axis=0)
        u[:, i0:i1] = (cr * w[None]).sum(2)
    return u


@pytest.mark.parametrize("n", [300, 1000, 5000])
def test_bve_fp32c_clustered(lg, n):
    """Sphere FP32C with half the points in a tight cluster (spacings down to ~1e-4 of the
    radius, against ~0.05 in the scatter) next to a uniform scatter, smooth vorticity: the
    near groups of a warp take the full-precision path.  The reference is the FP64 chord
    form; the reference loop's 1 - x_i.x_j loses ~2^-53 / (1 - x_i.x_j) relative.  (Closer
    than ~1e-6 the sum is ill-conditioned in the FP64 positions themselves: a^2 - x_i.x_j
    then depends on |x|^2 - a^2 at the 1e-16 level, which the inputs do not carry.)"""
    rng = np.random.default_rng(11 + n)
    m = n // 2
    p = rng.normal(size=(3, n))
    c0 = np.array([0.3, -0.5, 0.8])
    p[:, n - m:] = c0[:, None] + 1e-2 * rng.normal(size=(3, m))
    p /= np.linalg.norm(p, axis=0)
    zeta = np.exp(-4.0 * ((p - c0[:, None] / np.linalg.norm(c0)) ** 2).sum(0)) - 0.3 * p[2]
    area = rng.uniform(0.5, 1.5, size=n) * 4 * np.pi / n
    act = (rng.random(n) < 0.8).astype(np.int32)
    ref = bve_chord_reference(p, zeta, area, act)
    got = lg.bve_sphere_velocity(p[0], p[1], p[2], zeta, area, act, 1.0, mode="fp32c")
    assert rel_linf(got, ref) <= FP32C_TOL


def test_plane_fp32c_translated(lg, wl, oracle_mod):
    """The Lamb-dipole configuration moved to (1000, -2000): FP32C keeps its accuracy (hi/lo
    positions, group origins at the centroids)."""
    c = wl.config_colliding_dipoles(5)
    x, y = c["x"] + 1000.0, c["y"] - 2000.0
    args = (x, y, c["omega"], c["area"], c["active"])
    ref = oracle_mod.plane_velocity(*args, 0.0)
    assert rel_linf(lg.planar_incompressible_velocity(*args, 0.0, mode="fp32c"), ref) <= FP32C_TOL


def test_pse_reference_thresholds_on_gpu(lg, wl):
    """The reference regression test's thresholds hold for the GPU Laplacian (both modes)."""
    m = lg.PolyMesh2d(205, 3, 1.0)
    eps = m.max_edge_length ** 0.6
    f = wl.y54(m.x, m.y, m.z)
    exact = -30.0 * f
    for mode in ("fp64", "fp32c"):
        lap = lg.pse_sphere_laplacian_at_particles(m.x, m.y, m.z, f, m.area, m.active, eps, mode=mode)
        err = np.abs(lap - exact)
        assert err.max() / np.abs(exact).max() <= 0.0175
        blk = slice(0, m.n // 4)
        act = m.active[blk].astype(bool)
        l2 = np.sum(err[blk][act] ** 2 * m.area[blk][act]) / np.sum(exact[blk][act] ** 2 * m.area[blk][act])
        assert l2 <= 1.18e-4
        lc = lg.pse_sphere_laplacian_at_particles(m.x, m.y, m.z, np.full(m.n, 2.0), m.area, m.active, eps, mode=mode)
        assert np.abs(lc).max() <= 1e-10


@pytest.mark.parametrize("kernel", [0, 1])
def test_pse_vs_oracle(lg, wl, oracle_mod, kernel):
    c = wl.config_pse_cubed(4)
    eps = c["eps_k8"] if kernel == 0 else c["eps_gauss"]
    args = (c["x"], c["y"], c["z"], c["f"], c["area"], c["active"], eps)
    ref = oracle_mod.pse_laplacian(*args, 1.0, kernel)
    got = lg.pse_sphere_laplacian_at_particles(*args, 1.0, kernel)
    assert rel_linf(got, ref) <= 1e-12
    got32 = lg.pse_sphere_laplacian_at_particles(*args, 1.0, kernel, mode="fp32c")
    assert rel_linf(got32, ref) <= 1e-4


@pytest.mark.parametrize("nest,eps", [(6, 0.05), (6, 0.06), (7, None)])
def test_pse_k8_geodesic_series_vs_oracle(lg, wl, oracle_mod, nest, eps):
    """Cubed sphere with eps <= 0.06 (nest 7: eps = h^0.75): the FP32C K8-geodesic sum takes the
    chord-series angle; checked against the oracle on a block of targets."""
    c = wl.config_pse_cubed(nest)
    eps = c["eps_k8"] if eps is None else eps
    assert eps <= 0.06
    n = c["x"].size
    ib, m = n // 3, 4096
    args = (c["x"], c["y"], c["z"], c["f"], c["area"], c["active"], eps)
    ref = oracle_mod.pse_laplacian(*args, 1.0, 0, ib=ib, ie=ib + m)
    got = lg.pse_sphere_laplacian_at_particles(*args, 1.0, 0, i_begin=ib + 1, i_end=ib + m, mode="fp32c")
    assert rel_linf(got[ib:ib + m], ref) <= 1e-4


@pytest.mark.parametrize("nest,power,ib,m", [(4, 0.5, 0, None), (6, 0.5, 20000, 2048), (7, None, 60000, 2048)])
def test_pse_gradient_divergence_vs_oracle(lg, wl, oracle_mod, nest, power, ib, m):
    """PSE gradient of y54 and divergence of its exact gradient: FP64 within 1e-12 of the
    oracle (CUDA's and the C library's exp and atan2 may differ by an ulp), FP32C within
    1e-4.  eps = h^0.5 at nests 4 and 6 (0.31 and 0.16: the asin angle), 0.05 at nest 7 (the
    chord series); a block of targets where the oracle would be slow."""
    c = wl.config_pse_cubed(nest)
    n = c["x"].size
    eps = c["mesh"].max_edge_length ** power if power else 0.05
    ie = n if m is None else ib + m
    f = wl.y54(c["x"], c["y"], c["z"])
    v = wl.y54_surface_gradient(c["x"], c["y"], c["z"])
    pos = (c["x"], c["y"], c["z"])
    ref_g = np.stack(oracle_mod.pse_sphere_gradient(*pos, f, c["area"], c["active"], eps, ib=ib, ie=ie))
    ref_d = oracle_mod.pse_sphere_divergence(*pos, *v, c["area"], c["active"], eps, ib=ib, ie=ie)
    for mode, tol in (("fp64", 1e-12), ("fp32c", 1e-4)):
        if mode == "fp64" and m is not None and nest > 6:
            continue  # the FP64 sweep of nest 7 is covered by the smaller cases
        g = np.stack(lg.pse_sphere_gradient_at_particles(*pos, f, c["area"], c["active"], eps, i_begin=ib + 1,
                                                         i_end=ie, mode=mode))[:, ib:ie]
        d = lg.pse_sphere_divergence_at_particles(*pos, *v, c["area"], c["active"], eps, i_begin=ib + 1, i_end=ie,
                                                  mode=mode)[ib:ie]
        assert np.abs(g - ref_g).max() <= tol * np.abs(ref_g).max()
        assert np.abs(d - ref_d).max() <= tol * np.abs(ref_d).max()


@pytest.mark.parametrize("nest,power,m", [(5, 0.75, None), (5, 0.4, None), (7, 0.75, 2048)])
@pytest.mark.parametrize("kernel", [2, 1])
def test_pse_plane_fp32c_vs_oracle(lg, oracle_mod, nest, power, m, kernel):
    """Planar PSE Laplacian (K8 and Gaussian of the chord) on the quad mesh of [-4,4]^2, FP32C
    within 1e-4 of the oracle; eps = h^0.75 (the group cutoff skips most of the plane) and
    h^0.4 (it skips little); a block of targets at nest 7."""
    mesh = lg.PolyMesh2d(lg.QUAD_RECT_SEED, nest, 4.0)
    x, y = mesh.x, mesh.y
    rng = np.random.default_rng(nest)
    f = np.exp(-(x * x + y * y)) * np.cos(2.0 * x) + 1e-3 * rng.random(mesh.n)
    eps = mesh.max_edge_length ** power
    n = mesh.n
    ib = n // 3 if m else 0
    ie = ib + m if m else n
    ref = oracle_mod.pse_laplacian(x, y, None, f, mesh.area, mesh.active, eps, 1.0, kernel, ib=ib, ie=ie)
    got = lg.pse_plane_laplacian_at_particles(x, y, f, mesh.area, mesh.active, eps, kernel=kernel,
                                              i_begin=ib + 1, i_end=ie, mode="fp32c")[ib:ie]
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def test_check_finite_flag(lg):
    n = 4
    x = np.array([1.0, 0.0, 0.0, np.nan])
    y = np.array([0.0, 1.0, 0.0, 0.0])
    z = np.array([0.0, 0.0, 1.0, 0.0])
    act = np.ones(n, np.int32)
    with pytest.raises(lg.LpmError) as e:
        lg.bve_sphere_velocity(x, y, z, np.ones(n), np.ones(n), act, 1.0, mode=lg.MODE_FP64 | lg.FLAG_CHECK_FINITE)
    assert e.value.code == -4


# ------------------------------------------------------------------ stream functions, FP32C
# a^2 - x_i.x_j is formed without cancellation and the log is good to ~1 ulp; the terms
# cancel to a much smaller psi, so the bound is relative to max|psi| over the targets.
STREAM_TOL = 1e-6


def test_golden_stream_fp32c(lg):
    g = np.load(GOLDEN / "bve_icos2.npz")
    pr, pa = lg.set_stream_functions_on_mesh(g["x"], g["y"], g["z"], g["zeta"], g["absvort"], g["area"],
                                             g["active"], 1.0, mode="fp32c")
    assert rel_linf(pr, g["psi_rel"]) <= STREAM_TOL and rel_linf(pa, g["psi_abs"]) <= STREAM_TOL
    gp = np.load(GOLDEN / "plane_quad3.npz")
    ps = lg.set_stream_function_on_mesh(gp["x"], gp["y"], gp["omega"], gp["area"], gp["active"], mode="fp32c")
    assert rel_linf(ps, gp["psi"]) <= STREAM_TOL


@pytest.mark.parametrize("radius", [1.0, 6.37122e6])
def test_sphere_stream_fp32c_vs_oracle(lg, wl, oracle_mod, radius):
    """RH54 wave on a nest-4 icosahedral mesh, unit and Earth radius (absolute vorticity with
    the Earth's rotation rate scaled to the radius)."""
    c = wl.config_rh54_icos(4, seed=5)
    x, y, z = c["x"] * radius, c["y"] * radius, c["z"] * radius
    area = c["area"] * radius ** 2
    absv = c["zeta"] + 2.0 * (2.0 * np.pi) * c["z"]
    ref = oracle_mod.bve_stream(x, y, z, c["zeta"], absv, area, c["active"], radius)
    got = lg.set_stream_functions_on_mesh(x, y, z, c["zeta"], absv, area, c["active"], radius, mode="fp32c")
    assert rel_linf(got[0], ref[0]) <= STREAM_TOL and rel_linf(got[1], ref[1]) <= STREAM_TOL


@pytest.mark.parametrize("n", [1, 2, 33, 257, 1000])
def test_stream_fp32c_ragged_inactive_block(lg, oracle_mod, n):
    """Odd sizes, random activity (inactive targets have no self term to remove), a block range,
    and points slightly off the sphere (both signs of |x|^2 - a^2)."""
    rng = np.random.default_rng(100 + n)
    p = rng.normal(size=(3, n))
    p /= np.linalg.norm(p, axis=0)
    p *= 1.0 + 1e-9 * rng.normal(size=n)
    zeta = rng.normal(size=n)
    absv = zeta + rng.normal(size=n)
    area = rng.uniform(0.5, 1.5, size=n) * 4 * np.pi / n
    act = (rng.random(n) < 0.7).astype(np.int32)
    if not act.any():
        act[0] = 1
    ib, ie = (n // 3 + 1, n) if n > 3 else (1, n)
    ref = oracle_mod.bve_stream(p[0], p[1], p[2], zeta, absv, area, act)
    got = lg.set_stream_functions_on_mesh(p[0], p[1], p[2], zeta, absv, area, act, 1.0, i_begin=ib, i_end=ie,
                                          mode="fp32c")
    sl = slice(ib - 1, ie)
    # scale: max|psi|, or the sum of |zeta A| when psi nearly cancels (one active source)
    mass = np.sum(np.abs(zeta * area) * act)
    for got_c, ref_c in zip(got, ref):
        assert np.abs(got_c[sl] - ref_c[sl]).max() <= STREAM_TOL * max(np.abs(ref_c[sl]).max(), mass)
    q = rng.normal(size=(2, n))
    pref = oracle_mod.plane_stream(q[0], q[1], zeta, area, act)
    pgot = lg.set_stream_function_on_mesh(q[0], q[1], zeta, area, act, i_begin=ib, i_end=ie, mode="fp32c")
    assert np.abs(pgot[sl] - pref[sl]).max() <= STREAM_TOL * max(np.abs(pref[sl]).max(), mass)


def test_plane_stream_fp32c_dipoles(lg, wl, oracle_mod):
    c = wl.config_colliding_dipoles(5)
    ref = oracle_mod.plane_stream(c["x"], c["y"], c["omega"], c["area"], c["active"])
    got = lg.set_stream_function_on_mesh(c["x"], c["y"], c["omega"], c["area"], c["active"], mode="fp32c")
    assert rel_linf(got, ref) <= STREAM_TOL
