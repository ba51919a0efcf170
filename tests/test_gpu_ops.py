"""GPU parity of the remaining PSE operators and the shallow-water integrals (LPM_MODE_FP64)
through the C ABI, against the oracle: bit-identical where the loop has no transcendental
function (the SWE velocities and double dot products), within 1e-12 of max|result| where
exp/atan2 enter (CUDA's and the C library's may differ by an ulp).  Block ranges
(i_begin/i_end) and random activity masks are covered."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


def rel(got, ref):
    return np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)


def _plane(lg, nest, seed, frac_active=1.0):
    m = lg.PolyMesh2d(202, nest, 4.0)
    act = m.active.copy()
    if frac_active < 1.0:
        rng = np.random.default_rng(seed)
        act = act * (rng.random(m.n) < frac_active).astype(np.int32)
    eps = 2.0 * np.sqrt(m.area[m.active == 1].max())
    return m, act, eps


@pytest.mark.parametrize("nest,frac,block", [(3, 1.0, None), (4, 0.7, (17, 1500))])
def test_pse_plane_gradient_second_ddot(lg, oracle_mod, nest, frac, block):
    m, act, eps = _plane(lg, nest, 11, frac)
    rng = np.random.default_rng(2)
    f = np.sin(m.x) * np.cos(0.5 * m.y) + 0.01 * rng.random(m.n)
    ib, ie = (1, m.n) if block is None else block
    gx, gy = lg.pse_plane_gradient_at_particles(m.x, m.y, f, m.area, act, eps, ib, ie)
    rx, ry = oracle_mod.pse_plane_gradient(m.x, m.y, f, m.area, act, eps, ib - 1, ie)
    assert rel(gx[ib - 1:ie], rx) <= TOL and rel(gy[ib - 1:ie], ry) <= TOL
    assert np.all(gx[:ib - 1] == 0) and np.all(gx[ie:] == 0)
    xx, xy, yy = lg.pse_plane_second_partials_at_particles(m.x, m.y, f, 0.5 * f, m.area, act, eps, ib, ie)
    r = oracle_mod.pse_plane_second_partials(m.x, m.y, f, 0.5 * f, m.area, act, eps, ib - 1, ie)
    for g, rr in zip((xx, xy, yy), r):
        assert rel(g[ib - 1:ie], rr) <= TOL
    u, v = np.cos(m.y), 0.3 * np.sin(m.x)
    dd = lg.pse_plane_double_dot_product_at_particles(m.x, m.y, u, v, m.area, act, eps, ib, ie)
    rd = oracle_mod.pse_plane_double_dot(m.x, m.y, u, v, m.area, act, eps, ib - 1, ie)
    assert rel(dd[ib - 1:ie], rd) <= TOL


@pytest.mark.parametrize("radius", [1.0, 6.37122e6])
def test_pse_sphere_double_dot(lg, oracle_mod, radius):
    m = lg.PolyMesh2d(205, 3, 1.0)
    x, y, z = m.x * radius, m.y * radius, m.z * radius
    area = m.area * radius ** 2
    u, v, w = -m.y, m.x, 0.2 * m.z
    eps = 0.2 * radius
    got = lg.pse_sphere_double_dot_product_at_particles(x, y, z, u, v, w, area, m.active, eps, radius)
    ref = oracle_mod.pse_sphere_double_dot(x, y, z, u, v, w, area, m.active, eps, radius)
    assert rel(got, ref) <= TOL


def test_pse_interpolation_plane_and_sphere(lg, oracle_mod):
    m, act, eps = _plane(lg, 4, 0)
    f = np.cos(m.x) * np.sin(m.y)
    rng = np.random.default_rng(9)
    qx, qy = rng.uniform(-3, 3, 257), rng.uniform(-3, 3, 257)
    got = lg.pse_interpolate_scalar(m.x, m.y, None, f, m.area, act, eps, qx, qy)
    ref = oracle_mod.pse_interpolate(m.x, m.y, None, f, m.area, act, eps, qx, qy, None, 0)
    assert rel(got, ref) <= TOL
    s = lg.PolyMesh2d(206, 4, 1.0)
    q = rng.standard_normal((3, 100))
    q /= np.linalg.norm(q, axis=0)
    fs = 1.0 + s.z + s.x * s.y
    eps_s = 2.0 * np.sqrt(s.area[s.active == 1].max())
    got = lg.pse_interpolate_scalar(s.x, s.y, s.z, fs, s.area, s.active, eps_s, q[0], q[1], q[2],
                                    geometry=lg.GEOMETRY_SPHERE)
    ref = oracle_mod.pse_interpolate(s.x, s.y, s.z, fs, s.area, s.active, eps_s, q[0], q[1], q[2], 1)
    assert rel(got, ref) <= TOL


@pytest.mark.parametrize("nest,block", [(3, None), (4, (100, 2000))])
def test_swe_plane_rhs(lg, oracle_mod, nest, block):
    m, act, eps = _plane(lg, nest, 4, 0.9)
    vort = np.exp(-(m.x ** 2 + m.y ** 2))
    div = 0.3 * np.exp(-((m.x - 1) ** 2 + m.y ** 2))
    sh = 1.0 + 0.1 * np.cos(m.x)
    ib, ie = (1, m.n) if block is None else block
    got = lg.swe_plane_rhs_integrals(m.x, m.y, vort, div, sh, m.area, act, eps, ib, ie)
    ref = oracle_mod.swe_plane_rhs(m.x, m.y, vort, div, sh, m.area, act, eps, ib - 1, ie)
    s = slice(ib - 1, ie)
    # velocity and double dot: no transcendental function in the loop -> bit-identical
    assert np.array_equal(got[0][s], ref[0]) and np.array_equal(got[1][s], ref[1])
    assert np.array_equal(got[2][s], ref[2])
    assert rel(got[3][s], ref[3]) <= TOL


@pytest.mark.parametrize("radius,sphere_radius", [(1.0, 1.0), (6.37122e6, 1.0)])
def test_swe_sphere_rhs(lg, oracle_mod, radius, sphere_radius):
    m = lg.PolyMesh2d(205, 3, 1.0)
    x, y, z = m.x * radius, m.y * radius, m.z * radius
    area = m.area * radius ** 2
    zeta = np.exp(-4 * ((m.x - 0.5) ** 2 + m.y ** 2 + (m.z - 0.7) ** 2))
    div = 0.1 * np.cos(3 * m.z)
    sh = 1.0 + 0.2 * m.z
    eps = 0.25
    got = lg.swe_sphere_rhs_integrals(x, y, z, zeta, div, sh, area, m.active, radius, eps, sphere_radius, 5, 1800)
    ref = oracle_mod.swe_sphere_rhs(x, y, z, zeta, div, sh, area, m.active, radius, sphere_radius, eps, 4, 1800)
    s = slice(4, 1800)
    for c in range(3):
        assert np.array_equal(got[c][s], ref[c])
    assert np.all(got[3][s] == 0.0)
    assert rel(got[4][s], ref[4]) <= TOL


@pytest.mark.parametrize("n,frac,block", [(1000, 0.8, None), (4099, 1.0, (33, 4000))])
def test_beta_plane_velocity_and_stream(lg, oracle_mod, n, frac, block):
    rng = np.random.default_rng(n)
    x, y = rng.random(n), rng.uniform(-0.5, 0.5, n)
    area = rng.uniform(0.5, 1.5, n) / n
    zeta = np.sin(2 * np.pi * x) * np.exp(-8 * y * y)
    absv = zeta + 3.0 * y
    act = (rng.random(n) < frac).astype(np.int32)
    ib, ie = (1, n) if block is None else block
    # The reference's denominator cosh(2 pi dy) - cos(2 pi dx) cancels for close pairs: an ulp
    # of difference between CUDA's and the C library's cosh/cos (about 1e-16 of 1) becomes
    # 1e-16 / (2 pi^2 r^2) of that pair's term, ~1e-11 for the closest random pairs here.
    tol = 1e-9
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, ib, ie)
    ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act, ib - 1, ie)
    s = slice(ib - 1, ie)
    assert rel(u[s], ru) <= tol and rel(v[s], rv) <= tol
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, ib, ie)
    rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act, ib - 1, ie)
    assert rel(pr[s], rr) <= tol and rel(pa[s], ra) <= tol


def test_beta_plane_band_known_answer_gpu(lg):
    nx = ny = 64
    xs = (np.arange(nx) + 0.5) / nx
    ys = -0.5 + (np.arange(ny) + 0.5) / ny
    X, Y = (a.ravel() for a in np.meshgrid(xs, ys))
    A = np.full(X.size, 1.0 / (nx * ny))
    Z = np.where(np.abs(Y) < 0.25, 1.0, 0.0)
    u, v = lg.beta_plane_velocity(X, Y, Z, A, np.ones(X.size, dtype=np.int32))
    assert np.abs(u + Y)[np.abs(Y) < 0.2].max() < 1e-11 and np.abs(v).max() < 1e-12


FP32C_TOL = 1e-6


@pytest.mark.parametrize("n,frac,block,spread", [(1000, 0.8, None, 0.5), (5003, 1.0, (7, 4900), 0.5),
                                                 (3000, 0.9, None, 3.0)])
def test_beta_plane_velocity_fp32c(lg, oracle_mod, n, frac, block, spread):
    """FP32C against the oracle: random particles on the strip (y up to +-spread, so sinh/cosh
    reach e^(2 pi spread)), a cluster straddling the periodic boundary x = 0 ~ 1, positions
    shifted by whole periods (x outside [0, 1])."""
    rng = np.random.default_rng(n + 1)
    x, y = rng.random(n), rng.uniform(-spread, spread, n)
    x[:50] = np.mod(rng.normal(0.0, 1e-3, 50), 1.0)  # neighbours across x = 0 / 1
    y[:50] = rng.normal(0.0, 1e-3, 50)
    x[50:80] += rng.integers(-3, 4, 30)  # whole periods
    area = rng.uniform(0.5, 1.5, n) / n
    zeta = np.sin(2 * np.pi * x) * np.exp(-4 * y * y) + 0.3
    act = (rng.random(n) < frac).astype(np.int32)
    ib, ie = (1, n) if block is None else block
    s = slice(ib - 1, ie)
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, ib, ie, mode="fp32c")
    ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act, ib - 1, ie)
    scale = max(np.abs(ru).max(), np.abs(rv).max())
    assert max(np.abs(u[s] - ru).max(), np.abs(v[s] - rv).max()) <= FP32C_TOL * scale


def test_beta_plane_band_fp32c(lg):
    nx = ny = 128
    xs = (np.arange(nx) + 0.5) / nx
    ys = -0.5 + (np.arange(ny) + 0.5) / ny
    X, Y = (a.ravel() for a in np.meshgrid(xs, ys))
    A = np.full(X.size, 1.0 / (nx * ny))
    Z = np.where(np.abs(Y) < 0.25, 1.0, 0.0)
    u, v = lg.beta_plane_velocity(X, Y, Z, A, np.ones(X.size, dtype=np.int32), mode="fp32c")
    assert np.abs(u + Y)[np.abs(Y) < 0.2].max() < FP32C_TOL * 0.25 and np.abs(v).max() < FP32C_TOL * 0.25


@pytest.mark.parametrize("nest,frac,block", [(4, 1.0, None), (5, 0.9, (100, 7000))])
def test_swe_plane_rhs_fp32c(lg, oracle_mod, nest, frac, block):
    """FP32C planar SWE integrals against the FP64 oracle: velocity to 1e-6 of max|(u, v)|, the
    double dot product to 2e-6 of its max (a quadratic form of 1/r^2 sums; 6.9e-7 measured),
    the surface-height Laplacian to the planar PSE FP32C bound 1e-4."""
    m, act, eps = _plane(lg, nest, 7, frac)
    vort = 4.0 * np.exp(-((m.x - 0.5) ** 2 + m.y ** 2) / 0.3) - 4.0 * np.exp(-((m.x + 0.5) ** 2 + m.y ** 2) / 0.3)
    div = 0.5 * np.exp(-(m.x ** 2 + (m.y - 0.5) ** 2) / 0.5)
    sh = 1.0 + 0.1 * np.cos(m.x) * np.sin(0.5 * m.y)
    ib, ie = (1, m.n) if block is None else block
    s = slice(ib - 1, ie)
    got = lg.swe_plane_rhs_integrals(m.x, m.y, vort, div, sh, m.area, act, eps, ib, ie, mode="fp32c")
    ref = oracle_mod.swe_plane_rhs(m.x, m.y, vort, div, sh, m.area, act, eps, ib - 1, ie)
    vel = max(np.abs(ref[0]).max(), np.abs(ref[1]).max())
    err = [np.abs(got[0][s] - ref[0]).max() / vel, np.abs(got[1][s] - ref[1]).max() / vel,
           rel(got[2][s], ref[2]), rel(got[3][s], ref[3])]
    print("swe fp32c errors", err)
    assert err[0] <= FP32C_TOL and err[1] <= FP32C_TOL
    assert err[2] <= 2e-6
    assert err[3] <= 1e-4


@pytest.mark.parametrize("nest,radius,sphere_radius,block", [(4, 1.0, 1.0, None), (5, 6.37122e6, 1.0, (50, 20000)),
                                                             (4, 2.0, 2.0, None)])
def test_swe_sphere_rhs_fp32c(lg, oracle_mod, nest, radius, sphere_radius, block):
    """FP32C sphere SWE integrals against the FP64 oracle: velocity (rotational and potential
    parts in one sweep) to 1e-6 of max|(u, v, w)|, the surface-height Laplacian (the geodesic
    PSE sweep at eps a / SphereRadius) to the PSE FP32C bound 1e-4, doubleDot 0."""
    m = lg.PolyMesh2d(205, nest, 1.0)
    x, y, z = m.x * radius, m.y * radius, m.z * radius
    area = m.area * radius ** 2
    zeta = np.exp(-4 * ((m.x - 0.5) ** 2 + m.y ** 2 + (m.z - 0.7) ** 2)) + 0.3 * m.z
    div = 0.2 * np.cos(3 * m.z) * np.sin(2 * m.x)
    sh = 1.0 + 0.2 * m.z + 0.05 * m.x * m.y
    eps = 0.15 * sphere_radius
    ib, ie = (1, m.n) if block is None else block
    s = slice(ib - 1, ie)
    got = lg.swe_sphere_rhs_integrals(x, y, z, zeta, div, sh, area, m.active, radius, eps, sphere_radius, ib, ie,
                                      mode="fp32c")
    ref = oracle_mod.swe_sphere_rhs(x, y, z, zeta, div, sh, area, m.active, radius, sphere_radius, eps, ib - 1, ie)
    vel = max(np.abs(ref[c]).max() for c in range(3))
    err = [np.abs(got[c][s] - ref[c]).max() / vel for c in range(3)] + [rel(got[4][s], ref[4])]
    print("swe sphere fp32c errors", err)
    assert max(err[:3]) <= FP32C_TOL
    assert np.all(got[3][s] == 0.0)
    assert err[3] <= 1e-4


@pytest.mark.parametrize("n,frac,spread", [(1000, 0.8, 0.5), (4099, 1.0, 0.5), (3000, 0.9, 3.0)])
def test_beta_plane_stream_fp32c(lg, oracle_mod, n, frac, spread):
    """FP32C beta-plane stream functions against the oracle, to 1e-6 of max|psi|, with
    neighbours across the periodic boundary and positions shifted by whole periods."""
    rng = np.random.default_rng(n + 7)
    x, y = rng.random(n), rng.uniform(-spread, spread, n)
    x[:50] = np.mod(rng.normal(0.0, 1e-3, 50), 1.0)
    y[:50] = rng.normal(0.0, 1e-3, 50)
    x[50:80] += rng.integers(-3, 4, 30)
    area = rng.uniform(0.5, 1.5, n) / n
    zeta = np.sin(2 * np.pi * x) * np.exp(-4 * y * y)
    absv = zeta + 5.0 * y
    act = (rng.random(n) < frac).astype(np.int32)
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, mode="fp32c")
    rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act)
    err = (rel(pr, rr), rel(pa, ra))
    print("beta stream fp32c", err)
    assert max(err) <= FP32C_TOL


def test_beta_plane_fp32c_far_groups_quad7(lg, oracle_mod):
    """The beta-plane particle set at quad nest 7 (R = 0.019 for 64-source groups, so most
    target/group pairs take the complex far form), FP32C against the oracle on two target
    blocks, velocity and stream functions to 1e-6 of their max."""
    import workloads as wl

    c = wl.config_beta_plane(7)
    x, y, zeta, area, act = c["x"], c["y"], c["zeta"], c["area"], c["active"]
    absv = zeta + 3.0 * y
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, mode="fp32c")
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, mode="fp32c")
    for ib, ie in ((0, 2048), (70001, 72048)):
        ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act, ib, ie)
        rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act, ib, ie)
        s = slice(ib, ie)
        assert max(rel(u[s], ru), rel(v[s], rv)) <= FP32C_TOL
        assert max(rel(pr[s], rr), rel(pa[s], ra)) <= FP32C_TOL


def test_beta_plane_fp32c_distant_clusters(lg, oracle_mod):
    """Two compact clusters 14 apart in y (and a sparse band between them): the velocity's far
    form clamps |y_i - y_o| to 6 (the terms have reached their limits there), and the stream's
    far form hands |y_i - y_o| > 6 to the direct form."""
    rng = np.random.default_rng(11)
    n = 3000
    x = rng.random(n)
    y = np.concatenate([rng.normal(-7.0, 0.02, 1400), rng.normal(7.0, 0.02, 1400), rng.uniform(-8, 8, 200)])
    area = rng.uniform(0.5, 1.5, n) / n
    zeta = np.cos(2 * np.pi * x) + 0.2 * np.sign(y)
    absv = zeta + 0.5 * y
    act = np.ones(n, np.int32)
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, mode="fp32c")
    ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act)
    assert max(rel(u, ru), rel(v, rv)) <= FP32C_TOL
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, mode="fp32c")
    rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act)
    assert max(rel(pr, rr), rel(pa, ra)) <= FP32C_TOL


@pytest.mark.parametrize("radius", [0.03, 0.08])
def test_beta_plane_fp32c_targets_just_beyond_near_limit(lg, oracle_mod, radius):
    """Targets in the band 4.05R-4.95R of one compact group of 64 sources: every warp takes the
    complex far form there (the near limit is max(4R, 0.02)), where its cancellation is the
    largest.  Velocity and stream functions against the oracle to 1e-6 of their max."""
    rng = np.random.default_rng(int(radius * 1000))
    ns, nt = 64, 4096
    sx = 0.5 + radius * 0.5 * rng.uniform(-1, 1, ns)
    sy = radius * 0.5 * rng.uniform(-1, 1, ns)
    o = np.array([sx.mean(), sy.mean()])
    R = np.sqrt((sx - o[0]) ** 2 + (sy - o[1]) ** 2).max()
    rho = R * rng.uniform(4.05, 4.95, nt)
    th = rng.uniform(0.0, 2.0 * np.pi, nt)
    x = np.concatenate([sx, o[0] + rho * np.cos(th)])
    y = np.concatenate([sy, o[1] + rho * np.sin(th)])
    area = np.concatenate([rng.uniform(0.5, 1.5, ns) * 1e-3, np.zeros(nt)])
    zeta = np.concatenate([rng.uniform(-1.0, 1.0, ns) + 0.3, np.zeros(nt)])
    absv = zeta + 2.0 * y
    act = np.concatenate([np.ones(ns), np.zeros(nt)]).astype(np.int32)
    ib, ie = ns + 1, ns + nt
    s = slice(ib - 1, ie)
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, ib, ie, mode="fp32c")
    ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act, ib - 1, ie)
    scale = max(np.abs(ru).max(), np.abs(rv).max())
    assert max(np.abs(u[s] - ru).max(), np.abs(v[s] - rv).max()) <= FP32C_TOL * scale
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, ib, ie, mode="fp32c")
    rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act, ib - 1, ie)
    assert max(rel(pr[s], rr), rel(pa[s], ra)) <= FP32C_TOL


@pytest.mark.parametrize("n", [1, 2, 63, 65, 257, 1031])
def test_beta_plane_fp32c_ragged_and_empty(lg, oracle_mod, n):
    """Ragged sizes (partial groups and tiles, inert records) and a set with no active source
    (every sum is exactly zero)."""
    rng = np.random.default_rng(n)
    x, y = rng.random(n), rng.uniform(-0.5, 0.5, n)
    area = rng.uniform(0.5, 1.5, n) / n
    zeta = np.sin(2 * np.pi * x) + y
    absv = zeta + y
    act = (rng.random(n) < 0.8).astype(np.int32)
    act[0] = 1
    u, v = lg.beta_plane_velocity(x, y, zeta, area, act, mode="fp32c")
    ru, rv = oracle_mod.beta_plane_velocity(x, y, zeta, area, act)
    scale = max(np.abs(ru).max(), np.abs(rv).max(), 1e-300)
    assert max(np.abs(u - ru).max(), np.abs(v - rv).max()) <= FP32C_TOL * scale
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, act, mode="fp32c")
    rr, ra = oracle_mod.beta_plane_stream(x, y, zeta, absv, area, act)
    scale = max(np.abs(rr).max(), np.abs(ra).max(), 1e-300)
    assert max(np.abs(pr - rr).max(), np.abs(pa - ra).max()) <= FP32C_TOL * scale
    none = np.zeros(n, np.int32)
    u, v = lg.beta_plane_velocity(x, y, zeta, area, none, mode="fp32c")
    pr, pa = lg.beta_plane_stream_functions(x, y, zeta, absv, area, none, mode="fp32c")
    assert not np.any(u) and not np.any(v) and not np.any(pr) and not np.any(pa)


def test_pse_fp64_tile_cutoff_plane(lg, oracle_mod):
    """The FP64 PSE sweeps skip source tiles beyond r = 7 (every kernel below 1e-14 of its peak):
    at quad nest 6 on [-4,4]^2 with eps = 2h = 0.25 (reach 1.75) most tiles are out of a warp's
    reach, and every planar operator stays within 1e-12 of the all-pairs oracle, on a block of
    targets too."""
    m, act, eps = _plane(lg, 6, 21)
    f = np.exp(-0.3 * (m.x ** 2 + m.y ** 2)) * np.cos(m.x) + 0.2
    u, v = np.cos(0.5 * m.y), 0.3 * np.sin(m.x)
    for ib, ie in ((1, m.n), (5001, 9000)):
        s = slice(ib - 1, ie)
        gx, gy = lg.pse_plane_gradient_at_particles(m.x, m.y, f, m.area, act, eps, ib, ie)
        rx, ry = oracle_mod.pse_plane_gradient(m.x, m.y, f, m.area, act, eps, ib - 1, ie)
        assert rel(gx[s], rx) <= TOL and rel(gy[s], ry) <= TOL
        xx, xy, yy = lg.pse_plane_second_partials_at_particles(m.x, m.y, u, v, m.area, act, eps, ib, ie)
        r = oracle_mod.pse_plane_second_partials(m.x, m.y, u, v, m.area, act, eps, ib - 1, ie)
        for g, rr in zip((xx, xy, yy), r):
            assert rel(g[s], rr) <= TOL
        dd = lg.pse_plane_double_dot_product_at_particles(m.x, m.y, u, v, m.area, act, eps, ib, ie)
        rd = oracle_mod.pse_plane_double_dot(m.x, m.y, u, v, m.area, act, eps, ib - 1, ie)
        assert rel(dd[s], rd) <= TOL
        lap = lg.pse_plane_laplacian_at_particles(m.x, m.y, f, m.area, act, eps, kernel=lg.PSE_K8_CHORD,
                                                  i_begin=ib, i_end=ie, mode="fp64")
        rl = oracle_mod.pse_laplacian(m.x, m.y, None, f, m.area, act, eps, 1.0, oracle_mod.PSE_K8_CHORD, ib - 1, ie)
        assert rel(lap[s], rl) <= TOL
    rng = np.random.default_rng(4)
    qx, qy = rng.uniform(-3.5, 3.5, 2000), rng.uniform(-3.5, 3.5, 2000)
    got = lg.pse_interpolate_scalar(m.x, m.y, None, f, m.area, act, eps, qx, qy)
    ref = oracle_mod.pse_interpolate(m.x, m.y, None, f, m.area, act, eps, qx, qy, None, 0)
    assert rel(got, ref) <= TOL


@pytest.mark.parametrize("radius", [1.0, 6.37122e6])
def test_pse_fp64_tile_cutoff_sphere(lg, oracle_mod, radius):
    """The great-circle FP64 PSE sweeps with the tile cutoff (reach 7 eps / radius on unit
    directions) at cubed nest 5 with eps = 0.06 radius: Laplacian (K8 geodesic and Gaussian
    chord), gradient, divergence and double dot within 1e-12 of the all-pairs oracle."""
    m = lg.PolyMesh2d(lg.CUBED_SPHERE_SEED, 5, 1.0)
    x, y, z = m.x * radius, m.y * radius, m.z * radius
    area = m.area * radius ** 2
    act = m.active.copy()
    f = np.cos(3.0 * m.x) * np.sin(2.0 * m.z) + 0.5
    u, v, w = -m.y, m.x, 0.2 * m.z
    eps = 0.06 * radius
    for origin in (False, True):
        if origin:
            # a particle at the centre: no direction, and at great-circle distance 0 from every
            # other (atan2(0, 0) = 0), so no tile may be skipped for it or for its tile
            x, y, z, area, f, u, v, w = (np.append(a, val) for a, val in
                                         ((x, 0.0), (y, 0.0), (z, 0.0), (area, 1e-4 * radius ** 2), (f, 0.7),
                                          (u, 0.1), (v, 0.2), (w, 0.3)))
            act = np.append(act, 1).astype(np.int32)
        for kern in (lg.PSE_K8_GEODESIC, lg.PSE_GAUSS_CHORD):
            got = lg.pse_sphere_laplacian_at_particles(x, y, z, f, area, act, eps, radius, kern, mode="fp64")
            ref = oracle_mod.pse_laplacian(x, y, z, f, area, act, eps, radius, kern)
            assert rel(got, ref) <= TOL
        g = lg.pse_sphere_gradient_at_particles(x, y, z, f, area, act, eps, radius, mode="fp64")
        r = oracle_mod.pse_sphere_gradient(x, y, z, f, area, act, eps, radius)
        for a, b in zip(g, r):
            assert rel(a, b) <= TOL
        d = lg.pse_sphere_divergence_at_particles(x, y, z, u, v, w, area, act, eps, radius, mode="fp64")
        rd = oracle_mod.pse_sphere_divergence(x, y, z, u, v, w, area, act, eps, radius)
        assert rel(d, rd) <= TOL
        dd = lg.pse_sphere_double_dot_product_at_particles(x, y, z, u, v, w, area, act, eps, radius)
        rdd = oracle_mod.pse_sphere_double_dot(x, y, z, u, v, w, area, act, eps, radius)
        assert rel(dd, rdd) <= TOL
