"""CPU tests of the oracle's remaining PSE operators and shallow-water integrals
(src/PSEDirectSum.f90:128-456, src/SWEPlaneSolver.f90:457-571, src/SphereSWESolver.f90:299-372):
known answers for the planar PSE operators, cross-checks of the sphere double dot product and
the SWE integrals against independent numpy restatements and against the velocity and
Laplacian sums they contain, and the C ABI's refusal of LPM_MODE_FP32C for them."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def plane(built_lib):
    m = built_lib.PolyMesh2d(202, 5, 4.0)  # quad mesh on [-4, 4]^2, 8321 particles, h = 1/8
    h = np.sqrt(m.area[m.active == 1].max())
    return m, 2.0 * h


@pytest.fixture(scope="module")
def sphere(built_lib):
    m = built_lib.PolyMesh2d(205, 3, 1.0)  # icosahedral nest 3, 1922 particles
    return m


def _inner(m):
    return (np.abs(m.x) < 2.0) & (np.abs(m.y) < 2.0)


def test_plane_gradient_known_answer(plane, oracle_mod):
    """Exact for f = 0.3 x - 0.7 y + 0.1 x y away from the boundary."""
    m, eps = plane
    f = 0.3 * m.x - 0.7 * m.y + 0.1 * m.x * m.y
    gx, gy = oracle_mod.pse_plane_gradient(m.x, m.y, f, m.area, m.active, eps)
    i = _inner(m)
    assert np.abs(gx - (0.3 + 0.1 * m.y))[i].max() < 1e-8
    assert np.abs(gy - (-0.7 + 0.1 * m.x))[i].max() < 1e-8


def test_plane_second_partials_known_answer(plane, oracle_mod):
    """The Hessian [[2, 3], [3, -2]] of x^2 + 3 x y - y^2 from its exact gradient."""
    m, eps = plane
    xx, xy, yy = oracle_mod.pse_plane_second_partials(m.x, m.y, 2 * m.x + 3 * m.y, 3 * m.x - 2 * m.y, m.area,
                                                       m.active, eps)
    i = _inner(m)
    assert np.abs(xx - 2.0)[i].max() < 1e-8
    assert np.abs(xy - 3.0)[i].max() < 1e-8
    assert np.abs(yy + 2.0)[i].max() < 1e-8


def test_plane_double_dot_known_answer(plane, oracle_mod):
    """u = (a x + b y, c x + d y): ux ux + 2 uy vx + vy vy = a^2 + 2 b c + d^2."""
    m, eps = plane
    a, b, c, d = 0.5, -1.2, 0.8, 0.3
    dd = oracle_mod.pse_plane_double_dot(m.x, m.y, a * m.x + b * m.y, c * m.x + d * m.y, m.area, m.active, eps)
    assert np.abs(dd - (a * a + 2 * b * c + d * d))[_inner(m)].max() < 1e-8


def test_plane_interpolation_known_answer(plane, oracle_mod):
    m, eps = plane
    f = np.cos(m.x) * np.sin(m.y)
    qx = np.array([0.1, -0.5, 1.3, 0.0])
    qy = np.array([0.2, 0.7, -1.1, 0.0])
    got = oracle_mod.pse_interpolate(m.x, m.y, None, f, m.area, m.active, eps, qx, qy, None, 0)
    assert np.abs(got - np.cos(qx) * np.sin(qy)).max() < 1e-6


def test_sphere_interpolation_converges(built_lib, oracle_mod):
    """The planar delta kernel on the sphere carries an O(eps^2) curvature error: a few
    percent at icos nest 3 with eps = 2h, and it falls with refinement."""
    q = np.array([[0.6, 0.0, 0.8], [0.0, -1.0, 0.0], [1 / np.sqrt(3)] * 3])
    want = 1.0 + q[:, 2] + q[:, 0] * q[:, 1]
    errs = []
    for nest in (3, 4):
        m = built_lib.PolyMesh2d(205, nest, 1.0)
        eps = 2.0 * np.sqrt(m.area[m.active == 1].max())
        f = 1.0 + m.z + m.x * m.y
        got = oracle_mod.pse_interpolate(m.x, m.y, m.z, f, m.area, m.active, eps, q[:, 0], q[:, 1], q[:, 2], 1)
        errs.append(np.abs(got - want).max())
    assert errs[0] < 0.05 and errs[1] < 0.5 * errs[0]


def _sphere_ddot_numpy(x, y, z, u, v, w, area, active, eps, radius):
    out = np.zeros(x.size)
    j = active.astype(bool)
    for i in range(x.size):
        a = np.stack([x[i], y[i], z[i]])
        b = np.stack([x[j], y[j], z[j]])
        cr = np.cross(a[:, None], b, axis=0)
        d = np.arctan2(np.sqrt((cr * cr).sum(0)), (a[:, None] * b).sum(0)) * radius
        k = (-20 + 20 * (d / eps) ** 2 - 5 * (d / eps) ** 4 + (d / eps) ** 6 / 3) * np.exp(-(d / eps) ** 2) / np.pi
        k = k / eps ** 2 * area[j] / eps
        dx = (x[i] - x[j], y[i] - y[j], z[i] - z[j])
        su, sv, sw = u[j] + u[i], v[j] + v[i], w[j] + v[i]
        g = [[(s * dd * k).sum() for dd in dx] for s in (su, sv, sw)]
        out[i] = (g[0][0] ** 2 + g[1][1] ** 2 + g[2][2] ** 2 + 2 * (g[0][1] * g[1][0] + g[0][2] * g[2][0]
                                                                 + g[1][2] * g[2][1])) / eps ** 2
    return out


def test_sphere_double_dot_vs_numpy(built_lib, oracle_mod):
    m = built_lib.PolyMesh2d(205, 2, 1.0)
    rng = np.random.default_rng(3)
    u, v, w = (rng.standard_normal(m.n) for _ in range(3))
    eps = 0.3
    got = oracle_mod.pse_sphere_double_dot(m.x, m.y, m.z, u, v, w, m.area, m.active, eps, 1.0)
    ref = _sphere_ddot_numpy(m.x, m.y, m.z, u, v, w, m.area, m.active, eps, 1.0)
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def _swe_plane_numpy(x, y, vort, div, sh, area, active, eps):
    n = x.size
    u, v, dd, lap = (np.zeros(n) for _ in range(4))
    j = np.nonzero(active)[0]
    for i in range(n):
        dx, dy = x[i] - x[j], y[i] - y[j]
        sq = dx * dx + dy * dy
        r = np.sqrt(sq) / eps
        k8 = (40 - 40 * r ** 2 + 10 * r ** 4 - 2 * r ** 6 / 3) * np.exp(-r * r) / np.pi
        lap[i] = (k8 / eps ** 2 * (sh[j] - sh[i]) * area[j]).sum() / eps ** 2
        o = j != i
        dx, dy, sq, jj = dx[o], dy[o], sq[o], j[o]
        rot = vort[jj] * area[jj] / (2 * np.pi * sq)
        pot = div[jj] * area[jj] / (2 * np.pi * sq)
        d2 = np.pi * sq * sq
        u[i] = (-dy * rot + dx * pot).sum()
        v[i] = (dx * rot + dy * pot).sum()
        cu = dx * div[jj] - dy * vort[jj]
        cv = dy * div[jj] + dx * vort[jj]
        ux = (pot - dx * cu * area[jj] / d2).sum()
        uy = (-rot - dy * cu * area[jj] / d2).sum()
        vx = (rot - dx * cv * area[jj] / d2).sum()
        vy = (pot - dy * cv * area[jj] / d2).sum()
        dd[i] = ux * ux + 2 * uy * vx + vy * vy
    return u, v, dd, lap


def test_swe_plane_vs_numpy_and_parts(built_lib, oracle_mod):
    m = built_lib.PolyMesh2d(202, 3, 4.0)
    rng = np.random.default_rng(5)
    vort = np.exp(-(m.x ** 2 + m.y ** 2))
    div = 0.3 * np.exp(-((m.x - 1) ** 2 + m.y ** 2))
    sh = 1.0 + 0.1 * np.cos(m.x) + 0.01 * rng.random(m.n)
    eps = 2.0 * np.sqrt(m.area[m.active == 1].max())
    got = oracle_mod.swe_plane_rhs(m.x, m.y, vort, div, sh, m.area, m.active, eps)
    ref = _swe_plane_numpy(m.x, m.y, vort, div, sh, m.area, m.active, eps)
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() <= 1e-11 * np.abs(r).max()
    # with zero divergence the velocity is the planar Biot-Savart sum, and lapSurf is the PSE
    # planar Laplacian of the surface height
    u, v, _, lap = oracle_mod.swe_plane_rhs(m.x, m.y, vort, 0 * div, sh, m.area, m.active, eps)
    ub, vb = oracle_mod.plane_velocity(m.x, m.y, vort, m.area, m.active, 0.0)
    assert np.abs(u - ub).max() <= 1e-13 * np.abs(ub).max() and np.abs(v - vb).max() <= 1e-13 * np.abs(vb).max()
    lp = oracle_mod.pse_laplacian(m.x, m.y, None, sh, m.area, m.active, eps, 1.0, oracle_mod.PSE_K8_CHORD)
    assert np.abs(lap - lp).max() <= 1e-12 * np.abs(lp).max()


def test_swe_sphere_vs_parts(sphere, oracle_mod):
    """Zero divergence: (u, v, w) is the BVE velocity on the unit sphere, lapSurf is eps^2 times
    the PSE K8-geodesic Laplacian of the surface height, and doubleDot is 0."""
    m = sphere
    zeta = np.exp(-4 * ((m.x - 0.5) ** 2 + m.y ** 2 + (m.z - 0.7) ** 2))
    zeta -= (zeta * m.area).sum() / m.area.sum()
    sh = 1.0 + 0.2 * m.z
    eps = 0.25
    u, v, w, dd, lap = oracle_mod.swe_sphere_rhs(m.x, m.y, m.z, zeta, 0 * zeta, sh, m.area, m.active, 1.0, 1.0, eps)
    ub, vb, wb = oracle_mod.bve_velocity(m.x, m.y, m.z, zeta, m.area, m.active, 1.0)
    scale = max(np.abs(ub).max(), np.abs(vb).max(), np.abs(wb).max())
    assert max(np.abs(u - ub).max(), np.abs(v - vb).max(), np.abs(w - wb).max()) <= 1e-13 * scale
    lp = oracle_mod.pse_laplacian(m.x, m.y, m.z, sh, m.area, m.active, eps, 1.0, oracle_mod.PSE_K8_GEODESIC)
    assert np.abs(lap - eps * eps * lp).max() <= 1e-12 * np.abs(eps * eps * lp).max()
    assert np.all(dd == 0.0)
    # the potential part: a pure divergence field gives velocity along -x_j weighted sums
    div = np.cos(3 * m.z)
    u2, v2, w2, _, _ = oracle_mod.swe_sphere_rhs(m.x, m.y, m.z, 0 * zeta, div, sh, m.area, m.active, 1.0, 1.0, eps)
    act = m.active == 1
    i = 7
    dp = m.x[i] * m.x + m.y[i] * m.y + m.z[i] * m.z
    pot = div * m.area / (4 * np.pi * (1 - dp))
    sel = act & (np.arange(m.n) != i)
    assert abs(u2[i] + (m.x * pot)[sel].sum()) <= 1e-12 * np.abs(m.x * pot)[sel].sum()


@pytest.mark.parametrize("call", ["plane_grad", "plane_second", "plane_ddot", "sphere_ddot", "interp"])
def test_fp32c_rejected_for_fp64_only_operators(lg, call):
    n = 4
    x = np.linspace(0.0, 1.0, n)
    a = np.ones(n)
    act = np.ones(n, dtype=np.int32)
    fn = {
        "plane_grad": lambda: lg.pse_plane_gradient_at_particles(x, x, a, a, act, 0.1, mode="fp32c"),
        "plane_second": lambda: lg.pse_plane_second_partials_at_particles(x, x, a, a, a, act, 0.1, mode="fp32c"),
        "plane_ddot": lambda: lg.pse_plane_double_dot_product_at_particles(x, x, a, a, a, act, 0.1, mode="fp32c"),
        "sphere_ddot": lambda: lg.pse_sphere_double_dot_product_at_particles(x, x, x, a, a, a, a, act, 0.1,
                                                                             mode="fp32c"),
        "interp": lambda: lg.pse_interpolate_scalar(x, x, None, a, a, act, 0.1, x[:2], x[:2], mode="fp32c"),
    }[call]
    with pytest.raises(lg.LpmError) as e:
        fn()
    assert "FP64" in str(e.value)


def _band(nx=64, ny=64, b=0.25):
    xs = (np.arange(nx) + 0.5) / nx
    ys = -0.5 + (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(xs, ys)
    X, Y = X.ravel(), Y.ravel()
    return X, Y, np.full(X.size, 1.0 / (nx * ny)), np.where(np.abs(Y) < b, 1.0, 0.0)


def test_beta_plane_band_known_answer(oracle_mod):
    """A band of uniform vorticity |y| < b on the periodic strip is a pair of vortex sheets:
    u = -zeta y inside, -+zeta b outside, v = 0 (the x-integral of the periodic kernel is
    1/sinh|2 pi dy|, and a midpoint grid sums it exactly)."""
    X, Y, A, Z = _band()
    u, v = oracle_mod.beta_plane_velocity(X, Y, Z, A, np.ones(X.size, dtype=np.int32))
    inside, outside = np.abs(Y) < 0.2, np.abs(Y) > 0.3
    assert np.abs(u + Y)[inside].max() < 1e-11
    assert np.abs(np.abs(u) - 0.25)[outside].max() < 1e-11
    assert np.abs(v).max() < 1e-12


def test_beta_plane_stream_vs_numpy(oracle_mod):
    rng = np.random.default_rng(8)
    n = 300
    x, y = rng.random(n), rng.uniform(-0.5, 0.5, n)
    a = rng.uniform(0.5, 1.5, n) / n
    zr, za = rng.standard_normal(n), rng.standard_normal(n)
    act = (rng.random(n) < 0.8).astype(np.int32)
    pr, pa = oracle_mod.beta_plane_stream(x, y, zr, za, a, act)
    j = act == 1
    for i in (0, 17, 299):
        m = j & (np.arange(n) != i)
        g = np.log(np.cosh(2 * np.pi * (y[i] - y[m])) - np.cos(2 * np.pi * (x[i] - x[m]))) / (4 * np.pi)
        assert abs(pr[i] - (g * zr[m] * a[m]).sum()) <= 1e-12 * np.abs(g * zr[m] * a[m]).sum()
        assert abs(pa[i] - (g * za[m] * a[m]).sum()) <= 1e-12 * np.abs(g * za[m] * a[m]).sum()


def _beta_groups(rng, n_groups=6, per=64):
    """Compact groups of sources on the strip, each with its centroid z_o and radius R."""
    groups = []
    for _ in range(n_groups):
        c = np.array([rng.random(), rng.uniform(-0.5, 0.5)])
        pts = c + rng.normal(0.0, 0.01, (per, 2))
        groups.append(pts)
    return groups


def test_beta_complex_far_form_identity(oracle_mod):
    """The beta-plane FP32C far form, in FP64 numpy: with e = exp(2 pi i (z - z_o)) about a
    group's centroid, the group's velocity at a far target is u = S_g + 2 Re G, v = -2 Im G,
    G = sum_j S_j e_j / (e_i - e_j); it equals the reference sum (the oracle) to rounding,
    for targets beyond 4R of the group in the periodic distance, across x = 0 / 1 too."""
    rng = np.random.default_rng(31)
    groups = _beta_groups(rng)
    tx, ty = rng.random(300), rng.uniform(-1.5, 1.5, 300)
    for pts in groups:
        ns = len(pts)
        zeta = rng.uniform(-1.0, 1.0, ns)
        area = rng.uniform(0.5, 1.5, ns) * 1e-4
        x = np.concatenate([pts[:, 0], tx])
        y = np.concatenate([pts[:, 1], ty])
        zz = np.concatenate([zeta, np.zeros(tx.size)])
        aa = np.concatenate([area, np.zeros(tx.size)])
        act = np.concatenate([np.ones(ns), np.zeros(tx.size)]).astype(np.int32)
        ru, rv = oracle_mod.beta_plane_velocity(x, y, zz, aa, act, ns, ns + tx.size)
        zo = pts.mean(0)
        R = np.sqrt(((pts - zo) ** 2).sum(1)).max()
        S = 0.5 * zeta * area
        ej = np.exp(2j * np.pi * ((pts[:, 0] - zo[0]) + 1j * (pts[:, 1] - zo[1])))
        dx = tx - zo[0]
        dx -= np.rint(dx)
        far = dx * dx + (ty - zo[1]) ** 2 > (4.0 * R) ** 2  # the kernels' near limit, 4R
        ei = np.exp(2j * np.pi * (dx + 1j * (ty - zo[1])))
        G = (S[None, :] * ej[None, :] / (ei[:, None] - ej[None, :])).sum(1)
        u = S.sum() + 2.0 * G.real
        v = -2.0 * G.imag
        scale = max(np.abs(ru).max(), np.abs(rv).max())
        assert far.sum() > 200
        assert np.abs(u - ru)[far].max() <= 1e-12 * scale and np.abs(v - rv)[far].max() <= 1e-12 * scale


def test_beta_stream_far_form_identity(oracle_mod):
    """The beta-plane stream far form, in FP64 numpy: |e_i - e_j|^2 = 2 |e_i| |e_j| (cosh 2 pi dy -
    cos 2 pi dx) with ln|e| = -2 pi (y - y_o), so a group adds sum_j w_j ln|e_i - e_j|^2 +
    W 2 pi (y_i - y_o) + C, W = sum w_j, C = sum w_j (2 pi (y_j - y_o) - ln 2), w = q A / (4 pi);
    it equals the oracle's log(cosh - cos) / (4 pi) sum to rounding."""
    rng = np.random.default_rng(32)
    groups = _beta_groups(rng)
    tx, ty = rng.random(300), rng.uniform(-2.0, 2.0, 300)
    for pts in groups:
        ns = len(pts)
        q = rng.uniform(-1.0, 1.0, ns)
        area = rng.uniform(0.5, 1.5, ns) * 1e-4
        x = np.concatenate([pts[:, 0], tx])
        y = np.concatenate([pts[:, 1], ty])
        qq = np.concatenate([q, np.zeros(tx.size)])
        aa = np.concatenate([area, np.zeros(tx.size)])
        act = np.concatenate([np.ones(ns), np.zeros(tx.size)]).astype(np.int32)
        rr, _ = oracle_mod.beta_plane_stream(x, y, qq, qq, aa, act, ns, ns + tx.size)
        zo = pts.mean(0)
        w = q * area / (4.0 * np.pi)
        W = w.sum()
        C = (w * (2.0 * np.pi * (pts[:, 1] - zo[1]) - np.log(2.0))).sum()
        ej = np.exp(2j * np.pi * ((pts[:, 0] - zo[0]) + 1j * (pts[:, 1] - zo[1])))
        ei = np.exp(2j * np.pi * ((tx - zo[0]) + 1j * (ty - zo[1])))
        lg = np.log(np.abs(ei[:, None] - ej[None, :]) ** 2)
        psi = (w[None, :] * lg).sum(1) + W * 2.0 * np.pi * (ty - zo[1]) + C
        assert np.abs(psi - rr).max() <= 1e-12 * np.abs(rr).max()
