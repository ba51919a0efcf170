"""The FP64 PSE sweeps' tile cutoff (seq_fp64_kernel with tile_bounds64_kernel) restated in
numpy: a warp skips a 64-source tile when every target is farther than the tile's radius plus
the reach from its centre, in unit directions (reach 7 eps / radius, great-circle kernels) or
raw positions (reach 7 eps).  Every pair of a skipped tile must then have r = distance / eps
>= 7 -- the great-circle distance is never shorter than the chord of the unit directions --
so each kernel (a polynomial times exp(-r^2)) is below 1e-14 of its peak there.  Also the
FP32C sweeps' angle series for eps <= 0.06 a, up to and beyond the same cutoff."""
import numpy as np

TILE = 64


def _balls(P):
    out = []
    for t in range(0, len(P), TILE):
        Q = P[t:t + TILE]
        c = Q.mean(0)
        r = np.sqrt(((Q - c) ** 2).sum(1)).max()
        out.append((c, r * (1 + 1e-9) + 1e-9 * np.abs(c).sum()))
    return out


def test_sphere_cutoff_is_conservative():
    rng = np.random.default_rng(7)
    radius, eps = 6.37e6, 0.03 * 6.37e6
    S = rng.normal(size=(4096, 3))
    S /= np.linalg.norm(S, axis=1)[:, None]
    S = S[np.argsort(np.arctan2(S[:, 1], S[:, 0]) + 10 * np.round(S[:, 2] * 8))]  # some locality
    T = rng.normal(size=(512, 3))
    T /= np.linalg.norm(T, axis=1)[:, None]
    reach = 7 * eps / radius
    skipped = 0
    for t, (c, r) in enumerate(_balls(S)):
        far = np.sqrt(((T - c) ** 2).sum(1)) > r + reach
        if not far.any():
            continue
        Q = S[t * TILE:(t + 1) * TILE]
        ang = np.arctan2(np.linalg.norm(np.cross(T[far][:, None, :], Q[None, :, :]), axis=2),
                         (T[far][:, None, :] * Q[None, :, :]).sum(2))
        assert (ang * radius / eps).min() >= 7.0
        skipped += far.sum()
    assert skipped > 0


def test_plane_cutoff_is_conservative():
    rng = np.random.default_rng(8)
    eps = 0.1
    P = np.stack([rng.uniform(-4, 4, 4096), rng.uniform(-4, 4, 4096), np.zeros(4096)], 1)
    P = P[np.lexsort((P[:, 0], np.round(P[:, 1] * 2)))]
    T = np.stack([rng.uniform(-4, 4, 512), rng.uniform(-4, 4, 512), np.zeros(512)], 1)
    skipped = 0
    for t, (c, r) in enumerate(_balls(P)):
        far = np.sqrt(((T - c) ** 2).sum(1)) > r + 7 * eps
        if not far.any():
            continue
        Q = P[t * TILE:(t + 1) * TILE]
        d = np.sqrt(((T[far][:, None, :] - Q[None, :, :]) ** 2).sum(2))
        assert (d / eps).min() >= 7.0
        skipped += far.sum()
    assert skipped > 0


def test_fp32c_angle_series_up_to_the_cutoff():
    """The FP32C great-circle kernels take theta^2 = 4 asin^2(c/2) from the chord c by its
    series in v = c^2 (pse_r2 with kPseAngleSeries, coefficients 1, 1/12, 1/90, 1/560, 1/3150
    as the float constants the kernel holds) when eps <= 0.06 a.  Up to the cutoff r = 7 the
    truncation stays below 1e-8 relative, under an FP32 ulp.  The series grows with v, so a
    pair beyond the cutoff still has r^2 >= 49 (1 - 1e-8): its kernel stays negligible when a
    warp evaluates it anyway."""
    coef = np.array([3.1746032e-4, 1.7857143e-3, 1.1111111e-2, 8.3333336e-2, 1.0], dtype=np.float32).astype(np.float64)

    def theta2(v):
        return v * np.polyval(coef, v)

    for eps_a in (0.005, 0.02, 0.04, 0.06):
        v_cut = (2.0 * np.sin(3.5 * eps_a)) ** 2
        v = np.linspace(v_cut * 1e-6, v_cut, 20001)
        exact = 4.0 * np.arcsin(np.sqrt(v) / 2.0) ** 2
        assert np.abs(theta2(v) / exact - 1.0).max() <= 1e-8
        beyond = np.linspace(v_cut, 4.0, 20001)
        assert (theta2(beyond) / eps_a ** 2).min() >= 49.0 * (1.0 - 1e-8)
