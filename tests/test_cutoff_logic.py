"""The FP64 PSE sweeps' tile cutoff (seq_fp64_kernel with tile_bounds64_kernel) restated in
numpy: a warp skips a 64-source tile when every target is farther than the tile's radius plus
the reach from its centre, in unit directions (reach 7 eps / radius, great-circle kernels) or
raw positions (reach 7 eps).  Every pair of a skipped tile must then have r = distance / eps
>= 7 -- the great-circle distance is never shorter than the chord of the unit directions --
so each kernel (a polynomial times exp(-r^2)) is below 1e-14 of its peak there."""
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
