"""The FP32C PSE sweeps' tile culling (cta_target_ball and cull_tiles in csrc/engine.cuh, with
the tests of pse_rel_sweep_kernel and plane_pse_rel_sweep_kernel) restated in numpy float32.

A CTA takes the ball around its targets' hi parts (centroid, largest distance) and leaves out a
group (centroid o, radius R) when |c - o| >= (R_ball + R + c_cut) (1 + 1e-4) + 1e-5 (1 + |c|_1).
The culling must be conservative against the warps' own test, which skips a group when every
target of the warp has |t - o| >= R + c_cut: then the sums are the same with and without it.
Here every target of a CTA that culls a group must be at least R + c_cut from its centroid,
with room for the float rounding of the warps' test.  The CTAs of a block then split its
in-reach tiles round robin (cull_window's pick, restated at the end): each tile goes to one CTA.
"""
import numpy as np

GROUP = 32  # PseRel::kGroup, PlanePseRel::kGroup
CTA_TARGETS = 512


def _f32(a):
    return np.asarray(a, dtype=np.float32)


def _groups(S):
    """Group centroids (FP64, stored as float hi parts) and radii (FP64 max distance, as float)."""
    out = []
    for g in range(0, len(S), GROUP):
        Q = S[g:g + GROUP]
        o = Q.mean(0)
        out.append((_f32(o), np.float32(np.sqrt(((Q - o) ** 2).sum(1)).max())))
    return out


def _ball(T):
    """cta_target_ball in float32: the mean of the hi parts, then the largest distance."""
    h = _f32(T)
    c = h.sum(0, dtype=np.float32) * np.float32(1.0 / len(h))
    d2 = ((h - c) ** 2).sum(1, dtype=np.float32)
    return c.astype(np.float32), np.float32(np.sqrt(d2.max()))


def _culled(c, rb, o, R, c_cut):
    lim = np.float32((rb + R + np.float32(c_cut)) * np.float32(1.0001)) + \
        np.float32(1e-5) * (np.float32(1) + np.abs(c).sum(dtype=np.float32))
    d = (o - c).astype(np.float32)
    return (d * d).sum(dtype=np.float32) >= lim * lim


def _check(S, T, c_cut):
    groups = _groups(S)
    culled = 0
    for b in range(0, len(T), CTA_TARGETS):
        Tb = T[b:b + CTA_TARGETS]
        c, rb = _ball(Tb)
        for o, R in groups:
            if not _culled(c, rb, o, R, c_cut):
                continue
            culled += 1
            # every target of the CTA is out of the group's reach, with margin for the warps'
            # float test (relative rounding well below 1e-6)
            dist = np.sqrt(((Tb - o.astype(np.float64)) ** 2).sum(1))
            assert dist.min() >= (float(R) + c_cut) * (1 + 1e-6)
    return culled


def _curve_order(P):
    """Spatial locality, as the Hilbert sort gives the kernels (a coarse grid order will do)."""
    q = np.floor((P + 8.0) * 4.0).astype(np.int64)
    return np.lexsort((q[:, 0], q[:, 1], q[:, 2]))


def test_sphere_culling_is_conservative():
    rng = np.random.default_rng(21)
    S = rng.normal(size=(16384, 3))
    S /= np.linalg.norm(S, axis=1)[:, None]
    S = S[_curve_order(S * 4.0)]
    T = rng.normal(size=(8192, 3))
    T /= np.linalg.norm(T, axis=1)[:, None]
    T = T[_curve_order(T * 4.0)]
    for eps in (0.01, 0.037, 0.1):
        assert _check(S, T, 7.0 * eps) > 0


def test_plane_culling_is_conservative():
    rng = np.random.default_rng(22)
    S = np.stack([rng.uniform(-4, 4, 16384), rng.uniform(-4, 4, 16384), np.zeros(16384)], 1)
    S = S[_curve_order(S)]
    T = np.stack([rng.uniform(-4, 4, 8192), rng.uniform(-4, 4, 8192), np.zeros(8192)], 1)
    T = T[_curve_order(T)]
    for eps in (0.02, 0.1):
        assert _check(S, T, 7.0 * eps) > 0


def test_plane_culling_far_from_the_origin():
    """Coordinates of size 1e4: the 1e-5 |c| widening covers the float rounding of |c - o|."""
    rng = np.random.default_rng(23)
    S = np.stack([1e4 + rng.uniform(-4, 4, 8192), -2e4 + rng.uniform(-4, 4, 8192), np.zeros(8192)], 1)
    S = S[_curve_order(S - S.mean(0))]
    T = np.stack([1e4 + rng.uniform(-4, 4, 4096), -2e4 + rng.uniform(-4, 4, 4096), np.zeros(4096)], 1)
    T = T[_curve_order(T - T.mean(0))]
    assert _check(S, T, 7.0 * 0.05) > 0


def test_nan_target_culls_nothing():
    S = np.random.default_rng(24).normal(size=(1024, 3))
    T = S[:CTA_TARGETS].copy()
    T[5, 1] = np.nan
    c, rb = _ball(T)
    assert not any(_culled(c, rb, o, R, 0.1) for o, R in _groups(S))


def _share_listing(rank0, total, shares, share):
    """cull_window's pick for one window, restated: the kept count and each kept rank's place."""
    first = rank0 + ((share - rank0 % shares) % shares + shares) % shares
    end = rank0 + total
    kept = (end - 1 - first) // shares + 1 if end > first else 0
    places = {r: (r - first) // shares for r in range(rank0, end) if r % shares == share}
    return kept, places


def test_round_robin_shares_list_every_tile_once():
    """Every in-reach tile of a block goes to exactly one of its CTAs, each CTA's list is dense
    (places 0..kept-1 in rank order) and the shares' counts differ by at most one."""
    rng = np.random.default_rng(25)
    for _ in range(200):
        shares = int(rng.integers(1, 33))
        windows = [int(rng.integers(0, 129)) for _ in range(int(rng.integers(1, 6)))]
        owner = {}
        counts = [0] * shares
        for share in range(shares):
            rank0 = 0
            for total in windows:
                kept, places = _share_listing(rank0, total, shares, share)
                assert sorted(places.values()) == list(range(kept))
                for r in places:
                    assert r not in owner
                    owner[r] = share
                counts[share] += kept
                rank0 += total
        assert sorted(owner) == list(range(sum(windows)))
        assert max(counts) - min(counts) <= 1
