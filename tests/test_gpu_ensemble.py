"""GPU tests of the batched ensemble (one persistent launch per RK4 stage for all instances)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def wl(built_lib):
    import workloads
    return workloads


@pytest.fixture(scope="module")
def instances(wl):
    return wl.config_ensemble(n_instances=7, seed=5, nests=(2, 3, 4))


def _split(st, sizes):
    offs = np.concatenate([[0], np.cumsum(sizes)])
    return [{k: v[offs[i]:offs[i + 1]] for k, v in st.items()} for i in range(len(sizes))]


def test_ensemble_fp64_bit_exact_vs_single_solvers(lg, instances):
    ens = lg.Ensemble(instances, mode="fp64")
    ens.timestep(0.01, 5)
    parts = _split(ens.get_state(), ens.sizes)
    for d, got in zip(instances, parts):
        s = lg.BVESolver(d["x"], d["y"], d["z"], d["rel_vort"], d["area"], d["active"], d["radius"],
                         d["rotation_rate"], mode="fp64")
        s.timestep(0.01, 5)
        ref = s.get_state()
        for k in ("x", "y", "z", "rel_vort", "u", "v", "w"):
            assert np.array_equal(got[k], ref[k]), k
        s.close()
    ens.close()


def test_ensemble_fp32c_velocity_vs_fp64(lg, instances):
    ens = lg.Ensemble(instances, mode="fp32c")
    parts = _split(ens.get_state(), ens.sizes)
    for d, got in zip(instances, parts):
        ref = lg.set_velocity_from_vorticity(d["x"], d["y"], d["z"], d["rel_vort"], d["area"], d["active"],
                                             d["radius"])
        err = np.abs(np.stack([got["u"], got["v"], got["w"]]) - np.stack(ref)).max() / np.abs(np.stack(ref)).max()
        assert err <= 1e-6
    ens.close()


def test_ensemble_fp32c_steps_track_fp64(lg, instances):
    e32 = lg.Ensemble(instances, mode="fp32c")
    e64 = lg.Ensemble(instances, mode="fp64")
    e32.timestep(0.01, 5)
    e64.timestep(0.01, 5)
    a, b = e32.get_state(), e64.get_state()
    # 5 steps of dt = 0.01 with velocity errors ~1e-7 relative: positions agree to ~1e-8
    assert np.abs(np.stack([a["x"] - b["x"], a["y"] - b["y"], a["z"] - b["z"]])).max() < 1e-7
    vel = np.stack([a["u"] - b["u"], a["v"] - b["v"], a["w"] - b["w"]])
    assert np.abs(vel).max() / np.abs(np.stack([b["u"], b["v"], b["w"]])).max() < 2e-6
    ms, launches = e32.kernel_timing()
    # per step: 4 stage kernels and 4 sums of (curve keys, radix sort, prep, sweep, finish)
    per_step, rem = divmod(launches, 5)
    assert ms > 0 and rem == 0 and per_step >= 4 + 4 * 5 and (per_step - 4) % 4 == 0
    e32.close()
    e64.close()


def test_ensemble_renormalize(lg, instances):
    ens = lg.Ensemble(instances, mode="fp32c")
    ens.timestep(0.01, 3, renormalize=True)
    st = ens.get_state()
    r = np.sqrt(st["x"] ** 2 + st["y"] ** 2 + st["z"] ** 2)
    assert np.abs(r - 1.0).max() < 1e-14
    ens.close()


def test_ensemble_bad_arguments(lg, instances):
    bad = [dict(instances[0])]
    bad[0]["radius"] = -1.0
    with pytest.raises(lg.LpmError):
        lg.Ensemble(bad)


def test_ensemble_mixed_radii_and_rotation(lg, wl):
    """Instances with different sphere radii (unit to Earth's) and rotation rates, and one with
    few active sources: FP64 bit-identical to single solvers, FP32C within 1e-6 of FP64."""
    base = wl.config_ensemble(n_instances=4, seed=9, nests=(2, 3))
    radii = [1.0, 6.37122e6, 0.25, 1.0e3]
    insts = []
    for d, a in zip(base, radii):
        e = dict(d)
        e["x"], e["y"], e["z"] = d["x"] * a, d["y"] * a, d["z"] * a
        e["area"] = d["area"] * a * a
        e["radius"] = a
        e["rotation_rate"] = 2.0 * np.pi / (a if a > 10 else 1.0)
        insts.append(e)
    act = insts[2]["active"].copy()
    act[np.nonzero(act)[0][3:]] = 0  # 3 active sources only
    insts[2]["active"] = act
    e64 = lg.Ensemble(insts, mode="fp64")
    e32 = lg.Ensemble(insts, mode="fp32c")
    e64.timestep(0.01, 3)
    e32.timestep(0.01, 3)
    p64, p32 = _split(e64.get_state(), e64.sizes), _split(e32.get_state(), e32.sizes)
    for d, g64, g32 in zip(insts, p64, p32):
        s = lg.BVESolver(d["x"], d["y"], d["z"], d["rel_vort"], d["area"], d["active"], d["radius"],
                         d["rotation_rate"], mode="fp64")
        s.timestep(0.01, 3)
        ref = s.get_state()
        for k in ("x", "y", "z", "rel_vort", "u", "v", "w"):
            assert np.array_equal(g64[k], ref[k]), k
        s.close()
        u64 = np.stack([g64["u"], g64["v"], g64["w"]])
        u32 = np.stack([g32["u"], g32["v"], g32["w"]])
        assert np.abs(u32 - u64).max() <= 1e-6 * np.abs(u64).max()
    e64.close()
    e32.close()


@pytest.mark.parametrize("tpt", [4, 8])
@pytest.mark.parametrize("per_slot", [4, 8, 16])
def test_ensemble_every_sweep_shape(lg, instances, tpt, per_slot):
    """Each of the persistent sweep's six configurations (the autotuner's choices), selected
    by hand: the velocity of every instance within 1e-6 of its FP64 sum, before and after two
    RK4 steps (the step graph is captured again for the selected shape)."""
    ens = lg.Ensemble(instances, mode="fp32c")
    ens.select_sweep(128, tpt, per_slot)
    assert ens.sweep_shape() == (128, tpt, 4 if tpt == 4 else 2, per_slot)
    ens.velocity()
    for steps in (0, 2):
        if steps:
            ens.timestep(0.01, steps)
        parts = _split(ens.get_state(), ens.sizes)
        for d, got in zip(instances, parts):
            ref = lg.bve_sphere_velocity(got["x"], got["y"], got["z"], got["rel_vort"], d["area"], d["active"],
                                         d["radius"], mode="fp64")
            err = np.abs(np.stack([got["u"], got["v"], got["w"]]) - np.stack(ref)).max() / np.abs(np.stack(ref)).max()
            assert err <= 1e-6
    with pytest.raises(lg.LpmError):
        ens.select_sweep(256, 4, 8)
    ens.close()
