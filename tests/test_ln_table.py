"""The FP32 log of the stream-function sweeps (ln_q2_shift, csrc/stream_rel.cuh) on the CPU:
the committed table is what its generator writes, and a float32 emulation of the device
sequence (FMA emulated exactly: float32 products are exact in float64) stays within about an
ulp of ln q over the whole positive normal range."""
import importlib.util
import io
import re
from contextlib import redirect_stdout
from pathlib import Path

import numpy as np
import pytest

CSRC = Path(__file__).resolve().parents[1] / "lpm-v2_gb300" / "csrc"
f32 = np.float32


def _table():
    text = (CSRC / "ln_table.cuh").read_text()
    arrs = re.findall(r"__constant__ float (\w+)\[32\] = \{(.*?)\};", text, re.S)
    out = {}
    for name, body in arrs:
        vals = [float.fromhex(v.strip().rstrip("f")) for v in body.split(",") if v.strip()]
        out[name] = np.array(vals, dtype=np.float32)
    return out["kLnTabInv"], out["kLnTabLog"]


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def ln_q_emulated(q, s=0):
    """ln q - s ln 2 as the device computes it, lane by lane."""
    inv_t, log_t = _table()
    b = q.astype(np.float32).view(np.int32)
    t = (b.astype(np.int64) - 0x3F3504F3).astype(np.int32)
    k = t >> 23
    mb = (b.astype(np.int64) - (k.astype(np.int64) << 23)).astype(np.int32)
    key = (mb >> 19) & 31
    m = mb.view(np.float32)
    kf = ((k + 0x4B400000).astype(np.int32).view(np.float32).astype(np.float64) + (-12582912.0 - s)).astype(np.float32)
    r = _fma(m, inv_t[key], np.full_like(m, -1.0))
    p = _fma(np.full_like(r, 0.2), r, np.full_like(r, -0.25))
    p = _fma(p, r, np.full_like(r, f32(0.33333334)))
    p = _fma(p, r, np.full_like(r, -0.5))
    bb = _fma((r.astype(np.float64) * r).astype(np.float32), p, r)
    a = _fma(kf, np.full_like(kf, f32(0.69314718)), log_t[key])
    return (a.astype(np.float64) + bb.astype(np.float64)).astype(np.float32)


def test_table_is_the_generators_output():
    pytest.importorskip("mpmath")
    spec = importlib.util.spec_from_file_location("gen_ln_table", CSRC / "gen_ln_table.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    with redirect_stdout(buf):
        gen.main()
    assert buf.getvalue() == (CSRC / "ln_table.cuh").read_text()


def test_table_entries_are_accurate():
    """ln c is the stored float to far below an ulp (accurate tables), |m/c - 1| <= 0.0306."""
    inv_t, log_t = _table()
    lnc = -np.log(inv_t.astype(np.float64))
    assert np.all(np.abs(lnc - log_t) <= 1e-3 * np.spacing(np.abs(log_t)))
    for key in range(6, 23):
        lo, hi = (0.5 + key / 32, 0.5 + (key + 1) / 32) if key < 16 else (1 + (key - 16) / 16, 1 + (key - 15) / 16)
        lo, hi = max(lo, 2 ** -0.5), min(hi, 2 ** 0.5)
        assert max(abs(lo * inv_t[key] - 1), abs(hi * inv_t[key] - 1)) <= 0.0306


def test_log_emulation_error():
    """Over the positive normal floats (log-uniform) and densely around 1: the error is at
    most 1.5 ulp of max(|ln q|, 1/2) -- the k ln 2 rounding and the table part -- and at most
    2.5e-9 absolute for q within 3 % of 1, where ln q itself is small (2.0e-9 measured)."""
    rng = np.random.default_rng(5)
    q = np.exp(rng.uniform(-87.0, 88.0, 400_000)).astype(np.float32)
    near = (1.0 + rng.uniform(-0.03, 0.03, 400_000)).astype(np.float32)
    for arr, absbound in ((q, None), (near, 2.5e-9)):
        got = ln_q_emulated(arr).astype(np.float64)
        ref = np.log(arr.astype(np.float64))
        err = np.abs(got - ref)
        scale = np.maximum(np.abs(ref), 0.5)
        assert np.all(err <= 1.5 * 2.0 ** -23 * scale)
        if absbound is not None:
            assert err.max() <= absbound


def test_log_shift_is_exact():
    """ln_q2_shift(q, shift_bias(s)) = ln q - s ln 2 with the shift in the exponent."""
    rng = np.random.default_rng(6)
    q = np.exp(rng.uniform(-20.0, 20.0, 10_000)).astype(np.float32)
    for s in (-3, -1, 1, 7):
        got = ln_q_emulated(q, s).astype(np.float64)
        ref = np.log(q.astype(np.float64)) - s * np.log(2.0)
        assert np.all(np.abs(got - ref) <= 1.5 * 2.0 ** -23 * np.maximum(np.abs(ref), 0.5))
