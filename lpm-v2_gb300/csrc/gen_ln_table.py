"""Writes ln_table.cuh: the 32-entry table of the FP32 natural log used by the stream-function
sweeps (ln_q2_shift in stream_rel.cuh).

A positive float q is split as q = 2^k m with m in [sqrt(1/2), sqrt(2)).  Bits 19..23 of m (the
exponent's lowest bit and the top four mantissa bits) select an entry (inv, lnc):
- keys 0..15 cover m in [1/2 + t/32, 1/2 + (t+1)/32), t = key;
- keys 16..31 cover m in [1 + t/16, 1 + (t+1)/16), t = key - 16.
Then ln m = lnc + ln(1 + r) with r = m inv - 1, |r| <= 0.032, and a degree-5 series.

inv is the float nearest 1/c (c = the interval's midpoint), moved by up to 4096 ulps so that
lnc = -ln(inv) lies within a few 1e-5 ulp of a float.  This is Gal's accurate-tables method
(S. Gal, "Computing elementary functions: a new approach for achieving high accuracy and good
performance", 1986).  The stored lnc then carries no rounding of its own, and no key adds a
systematic error to the sums.  ln(inv) is evaluated in 60-digit arithmetic (mpmath).

Usage: python gen_ln_table.py > ln_table.cuh
"""
import mpmath
import numpy as np

mpmath.mp.dps = 60
SEARCH = 4096


def entry(key):
    if key < 16:
        lo = 0.5 + key / 32.0
        hi = lo + 1.0 / 32.0
    else:
        lo = 1.0 + (key - 16) / 16.0
        hi = lo + 1.0 / 16.0
    c = 0.5 * (lo + hi)
    inv0 = np.float32(1.0 / c)
    best = None
    up = inv0
    down = inv0
    cands = [inv0]
    for _ in range(SEARCH):
        up = np.nextafter(up, np.float32(np.inf), dtype=np.float32)
        down = np.nextafter(down, np.float32(0), dtype=np.float32)
        cands += [up, down]
    for inv in cands:
        lnc = -mpmath.log(mpmath.mpf(float(inv)))
        lf = np.float32(float(lnc))
        ulp = float(np.spacing(np.abs(lf))) if lf != 0 else 2.0 ** -149
        err = abs(float(lnc - mpmath.mpf(float(lf)))) / ulp
        if best is None or err < best[0]:
            best = (err, inv, lf)
    err, inv, lf = best
    rmax = max(abs(lo * float(inv) - 1.0), abs(hi * float(inv) - 1.0))
    return inv, lf, err, rmax


def main():
    rows = [entry(k) for k in range(32)]
    worst = max(r[2] for r in rows)
    rmax = max(r[3] for r in rows)
    print("// ln_table.cuh -- generated by gen_ln_table.py (do not edit): the (1/c, ln c) table of")
    print("// ln_q2_shift.  Keys are bits 19..23 of m, q = 2^k m, m in [sqrt(1/2), sqrt(2)).  ln c is")
    print(f"// within {worst:.1e} ulp of the stored float (accurate tables); |m/c - 1| <= {rmax:.4f}.")
    print("#pragma once")
    print()
    print("namespace lpm {")
    print()
    print("__constant__ float kLnTabInv[32] = {")
    for k in range(0, 32, 4):
        print("    " + ", ".join(f"{float(rows[j][0]).hex()}f" for j in range(k, k + 4)) + ",")
    print("};")
    print("__constant__ float kLnTabLog[32] = {")
    for k in range(0, 32, 4):
        print("    " + ", ".join(f"{float(rows[j][1]).hex()}f" for j in range(k, k + 4)) + ",")
    print("};")
    print()
    print("}  // namespace lpm")


if __name__ == "__main__":
    main()
