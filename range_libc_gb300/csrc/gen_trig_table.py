"""Writes rlc_trig_table.h: the constants of the correctly rounded float sine/cosine
(rlc_trig.cuh), computed to 60 significant digits with mpmath.

  * pi/2 as a sum of four floats C0 + C1 + C2 + C3, each the float nearest to what the
    previous ones leave, for the argument reduction x - j * pi/2;
  * sin(k/256) and cos(k/256), k = 0 .. 203, each as a float pair hi + lo (hi the nearest
    float to the value, lo the nearest float to the remainder): about 48 correct bits.

    python range_libc_gb300/csrc/gen_trig_table.py
"""
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 60
KMAX = 203


def f32(v) -> np.float32:
    """The float nearest to the mpmath value v (via double, exact for the pairs used here:
    a 53-bit rounding followed by a 24-bit one is checked against the direct rounding)."""
    d = float(v)
    f = np.float32(d)
    # double rounding check: the exact value must round to the same float
    lo = mp.mpf(float(np.nextafter(f, np.float32(-np.inf))))
    hi = mp.mpf(float(np.nextafter(f, np.float32(np.inf))))
    fv = mp.mpf(float(f))
    assert abs(v - fv) <= abs(v - lo) and abs(v - fv) <= abs(v - hi)
    return f


def hexf(f: np.float32) -> str:
    """C hexadecimal float literal of f (its 24-bit significand needs 6 hex digits)."""
    if f == 0:
        return "0.0f"
    mant, exp = float(f).hex().split("p")
    head, frac = mant.split(".")
    return "%s.%sp%sf" % (head, frac[:6], exp)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    half_pi = mp.pi / 2
    parts, rem = [], half_pi
    for _ in range(4):
        p = f32(rem)
        parts.append(p)
        rem = rem - mp.mpf(float(p))
    two_over_pi = f32(2 / mp.pi)
    rows = []
    for k in range(KMAX + 1):
        s, c = mp.sin(mp.mpf(k) / 256), mp.cos(mp.mpf(k) / 256)
        sh = f32(s)
        sl = f32(s - mp.mpf(float(sh)))
        ch = f32(c)
        cl = f32(c - mp.mpf(float(ch)))
        rows.append((sh, sl, ch, cl))
    with open(os.path.join(here, "rlc_trig_table.h"), "w") as fh:
        fh.write("// Generated by gen_trig_table.py (mpmath, 60 digits); do not edit.\n")
        fh.write("// pi/2 = C0 + C1 + C2 + C3 (each the float nearest to the remainder), 2/pi rounded,\n")
        fh.write("// and sin(k/256), cos(k/256) for k = 0 .. %d as float pairs (hi, lo).\n" % KMAX)
        fh.write("#pragma once\n")
        for i, p in enumerate(parts):
            fh.write("#define RLC_TRIG_C%d %s\n" % (i, hexf(p)))
        fh.write("#define RLC_TRIG_TWO_OVER_PI %s\n" % hexf(two_over_pi))
        fh.write("#define RLC_TRIG_KMAX %d\n" % KMAX)
        fh.write("#define RLC_TRIG_TABLE_ROWS \\\n")
        for i, (sh, sl, ch, cl) in enumerate(rows):
            end = ", \\\n" if i < KMAX else "\n"
            fh.write("    {%s, %s, %s, %s}%s" % (hexf(sh), hexf(sl), hexf(ch), hexf(cl), end))


if __name__ == "__main__":
    main()
