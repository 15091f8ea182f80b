"""Prints the table of the float-float exponential in refmath.hpp: 2^(j/64)
for j = 0..63 as (hi, lo) float pairs, hi the float nearest to 2^(j/64) and
lo the float nearest to the remainder, so that hi + lo is within 2^-48 of
the exact value.  The same rows are the device table FF_EXP2_TAB_D and the
host table FF_EXP2_TAB_H.  Needs mpmath (bundled with sympy); the output is
pasted into refmath.hpp, so the build itself does not run this, and
tests/test_refmath_host.py checks that the header holds exactly these rows."""
import struct

import mpmath

mpmath.mp.prec = 200


def f32(v):
    """round-to-nearest float32 of an mpmath value (via double: exact for these magnitudes)"""
    return struct.unpack("<f", struct.pack("<f", float(mpmath.mpf(v))))[0]


def rows():
    out = []
    for j in range(64):
        v = mpmath.power(2, mpmath.mpf(j) / 64)
        hi = f32(v)
        lo = f32(v - mpmath.mpf(hi))
        out.append((hi, lo))
    return out


def main():
    for hi, lo in rows():
        print(f"\t{{ {float(hi).hex()}f, {float(lo).hex()}f }},")


if __name__ == "__main__":
    main()
