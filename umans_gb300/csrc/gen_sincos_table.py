"""Prints the constants of the float-float sine/cosine in refmath.hpp:
sin(j/64) and cos(j/64) as (hi, lo) float pairs for j = 0..52, and pi/2 split
into four floats (the first with 17 significant bits, so that k * P1 is exact
for |k| < 2^7).  Needs mpmath (bundled with sympy); the output is pasted into
refmath.hpp, so the build itself does not run this."""
import struct

import mpmath

mpmath.mp.prec = 200


def f32(v):
    """round-to-nearest float32 of an mpmath value (via double: exact for these magnitudes)"""
    return struct.unpack("<f", struct.pack("<f", float(mpmath.mpf(v))))[0]


def round_bits(v, bits):
    m, e = mpmath.frexp(v)
    return mpmath.ldexp(mpmath.nint(mpmath.ldexp(m, bits)), e - bits)


def ff(v):
    h = f32(v)
    return h, f32(v - h)


def hexf(x):
    return float(x).hex().replace("0x1.", "0x1.") + "f" if x != 0 else "0.0f"


def main():
    half_pi = mpmath.pi / 2
    p1 = round_bits(half_pi, 17)
    rest = half_pi - p1
    p2 = f32(rest); rest -= p2
    p3 = f32(rest); rest -= p3
    p4 = f32(rest)
    print(f"// pi/2 = P1 + P2 + P3 + P4 (+ {float(rest - p4):.3g})")
    for name, v in (("P1", float(p1)), ("P2", p2), ("P3", p3), ("P4", p4)):
        print(f"constexpr float SC_{name} = {hexf(v)};")
    print(f"constexpr float SC_TWO_OVER_PI = {hexf(f32(2 / mpmath.pi))};")
    print("// { sin hi, sin lo, cos hi, cos lo } of j/64")
    for j in range(53):
        c = mpmath.mpf(j) / 64
        sh, sl = ff(mpmath.sin(c))
        ch, cl = ff(mpmath.cos(c))
        print(f"\t{{ {hexf(sh)}, {hexf(sl)}, {hexf(ch)}, {hexf(cl)} }},")


if __name__ == "__main__":
    main()
