#!/usr/bin/env python3
"""Writes kz_srgb_table.h: the exact sRGB encode and decode tables of the 8-bit sRGB colour formats.

Encode (linear float -> 8-bit sRGB code), the sRGB transfer function of the Vulkan specification's colour
space conversions: s = 12.92 L for L <= 0.0031308, else 1.055 L^(1/2.4) - 0.055, and the code is s * 255
rounded to the nearest integer.  As a function of a float32 input it is a step function; the table holds
its 255 steps: threshold k (k = 1..255) is the smallest float32 L with 255 s(L) >= k - 1/2, so
code(L) = the number of thresholds <= L, for 0 < L < 1 (0 for L <= 0 or NaN, 255 for L >= 1).  No float32
lies exactly on a half-integer step (the linear segment's ties are not dyadic, the power segment's values
are irrational), so the rounding direction of ties never matters.

Decode (8-bit sRGB code -> linear float): c = k / 255; L = c / 12.92 for c <= 0.04045, else
((c + 0.055) / 1.055)^2.4, rounded to the nearest float32.

Both are evaluated in 60-digit decimal arithmetic and rounded exactly, so the table does not depend on the
host's libm.  Run from this directory: python gen_srgb_table.py
"""
import os
import struct
from decimal import Decimal, getcontext
from fractions import Fraction

getcontext().prec = 60
D = Decimal


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def bits_f32(b):
    return struct.unpack("<f", struct.pack("<I", b))[0]


def srgb_encode_exact(L):
    """255 s(L) for a float32 value L in [0, 1], as a Decimal"""
    L = D(Fraction(L).numerator) / D(Fraction(L).denominator)
    if L <= D("0.0031308"):
        s = D("12.92") * L
    else:
        s = D("1.055") * (L ** (D(1) / D("2.4"))) - D("0.055")
    return s * 255


def nearest_f32(q):
    """the float32 nearest to the rational q (ties to even)"""
    c = float(q)
    b = f32_bits(c)
    cands = [bits_f32(b), bits_f32(b + 1), bits_f32(b - 1) if b > 0 else bits_f32(b)]
    return min(cands, key=lambda v: (abs(Fraction(v) - q), f32_bits(v) & 1))


def thresholds():
    one = f32_bits(1.0)
    out = []
    for k in range(1, 256):
        target = D(k) - D("0.5")
        lo, hi = 0, one  # bit patterns of non-negative floats order like the floats
        while lo < hi:  # smallest pattern with 255 s >= target
            mid = (lo + hi) // 2
            if srgb_encode_exact(bits_f32(mid)) >= target:
                hi = mid
            else:
                lo = mid + 1
        out.append(bits_f32(lo))
    return out


def decode():
    out = []
    for k in range(256):
        c = D(k) / D(255)
        if c <= D("0.04045"):
            L = c / D("12.92")
        else:
            L = ((c + D("0.055")) / D("1.055")) ** D("2.4")
        out.append(nearest_f32(Fraction(L)))
    return out


def fmt(v):
    return "%sf" % float(v).hex() if v != 0.0 else "0.0f"


def main():
    thr, dec = thresholds(), decode()
    lines = ["/* kz_srgb_table.h - generated by gen_srgb_table.py (exact sRGB encode steps and decode values of the",
             " * 8-bit sRGB colour formats); do not edit. */",
             "#ifndef KZ_SRGB_TABLE_H", "#define KZ_SRGB_TABLE_H", "",
             "/* threshold k - 1 (k = 1..255): the smallest float L whose 8-bit sRGB code is k */",
             "#define KZ_SRGB_THRESHOLDS \\", "  { \\"]
    for i in range(0, 255, 6):
        lines.append("    " + ", ".join(fmt(v) for v in thr[i:i + 6]) + ("," if i + 6 < 255 else "") + " \\")
    lines += ["  }", "", "/* value k (k = 0..255): the linear float of 8-bit sRGB code k */",
              "#define KZ_SRGB_DECODE \\", "  { \\"]
    for i in range(0, 256, 6):
        lines.append("    " + ", ".join(fmt(v) for v in dec[i:i + 6]) + ("," if i + 6 < 256 else "") + " \\")
    lines += ["  }", "", "#endif", ""]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kz_srgb_table.h")
    with open(path, "w") as f:
        f.write("\n".join(lines))
    print("wrote", path)


if __name__ == "__main__":
    main()
