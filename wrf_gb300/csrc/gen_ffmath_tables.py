#!/usr/bin/env python3
"""Writes ffmath_tables.h: the tables of the table-driven float-float log and
exp in ffmath.h, computed here with 50-digit decimal arithmetic.

log table (128 entries, index j = top 7 mantissa bits of m in [1, 2)):
  rc[j]  a float close to 1 / c_j, c_j = 1 + (j + 1/2) / 128 (the bucket
         centre); bucket 0 uses c = 1 and bucket 127 uses c = 2, so that
         arguments next to 1 reduce exactly (r = m - 1 or m/2 - 1);
  t[j]   -log(rc[j]) as a float pair (hi + lo), minus log 2 for j >= 64,
         where the caller adds one to the exponent (m in [1.5, 2) is taken as
         m/2 in [0.75, 1), which keeps arguments in [0.75, 1.5) free of any
         log 2 term).
exp table (64 entries): 2^(j/64) as a float pair.

Run from this directory: python gen_ffmath_tables.py > ffmath_tables.h
"""
import struct
from decimal import Decimal, getcontext

getcontext().prec = 50


def f32(x):
    """Nearest float32 (round to nearest even) of a Decimal / float."""
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def split(d):
    """Decimal -> (hi, lo) float32 pair, hi + lo within ~2^-48 relative of d."""
    hi = f32(d)
    lo = f32(d - Decimal(hi))
    return hi, lo


def ln(d):
    return Decimal(d).ln()


LN2 = ln(2)


def fmt(x):
    return "%.9ef" % x


def main():
    rows = []
    for j in range(128):
        if j == 0:
            c = Decimal(1)
        elif j == 127:
            c = Decimal(2)
        else:
            c = 1 + (Decimal(j) + Decimal("0.5")) / 128
        rc = f32(1 / c)
        t = -ln(Decimal(rc))
        if j >= 64:
            t -= LN2
        hi, lo = split(t)
        rows.append((rc, hi, lo))
    ex = [split(Decimal(2) ** (Decimal(j) / 64)) for j in range(64)]
    print("// Generated by gen_ffmath_tables.py (50-digit decimal arithmetic); do not edit.")
    print("#pragma once")
    print("namespace wrfgpu_ff {")
    print("// {rc, -log(rc) [- log 2] hi, lo, 0}: log reduction table, see ffmath.h")
    print("#define WRFGPU_FF_LOG_TAB \\")
    print("  {" + ", \\\n   ".join("{%s, %s, %s, 0.f}" % (fmt(rc), fmt(hi), fmt(lo)) for rc, hi, lo in rows) + "}")
    print("// {hi, lo} of 2^(j/64)")
    print("#define WRFGPU_FF_EXP_TAB \\")
    print("  {" + ", \\\n   ".join("{%s, %s}" % (fmt(hi), fmt(lo)) for hi, lo in ex) + "}")
    # ln2 / 64 in three parts: hi with 13 significant bits (N * hi exact for |N| < 2^11)
    l64 = LN2 / 64
    hi = f32(l64)
    b = struct.unpack("I", struct.pack("f", hi))[0] & 0xFFFFF800
    hi = struct.unpack("f", struct.pack("I", b))[0]
    mid = f32(l64 - Decimal(hi))
    lo = f32(l64 - Decimal(hi) - Decimal(mid))
    print("constexpr float LN2_64_HI = %s, LN2_64_MID = %s, LN2_64_LO = %s;" % (fmt(hi), fmt(mid), fmt(lo)))
    print("constexpr float INV_LN2_64 = %s;" % fmt(f32(64 / LN2)))
    th, tl = split(Decimal(1) / 3)
    print("constexpr float THIRD_HI = %s, THIRD_LO = %s;" % (fmt(th), fmt(tl)))
    lh, ll = split(LN2)
    print("constexpr float LN2F_HI = %s, LN2F_LO = %s;" % (fmt(lh), fmt(ll)))
    print("}  // namespace wrfgpu_ff")


if __name__ == "__main__":
    main()
