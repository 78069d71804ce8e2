"""Generate fastmath_tables.h: the tables and split constants of the FP64
exp/exp10/log in fastmath.cuh, computed in 200-bit arithmetic with mpmath
and rounded to nearest.

    python dwarf-p-ice3_gb300/csrc/gen_fastmath_tables.py

exp (Tang, ACM TOMS 15(2), 1989): 2^(j/256), j = 0..255, as a double hi and
a float lo (the rounding error of hi, < 2^-53, needs only ~20 bits).

atan (table-driven reduction in the manner of Tang's methods): atan(j/64) and
pi/2 - atan(j/64), j = 0..64, as a double hi and a float lo.

log (Tang, ACM TOMS 16(4), 1990, with an exact reduction): the mantissa
z in [1, 2) is split into 128 intervals by its 7 leading fraction bits.
Intervals at or above sqrt(2) are folded (z/2, exponent + 1) so that results
near x = 1 never cancel against e*ln2.  For each interval c is its centre
(halved when folded) and invc a reciprocal of c rounded to 8 significant
bits, so that r = z*invc - 1 is exact in one FMA; the two intervals that
touch 1 use invc = 1 (log1p(r) alone, r exact).  The table stores
invc_tab = invc (halved for folded intervals, so r = fma(z, invc_tab, -1)
takes the unfolded z), -log(invc) of the unhalved reciprocal as a double hi
and a float lo, and the exponent increment of the fold.
"""
from __future__ import annotations

import os

import mpmath as mp
import numpy as np

mp.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))
FOLD = 53          # first interval [1 + 53/128, ...) at or above sqrt(2)


def dbl(x) -> float:
    return float(mp.mpf(x))          # round to nearest double


def flt(x) -> float:
    return float(np.float32(dbl(x)))  # nearest float (values here are far from float ties)


def round_bits(x, bits: int) -> float:
    """x rounded to `bits` significant bits (exactly representable)."""
    x = mp.mpf(x)
    e = int(mp.floor(mp.log(x, 2)))
    q = mp.mpf(2) ** (e - bits + 1)
    return float(mp.nint(x / q) * q)


def fhex(v: float) -> str:
    return f"{v.hex()}f" if v != 0.0 else "0.0f"


def main() -> None:
    lines = ["// Generated by gen_fastmath_tables.py (mpmath, 200-bit) - do not edit.",
             "#pragma once", "",
             "// 2^(j/256): {hi (double), lo (float)}, j = 0..255",
             "#define FM_EXP_TABLE_INIT { \\"]
    for j in range(256):
        v = mp.mpf(2) ** (mp.mpf(j) / 256)
        hi = dbl(v)
        lo = flt(v - mp.mpf(hi))
        lines.append(f"  {{{hi.hex()}, {fhex(lo)}, 0}}, \\")
    lines += ["}", "",
              "// per 7-bit mantissa interval: {invc_tab, -log(invc) hi, -log(invc) lo (float), fold}",
              "#define FM_LOG_TABLE_INIT { \\"]
    for i in range(128):
        centre = 1 + (mp.mpf(i) + mp.mpf(0.5)) / 128
        fold = i >= FOLD
        if fold:
            centre = centre / 2
        invc = 1.0 if i in (0, 127) else round_bits(1 / centre, 8)
        v = -mp.log(mp.mpf(invc))
        hi = dbl(v)
        lo = flt(v - mp.mpf(hi))
        invc_tab = invc / 2 if fold else invc
        lines.append(f"  {{{invc_tab.hex()}, {hi.hex()}, {fhex(lo)}, {1 if fold else 0}, 0.0}}, \\")
    lines += ["}", "",
              "// atan(j/64): {hi (double), lo (float)}, j = 0..64",
              "#define FM_ATAN_TABLE_INIT { \\"]
    for j in range(65):
        a = mp.atan(mp.mpf(j) / 64)
        ah = dbl(a)
        lines.append(f"  {{{ah.hex()}, {fhex(flt(a - mp.mpf(ah)))}, 0}}, \\")
    lines += ["}", "", "// pi/2 - atan(j/64): {hi (double), lo (float)}, j = 0..64",
              "#define FM_ATANC_TABLE_INIT { \\"]
    for j in range(65):
        b = mp.pi / 2 - mp.atan(mp.mpf(j) / 64)
        bh = dbl(b)
        lines.append(f"  {{{bh.hex()}, {fhex(flt(b - mp.mpf(bh)))}, 0}}, \\")
    lines += ["}", ""]
    ln2_hi = round_bits(mp.log(2), 42)             # e*ln2_hi exact for |e| < 2^11
    l256 = mp.log(2) / 256
    lg256 = mp.log10(2) / 256
    consts = {
        "FM_LN2_HI": ln2_hi.hex(), "FM_LN2_LO_F": fhex(flt(mp.log(2) - mp.mpf(ln2_hi))),
        "FM_INV_L256_F": fhex(flt(256 / mp.log(2))),
        "FM_L256_HI": dbl(l256).hex(), "FM_L256_LO_F": fhex(flt(l256 - mp.mpf(dbl(l256)))),
        "FM_INV_LG256_F": fhex(flt(256 / mp.log10(2))),
        "FM_LG256_HI": dbl(lg256).hex(), "FM_LG256_LO_F": fhex(flt(lg256 - mp.mpf(dbl(lg256)))),
        "FM_LN10": dbl(mp.log(10)).hex(), "FM_LN10_F": fhex(flt(mp.log(10))),
        "FM_PIO2": dbl(mp.pi / 2).hex(),
    }
    for k, v in consts.items():
        lines.append(f"#define {k} {v}")
    with open(os.path.join(HERE, "fastmath_tables.h"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
