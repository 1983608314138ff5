"""Generate mtg_fp64_tables.h: the tables of the table-driven FP64 exp and log of
mtg_common.cuh (the methods of P. T. P. Tang, ACM TOMS 15 (1989) 144 and 16 (1990)
378), computed here with 60-digit decimal arithmetic and rounded to doubles.

  exp: S_j = 2^(j/64), j = 0..63, as hi + lo; ln2/64 as L1 (32 significant bits,
       so n * L1 is exact for |n| < 2^21) + L2; 64/ln2.
  log: for m in (sqrt(1/2), sqrt(2)] split at 0.703125 + j/128 (j = 0..91), an
       approximate reciprocal inv_c_j with at most 10 significant bits (1 exactly
       for the two intervals around 1, so that log x near 1 has no cancellation),
       and -log(inv_c_j) as hi (a multiple of 2^-42, so e * LN2_HI + hi is exact)
       + lo; ln2 as LN2_HI (a multiple of 2^-42) + LN2_LO.

Usage: python mytrim_gb300/csrc/gen_fp64_tables.py > mytrim_gb300/csrc/mtg_fp64_tables.h
"""
from decimal import Decimal, getcontext
from fractions import Fraction

getcontext().prec = 60


def to_double(d):
    return float(Fraction(d))  # correctly rounded


def hexs(x):
    return float.hex(x)


def quantize(d, q):
    """d rounded to a multiple of q (a power of two), as a double."""
    f = Fraction(d) / q
    n = round(f)
    return float(n * q)


def main():
    ln2 = Decimal(2).ln()
    out = ["// Generated by gen_fp64_tables.py -- tables of the FP64 exp / log in mtg_common.cuh.",
           "#pragma once", "", "// clang-format off"]
    # exp
    L = ln2 / 64
    L1 = quantize(L, Fraction(1, 2 ** 37))  # 32 significant bits (L ~ 2^-6.5)
    L2 = to_double(L - Decimal(Fraction(L1).numerator) / Decimal(Fraction(L1).denominator))
    out.append(f"#define MTG_EXP_INV_L {hexs(to_double(64 / ln2))}")
    out.append(f"#define MTG_EXP_L1 {hexs(L1)}")
    out.append(f"#define MTG_EXP_L2 {hexs(L2)}")
    hi, lo = [], []
    for j in range(64):
        s = Decimal(2) ** (Decimal(j) / 64)
        h = to_double(s)
        hi.append(h)
        lo.append(to_double(s - Decimal(Fraction(h).numerator) / Decimal(Fraction(h).denominator)))
    out.append("#define MTG_EXP_TABLE_HI \\")
    out.append("  " + ", \\\n  ".join(", ".join(hexs(v) for v in hi[i:i + 4]) for i in range(0, 64, 4)))
    out.append("#define MTG_EXP_TABLE_LO \\")
    out.append("  " + ", \\\n  ".join(", ".join(hexs(v) for v in lo[i:i + 4]) for i in range(0, 64, 4)))
    # log
    q = Fraction(1, 2 ** 42)
    ln2_hi = quantize(ln2, q)
    ln2_lo = to_double(ln2 - Decimal(Fraction(ln2_hi).numerator) / Decimal(Fraction(ln2_hi).denominator))
    out.append(f"#define MTG_LOG_LN2_HI {hexs(ln2_hi)}")
    out.append(f"#define MTG_LOG_LN2_LO {hexs(ln2_lo)}")
    invc, lhi, llo = [], [], []
    for j in range(92):
        lo_m = Fraction(703125, 1000000) + Fraction(j, 128)
        if j in (37, 38):  # [0.9921875, 1.0078125): c = 1
            ic = Fraction(1)
        else:
            c = lo_m + Fraction(1, 256)
            ic = Fraction(round(Fraction(512) / c), 512)
        invc.append(float(ic))
        L = -(Decimal(ic.numerator) / Decimal(ic.denominator)).ln()
        h = quantize(L, q) if ic != 1 else 0.0
        lhi.append(h)
        llo.append(to_double(L - Decimal(Fraction(h).numerator) / Decimal(Fraction(h).denominator)) if ic != 1 else 0.0)
    for name, arr in (("MTG_LOG_INVC", invc), ("MTG_LOG_TABLE_HI", lhi), ("MTG_LOG_TABLE_LO", llo)):
        out.append(f"#define {name} \\")
        out.append("  " + ", \\\n  ".join(", ".join(hexs(v) for v in arr[i:i + 4]) for i in range(0, 92, 4)))
    out.append("// clang-format on")
    print("\n".join(out))


if __name__ == "__main__":
    main()
