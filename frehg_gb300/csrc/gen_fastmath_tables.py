"""Generate fastmath64_tables.h: the tables of the table-driven FP64 exp / log in fastmath64.cuh.

    python frehg_gb300/csrc/gen_fastmath_tables.py > frehg_gb300/csrc/fastmath64_tables.h

Values are computed with Python's decimal module at 60 significant digits and split into a
double `hi` (round to nearest) and the double nearest to the remainder `lo`.
  exp: T_j = 2^(j/64), j = 0..63
  log: c_j = 1 + (j + 1/2)/128 (the centre of the j-th of 128 mantissa intervals of [1, 2)),
       1/c_j rounded to double, ln(c_j) as hi + lo, j = 0..127
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
LN2 = Decimal(2).ln()


def split(v: Decimal):
    hi = float(v)
    lo = float(v - Decimal(hi))
    return hi, lo


def main():
    out = ["// Generated by gen_fastmath_tables.py: tables of the table-driven FP64 exp and log.",
           "#pragma once", "", "namespace fg {", "",
           "// 2^(j/64) = hi + lo, j = 0..63",
           "__device__ const double kExp2Tab[64][2] = {"]
    for j in range(64):
        hi, lo = split((LN2 * j / 64).exp())
        out.append(f"    {{{hi.hex()}, {lo.hex()}}},")
    out += ["};", "",
            "// c_j = 1 + (j + 1/2)/128: {1/c_j rounded, ln(c_j) hi, ln(c_j) lo}, j = 0..127",
            "__device__ const double kLogTab[128][3] = {"]
    for j in range(128):
        c = Decimal(1) + (Decimal(j) + Decimal("0.5")) / 128
        inv = float(Decimal(1) / c)
        hi, lo = split(c.ln())
        out.append(f"    {{{inv.hex()}, {hi.hex()}, {lo.hex()}}},")
    out += ["};", "", "}  // namespace fg", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
