"""Generate ff32_tables.h: tables and split constants of the float-float exp / log in ff32.cuh.

    python frehg_gb300/csrc/gen_ff32_tables.py > frehg_gb300/csrc/ff32_tables.h

Values are computed with Python's decimal module at 60 significant digits; a float-float value
is hi = the float nearest to it and lo = the float nearest to the remainder (together about 48
significant bits).
  exp: T_j = 2^(j/128), j = 0..127 (hi + lo, and the next float of the remainder)
  log: c_j = 1 + (j + 1/2)/256 (the centre of the j-th of 256 mantissa intervals of [1, 2)),
       1/c_j and ln(c_j) as float-float, j = 0..255
  ln2/128 = C1 + C2 + C3 with C1 10 significant bits (k C1 exact for |k| < 2^14);
  ln2 = L1 + L2 + L3 with L1 16 significant bits (e L1 exact for |e| < 2^8).
"""
from decimal import Decimal, getcontext
import struct

getcontext().prec = 60
LN2 = Decimal(2).ln()


def f32(v) -> float:
    """nearest float32 of a Decimal or float (exactly, via the double nearest to it when the
    value has more digits: the hi/lo split below keeps the remainder exact in Decimal)"""
    return struct.unpack("f", struct.pack("f", float(v)))[0]


def split(v: Decimal):
    hi = f32(v)
    lo = f32(v - Decimal(hi))
    return hi, lo


def trunc_bits(v: Decimal, bits: int) -> float:
    """v rounded to `bits` significant bits (a float32 with trailing zeros)"""
    e = 0
    x = v
    while x >= 1:
        x /= 2
        e += 1
    while x < Decimal("0.5"):
        x *= 2
        e -= 1
    m = int((x * (1 << bits)).to_integral_value())
    return float(Decimal(m) / (Decimal(2) ** bits) * (Decimal(2) ** e))


def lit(x: float) -> str:
    return "0.0f" if x == 0.0 else f"{x.hex()}f"


def main():
    step = LN2 / 128
    c1 = trunc_bits(step, 10)
    c2 = f32(step - Decimal(c1))
    c3 = f32(step - Decimal(c1) - Decimal(c2))
    l1 = trunc_bits(LN2, 16)
    l2 = f32(LN2 - Decimal(l1))
    l3 = f32(LN2 - Decimal(l1) - Decimal(l2))
    out = ["// Generated by gen_ff32_tables.py: tables of the float-float exp and log.",
           "#pragma once", "", "namespace fg {", "",
           f"constexpr float kFfInvLn2x128 = {lit(f32(128 / LN2))};  // 128 / ln 2",
           f"constexpr float kFfLn2x128C1 = {lit(c1)};  // ln2/128 = C1 + C2 + C3",
           f"constexpr float kFfLn2x128C2 = {lit(c2)};",
           f"constexpr float kFfLn2x128C3 = {lit(c3)};",
           f"constexpr float kFfLn2L1 = {lit(l1)};  // ln 2 = L1 + L2 + L3",
           f"constexpr float kFfLn2L2 = {lit(l2)};",
           f"constexpr float kFfLn2L3 = {lit(l3)};", "",
           "// 2^(j/128) = hi + lo, j = 0..127",
           "__device__ const float2 kFfExp2Tab[128] = {"]
    lo2s = []
    for j in range(128):
        t = (LN2 * j / 128).exp()
        hi, lo = split(t)
        lo2s.append(f32(t - Decimal(hi) - Decimal(lo)))
        out.append(f"    {{{lit(hi)}, {lit(lo)}}},")
    out += ["};", "",
            "// 2^(j/128) - hi - lo (expm1 adds it where its result is much smaller than 1)",
            "__device__ const float kFfExp2Lo2[128] = {"]
    out += [f"    {lit(v)}," for v in lo2s]
    out += ["};", "",
            "// c_j = 1 + (j + 1/2)/256: {1/c_j hi, 1/c_j lo, ln(c_j) hi, ln(c_j) lo}, j = 0..255",
            "__device__ const float4 kFfLogTab[256] = {"]
    for j in range(256):
        c = Decimal(1) + (Decimal(j) + Decimal("0.5")) / 256
        ih, il = split(Decimal(1) / c)
        lh, ll = split(c.ln())
        out.append(f"    {{{lit(ih)}, {lit(il)}, {lit(lh)}, {lit(ll)}}},")
    out += ["};", "", "}  // namespace fg", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
