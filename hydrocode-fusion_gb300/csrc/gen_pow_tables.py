"""Generates csrc/hydro_pow_tables.h: the constant tables of the double-double
pow in hydro_pow.cuh (Tang's table-driven logarithm and exponential).

  log table, i = 0..127:  c_i = double(1 / (1 + (i + 1/2)/128)),
                          -log(c_i) split into hi + lo doubles;
  exp table, j = 0..127:  2^(j/128) split into hi + lo doubles;
  ln2 split so that e*LN2_HI is exact for |e| < 2^11,
  ln2/128 split so that k*LN2N_HI is exact for |k| < 2^18.

Run: python csrc/gen_pow_tables.py > csrc/hydro_pow_tables.h
"""
from decimal import Decimal, getcontext
import math

getcontext().prec = 60


def split(x: Decimal):
    hi = float(x)
    lo = float(x - Decimal(hi))
    return hi, lo


def trunc_bits(x: Decimal, bits: int) -> float:
    """x rounded to a double with at most `bits` significant bits."""
    f = float(x)
    m, e = math.frexp(f)
    scaled = round(m * (1 << bits))
    return math.ldexp(scaled, e - bits)


LN2 = Decimal(2).ln()
out = ["// Generated by csrc/gen_pow_tables.py -- do not edit.", "#pragma once", ""]
ln2_hi = trunc_bits(LN2, 42)
out.append(f"#define HYDRO_LN2_HI {ln2_hi.hex()}")
out.append(f"#define HYDRO_LN2_LO {float(LN2 - Decimal(ln2_hi)).hex()}")
l2n = LN2 / 128
l2n_hi = trunc_bits(l2n, 34)
out.append(f"#define HYDRO_LN2N_HI {l2n_hi.hex()}")
out.append(f"#define HYDRO_LN2N_LO {float(l2n - Decimal(l2n_hi)).hex()}")
out.append(f"#define HYDRO_INV_LN2N {float(Decimal(128) / LN2).hex()}")
out.append("")
out.append("// {c_i, -log(c_i) hi, -log(c_i) lo}")
out.append("HYDRO_POW_TABLE(hydro_log_tab, 3 * 128) = {")
for i in range(128):
    c = float(Decimal(1) / (Decimal(1) + (Decimal(i) + Decimal("0.5")) / 128))
    hi, lo = split(-Decimal(c).ln())
    out.append(f"    {c.hex()}, {hi.hex()}, {lo.hex()},")
out.append("};")
out.append("")
out.append("// {2^(j/128) hi, lo}")
out.append("HYDRO_POW_TABLE(hydro_exp_tab, 2 * 128) = {")
for j in range(128):
    hi, lo = split(Decimal(2) ** (Decimal(j) / 128))
    out.append(f"    {hi.hex()}, {lo.hex()},")
out.append("};")
print("\n".join(out))
