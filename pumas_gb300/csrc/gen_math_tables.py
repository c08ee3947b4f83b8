"""Generate gp_math_tables.h: the tables of the engine's table-driven
double precision logarithm and exponential (gp_math.cuh).

For j = 0 .. 128 the mantissa interval around F_j = 1 + j / 128 gets
  invF_j = 1 / F_j rounded to 10 significant bits (so that m * invF_j is
           exact in a fused multiply-add for any 53 bit mantissa m),
  T_j    = -ln(invF_j) as a pair (hi, lo) of doubles, hi + lo correct to
           about 2^-106 (computed with 60 decimal digits by mpmath).
Entry 128 (F = 2) uses invF = 1/2 and T = ln 2 split as LN2_HI + LN2_LO,
the constants of the exponent term, so that k ln 2 + T cancels exactly.

For the exponential, 2^(j/32), j = 0 .. 31, as pairs (hi, lo), and ln 2 / 32
split into a high part of 42 bits and a low part.

usage: python gen_math_tables.py > gp_math_tables.h
"""
import mpmath

mpmath.mp.dps = 60


def split(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def round_bits(v, bits):
    m, e = mpmath.frexp(v)          # v = m 2^e, 0.5 <= m < 1
    s = mpmath.nint(m * 2 ** bits)
    return float(s * mpmath.mpf(2) ** (e - bits))


def main():
    ln2 = mpmath.log(2)
    # ln 2 with a high part of 42 significant bits: k * LN2_HI is exact for
    # |k| < 2^11.
    ln2_hi = round_bits(ln2, 42)
    ln2_lo = float(ln2 - mpmath.mpf(ln2_hi))
    rows = []
    for j in range(129):
        if j == 128:
            rows.append((0.5, ln2_hi, ln2_lo))
            continue
        F = 1 + mpmath.mpf(j) / 128
        inv = round_bits(1 / F, 10)
        hi, lo = split(-mpmath.log(mpmath.mpf(inv)))
        rows.append((inv, hi, lo))
    print("/* Generated by gen_math_tables.py: tables of gp_log (gp_math.cuh). */")
    print("#ifndef GP_MATH_TABLES_H")
    print("#define GP_MATH_TABLES_H")
    print("#ifndef GP_MATH_TABLE")
    print("#define GP_MATH_TABLE static const")
    print("#endif")
    print("#define GP_LN2_HI %s /* %r */" % (ln2_hi.hex(), ln2_hi))
    print("#define GP_LN2_LO %s /* %r */" % (ln2_lo.hex(), ln2_lo))
    print("/* {1 / F_j (10 bits), -ln(1 / F_j) high, low}, F_j = 1 + j / 128. */")
    print("GP_MATH_TABLE double gp_log_table[129][3] = {")
    for inv, hi, lo in rows:
        print("        { %s, %s, %s }," % (inv.hex(), hi.hex(), lo.hex()))
    print("};")
    l32 = ln2 / 32
    l32_hi = round_bits(l32, 42)
    l32_lo = float(l32 - mpmath.mpf(l32_hi))
    print("#define GP_L32_HI %s /* %r */" % (l32_hi.hex(), l32_hi))
    print("#define GP_L32_LO %s /* %r */" % (l32_lo.hex(), l32_lo))
    inv = float(32 / ln2)
    print("#define GP_INV_L32 %s /* %r */" % (inv.hex(), inv))
    print("/* {2^(j/32) high, low}. */")
    print("GP_MATH_TABLE double gp_exp_table[32][2] = {")
    for j in range(32):
        hi, lo = split(mpmath.mpf(2) ** (mpmath.mpf(j) / 32))
        print("        { %s, %s }," % (hi.hex(), lo.hex()))
    print("};")
    print("#endif")


if __name__ == "__main__":
    main()
