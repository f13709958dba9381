"""Generate dust2gpu/tables.hpp: correctly rounded constant tables for the
table-driven exp and log of math.hpp (double tables for exp's FP64 slow
path, fixed-point tables for the integer exp and log) and the reciprocals
of small integers used by the binomial inversion sampler.

Every value is computed in 60-digit decimal arithmetic and rounded once to
the nearest double; a "lo" entry holds the rounded remainder of the exact
value after its "hi" entry.

Run:  python dust2_gb300/csrc/dust2gpu/make_tables.py
"""

from decimal import Decimal, getcontext
from fractions import Fraction
from pathlib import Path

getcontext().prec = 60
LN2 = Decimal(2).ln()


def rn(x):
    """Round a Decimal/Fraction to the nearest double."""
    if isinstance(x, Decimal):
        x = Fraction(x)
    return float(x)


def hi_lo(x):
    hi = rn(x)
    lo = rn(Decimal(x) - Decimal(hi))
    return hi, lo


def fmt(v):
    return float(v).hex()


def main():
    out = []
    out.append("// Generated by make_tables.py -- do not edit.")
    out.append("#pragma once")
    out.append("")
    # exp: 2^(j/128), j = 0..127
    out.append("// 2^(j/128) = EXP2_HI[j] + EXP2_LO[j]")
    his, los = [], []
    for j in range(128):
        v = (LN2 * j / 128).exp()
        h, lo = hi_lo(v)
        his.append(h)
        los.append(lo)
    out.append("#define DUST2_EXP2_HI \\")
    out.append(",\\\n".join("  " + ", ".join(fmt(v) for v in his[i:i + 3])
                           for i in range(0, 128, 3)))
    out.append("#define DUST2_EXP2_LO \\")
    out.append(",\\\n".join("  " + ", ".join(fmt(v) for v in los[i:i + 3])
                           for i in range(0, 128, 3)))
    # log: F = j/256 for j = 181..363 (m in [sqrt(2)/2, sqrt(2))); the
    # fixed-point tables are written by fixed_point_tables()
    out.append("")
    j0, j1 = 181, 363
    out.append(f"#define DUST2_LOG_J0 {j0}")
    out.append(f"#define DUST2_LOG_N {j1 - j0 + 1}")
    # 1/x for x = 0..128 (entry 0 unused)
    out.append("")
    out.append("// 1/x, x = 0..128 (entry 0 is 0)")
    rec = [0.0] + [rn(Fraction(1, x)) for x in range(1, 129)]
    out.append("#define DUST2_RECIP_INT \\")
    out.append(",\\\n".join("  " + ", ".join(fmt(v) for v in rec[i:i + 3])
                           for i in range(0, len(rec), 3)))
    # constants
    out.append("")
    h, lo = hi_lo(LN2 / 128)
    # split ln2/128 so that k * hi is exact for |k| < 2^18
    hi_bits = rn(Fraction(LN2 / 128).limit_denominator(1 << 60))
    import math
    m, e = math.frexp(h)
    hi35 = math.ldexp(math.floor(math.ldexp(m, 35)), e - 35)
    lo35 = rn(Decimal(LN2) / 128 - Decimal(hi35))
    out.append(f"#define DUST2_LN2_128_HI {fmt(hi35)}")
    out.append(f"#define DUST2_LN2_128_LO {fmt(lo35)}")
    out.append(f"#define DUST2_INV_LN2_128 {fmt(rn(128 / LN2))}")
    del hi_bits, lo
    fixed_point_tables(out)
    Path(__file__).with_name("tables.hpp").write_text("\n".join(out) + "\n")


def fixed_point_tables(out):
    """Tables and constants of the integer-arithmetic exp and log: values
    rounded to the nearest integer after scaling by the stated power of
    two (90-digit decimal arithmetic)."""
    getcontext().prec = 90
    ln2 = Decimal(2).ln()

    def rint(v):
        return int(Decimal(v).to_integral_value())

    def u64(v):
        assert 0 <= v < 1 << 64, v
        return f"0x{v:016x}ull"

    def words(v):
        """A signed 128-bit integer as (high int64 word, low uint64 word)."""
        assert -(1 << 127) <= v < 1 << 127, v
        return v >> 64, v & ((1 << 64) - 1)

    def table(name, vals, per_line=3):
        out.append(f"#define {name} \\")
        out.append(",\\\n".join("  " + ", ".join(vals[i:i + per_line])
                                for i in range(0, len(vals), per_line)))

    out.append("")
    out.append("// Integer-arithmetic exp and log (math.hpp exp / log):")
    out.append("// 2^(j/128) * 2^63, j = 0..127")
    table("DUST2_EXP2_Q63",
          [u64(rint((ln2 * j / 128).exp() * (Decimal(2) ** 63)))
           for j in range(128)])
    j0, j1 = 181, 363
    out.append("// 256/j * 2^62, j = LOG_J0 + i")
    table("DUST2_LOG_INV_Q62",
          [u64(rint(Decimal(256) / j * (Decimal(2) ** 62)))
           for j in range(j0, j1 + 1)])
    his, los = [], []
    for j in range(j0, j1 + 1):
        h, lo = words(rint((Decimal(j) / 256).ln() * (Decimal(2) ** 96)))
        his.append(f"{h}ll")
        los.append(u64(lo))
    out.append("// log(j/256) * 2^96 = LOG_F96_HI[i] * 2^64 + LOG_F96_LO[i]")
    table("DUST2_LOG_F96_HI", his)
    table("DUST2_LOG_F96_LO", los)
    c = rint(128 / ln2 * (Decimal(2) ** 120))
    out.append("// 128/ln2 * 2^120 = EXP_C120_HI * 2^64 + EXP_C120_LO")
    out.append(f"#define DUST2_EXP_C120_HI {u64(c >> 64)}")
    out.append(f"#define DUST2_EXP_C120_LO {u64(c & ((1 << 64) - 1))}")
    out.append("// ln2 * 2^64; ln2 * 2^96 = LN2_96_HI * 2^64 + LN2_96_LO")
    out.append(f"#define DUST2_LN2_Q64 {u64(rint(ln2 * (Decimal(2) ** 64)))}")
    l96 = rint(ln2 * (Decimal(2) ** 96))
    out.append(f"#define DUST2_LN2_96_HI {u64(l96 >> 64)}")
    out.append(f"#define DUST2_LN2_96_LO {u64(l96 & ((1 << 64) - 1))}")
    getcontext().prec = 60


if __name__ == "__main__":
    main()
