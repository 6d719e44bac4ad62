"""Writes hf_fastmath_tables.h: the constants of the table-driven exp and log of
hf_fastmath.cuh, each the double nearest to its exact value (Python's decimal at 60
digits; float() of a decimal string rounds correctly).

  EXP_TAB[j]  = 2^(j/64),  EXPM_TAB[j] = 2^(-j/64)            j = 0..63
  LOG_F[j]    = log(F_j), LOG_IF[j] = 1/F_j,  F_j = 1 + (j + 0.5)/64   j = 0..63
  LN2_64_HI + LN2_64_LO = ln2/64 (HI with 36 significant bits: k*HI is exact for |k| < 2^17)
  LN2_HI + LN2_LO = ln2 (HI with 42 significant bits: m*HI is exact for |m| < 2^11)

Usage: python gen_fastmath.py > hf_fastmath_tables.h
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
LN2 = Decimal(2).ln()


def d(x):
    return float(str(x))


def hexd(x):
    return float(x).hex()


def split(v, bits):
    # v = hi + lo with hi carrying `bits` significant bits
    e = 0
    a = abs(v)
    while a >= 1:
        a /= 2
        e += 1
    while a < Decimal("0.5"):
        a *= 2
        e -= 1
    scale = Decimal(2) ** (bits - e)
    hi = (v * scale).to_integral_value() / scale
    return d(hi), d(v - hi)


def main():
    out = ["// Generated by gen_fastmath.py; do not edit.", "#pragma once", "namespace hf {", "namespace fm {"]
    exp_tab = [d((LN2 * j / 64).exp()) for j in range(64)]
    expm_tab = [d((-LN2 * j / 64).exp()) for j in range(64)]
    F = [1 + (Decimal(j) + Decimal("0.5")) / 64 for j in range(64)]
    log_f = [d(f.ln()) for f in F]
    log_if = [d(1 / f) for f in F]

    def arr(name, vals):
        out.append("static __device__ const double %s[64] = {" % name)
        for i in range(0, 64, 4):
            out.append("    " + ", ".join(hexd(v) for v in vals[i:i + 4]) + ",")
        out.append("};")

    arr("EXP_TAB", exp_tab)
    arr("EXPM_TAB", expm_tab)
    arr("LOG_F", log_f)
    arr("LOG_IF", log_if)
    h, l = split(LN2 / 64, 36)
    out.append("constexpr double LN2_64_HI = %s, LN2_64_LO = %s;" % (hexd(h), hexd(l)))
    h, l = split(LN2, 42)
    out.append("constexpr double LN2_HI = %s, LN2_LO = %s;" % (hexd(h), hexd(l)))
    out.append("constexpr double INV_LN2_64 = %s;  // 64/ln2" % hexd(d(64 / LN2)))
    out.append("constexpr double LN10 = %s, INV_LN10 = %s;" % (hexd(d(Decimal(10).ln())), hexd(d(1 / Decimal(10).ln()))))
    out += ["}  // namespace fm", "}  // namespace hf", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
