"""The table-driven exp, paired exp(x)/exp(-x) and log of the chemistry kernels
(hyperflow_gb300/csrc/hf_fastmath.cuh, after Tang 1989/1990), replayed on the CPU step
for step in double precision (a correctly rounded fma from exact rational arithmetic, the
same table constants parsed from hf_fastmath_tables.h), against libm: within 2 ulp over
the fast ranges (absolute 3e-16 near log's zero at x = 1)."""
import math
import os
import struct
from fractions import Fraction

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "hyperflow_gb300", "csrc")


def _tables():
    text = open(os.path.join(CSRC, "hf_fastmath_tables.h")).read()

    def arr(name):
        body = text.split("%s[64] = {" % name)[1].split("};")[0]
        return [float.fromhex(t) for t in body.replace("\n", " ").split(",") if t.strip()]

    def const(name):
        return float.fromhex(text.split(name + " = ")[1].split(",")[0].split(";")[0].strip())

    return {"EXP": arr("EXP_TAB"), "EXPM": arr("EXPM_TAB"), "LOGF": arr("LOG_F"), "LOGIF": arr("LOG_IF"),
            "L64H": const("LN2_64_HI"), "L64L": const("LN2_64_LO"), "LH": const("LN2_HI"), "LL": const("LN2_LO"),
            "I64": const("INV_LN2_64")}


T = _tables()


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def hi_lo(x):
    bits = struct.unpack("<q", struct.pack("<d", x))[0]
    return (bits >> 32), bits & 0xffffffff


def from_hi_lo(hi, lo):
    return struct.unpack("<d", struct.pack("<q", ((hi & 0xffffffff) << 32) | lo))[0]


def scale(v, m):
    hi, lo = hi_lo(v)
    return from_hi_lo(hi + m * (1 << 20), lo)


def reduce(x):
    SH = float.fromhex("0x1.8p52")
    t = fma(x, T["I64"], SH)
    k = struct.unpack("<q", struct.pack("<d", t))[0] & 0xffffffff
    k = k - (1 << 32) if k >= 1 << 31 else k  # the low word as a signed int
    kd = t - SH
    r = fma(-kd, T["L64H"], x)
    r = fma(-kd, T["L64L"], r)
    return k, r


def fexp(x):
    k, r = reduce(x)
    q = fma(fma(fma(r, 1.0 / 120.0, 1.0 / 24.0), r, 1.0 / 6.0), r, 0.5)
    p = fma(r * r, q, r)
    j = k & 63
    tj = T["EXP"][j]
    return scale(fma(tj, p, tj), (k - j) // 64)


def fexp_pair(x):
    k, r = reduce(x)
    r2 = r * r
    E = r2 * fma(r2, 1.0 / 24.0, 0.5)
    O = r * fma(r2, fma(r2, 1.0 / 120.0, 1.0 / 6.0), 1.0)
    j = k & 63
    m = (k - j) // 64
    tp, tm = T["EXP"][j], T["EXPM"][j]
    return scale(fma(tp, E + O, tp), m), scale(fma(tm, E - O, tm), -m)


def flog(x):
    hi, lo = hi_lo(x)
    m = (hi >> 20) - 1023
    j = (hi >> 14) & 63
    y = from_hi_lo((hi & 0x000fffff) | 0x3ff00000, lo)
    F = fma(float(j), 1.0 / 64.0, 1.0 + 1.0 / 128.0)
    u = (y - F) * T["LOGIF"][j]
    q = fma(fma(fma(fma(fma(u, 1.0 / 7.0, -1.0 / 6.0), u, 0.2), u, -0.25), u, 1.0 / 3.0), u, -0.5)
    l1p = fma(u * u, q, u)
    md = float(m)
    return fma(md, T["LH"], T["LOGF"][j]) + fma(md, T["LL"], l1p)


def ulps(got, ref):
    return abs(got - ref) / math.ulp(abs(ref))


@pytest.mark.parametrize("seed", [1, 2])
def test_exp_forms(seed):
    rng = np.random.default_rng(seed)
    xs = np.concatenate([rng.uniform(-699.0, 699.0, 400), rng.uniform(-2, 2, 400), rng.uniform(-300, 10, 200),
                         np.arange(-8, 9) * math.log(2) / 64])
    worst = 0.0
    for x in xs.tolist():
        e = fexp(x)
        ep, em = fexp_pair(x)
        worst = max(worst, ulps(e, math.exp(x)), ulps(ep, math.exp(x)), ulps(em, math.exp(-x)))
    assert worst <= 2.0, worst


def test_log():
    rng = np.random.default_rng(3)
    xs = np.concatenate([np.exp(rng.uniform(-700, 700, 500)), rng.uniform(150, 6000, 300), rng.uniform(0.5, 2, 300)])
    for x in xs.tolist():
        ref = math.log(x)
        err = abs(flog(x) - ref)
        assert err <= max(2.0 * math.ulp(abs(ref)), 3e-16), (x, err)
