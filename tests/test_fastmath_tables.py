"""The constants of the chemistry kernels' table-driven exp and log
(hyperflow_gb300/csrc/hf_fastmath_tables.h) are what gen_fastmath.py computes: each
the double nearest to the exact value (2^(j/64), 2^(-j/64), log F_j, 1/F_j and the
split ln2 constants)."""
import contextlib
import io
import math
import os
import sys

import numpy as np

CSRC = os.path.join(os.path.dirname(__file__), "..", "hyperflow_gb300", "csrc")


def test_committed_tables_match_generator():
    sys.path.insert(0, CSRC)
    try:
        import gen_fastmath
    finally:
        sys.path.pop(0)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        gen_fastmath.main()
    with open(os.path.join(CSRC, "hf_fastmath_tables.h")) as f:
        assert f.read() == buf.getvalue()


def _table(name):
    text = open(os.path.join(CSRC, "hf_fastmath_tables.h")).read()
    body = text.split("%s[64] = {" % name)[1].split("};")[0]
    return np.array([float.fromhex(t) for t in body.replace("\n", " ").split(",") if t.strip()])


def test_table_entries_within_half_ulp_of_libm():
    j = np.arange(64)
    F = 1.0 + (j + 0.5) / 64.0
    for name, ref in (("EXP_TAB", np.exp2(j / 64.0)), ("EXPM_TAB", np.exp2(-j / 64.0)), ("LOG_F", np.log(F)),
                      ("LOG_IF", 1.0 / F)):
        t = _table(name)
        assert t.shape == (64,)
        # the generator rounds the exact value; libm here is within an ulp of it
        assert np.all(np.abs(t - ref) <= np.spacing(np.abs(ref))), name


def test_split_constants():
    text = open(os.path.join(CSRC, "hf_fastmath_tables.h")).read()

    def const(name):
        return float.fromhex(text.split(name + " = ")[1].split(",")[0].split(";")[0].strip())

    hi, lo = const("LN2_64_HI"), const("LN2_64_LO")
    assert abs((hi + lo) - math.log(2) / 64) <= 1e-18
    # k * HI exact for |k| < 2^17: HI has at most 36 significant bits
    m, e = math.frexp(hi)
    assert (m * 2 ** 36).is_integer()
    hi, lo = const("LN2_HI"), const("LN2_LO")
    assert abs((hi + lo) - math.log(2)) <= 1e-17
    m, e = math.frexp(hi)
    assert (m * 2 ** 42).is_integer()
