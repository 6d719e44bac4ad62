"""The tuner's choice rule (hyperflow_gb300/tune.py): a candidate replaces the default
launch setting only when it is more than the margin faster."""
from hyperflow_gb300 import tune


def row(minb, coop, ms):
    return {"blocks_per_sm": minb, "coop_min_bucket": coop, "ms": ms}


def test_default_kept_within_margin():
    sweep = [row(4, 16, 100.0), row(4, 3, 98.0), row(8, 16, 120.0)]
    assert tune.pick(sweep, "ms") is sweep[0]


def test_faster_candidate_beyond_margin_wins():
    sweep = [row(4, 16, 100.0), row(4, 3, 40.0), row(8, 16, 120.0)]
    assert tune.pick(sweep, "ms") is sweep[1]


def test_default_fastest():
    sweep = [row(4, 3, 101.0), row(4, 16, 100.0)]
    assert tune.pick(sweep, "ms") is sweep[1]


def test_no_default_entry_takes_fastest():
    sweep = [row(5, 16, 90.0), row(4, 3, 80.0)]
    assert tune.pick(sweep, "ms") is sweep[1]


def test_margin_boundary():
    m = tune.MARGIN
    assert tune.pick([row(4, 16, 100.0), row(4, 5, 100.0 * (1 - m))], "ms")["coop_min_bucket"] == 16
    assert tune.pick([row(4, 16, 100.0), row(4, 5, 100.0 * (1 - m) - 1e-9)], "ms")["coop_min_bucket"] == 5
