"""The autotuner (hyperflow_gb300/tune.py): a measured sweep of the batched chemistry's
launch settings on a sample call, applied through hf_set_chem_tuning when it beats the
default by the tuner's margin, and of the flux form on one Euler stage."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_chemistry_tuner_applies_the_fastest_candidate(gpu):
    from hyperflow_gb300 import tune, workloads as W
    U, _ = W.chem_batch(2048, seed=31, diluent="N2")
    X = torch.from_numpy(U).cuda()
    before = X.clone()
    default = tune.get_chem_tuning(gpu)
    try:
        res = tune.tune_chemistry(gpu, X, 5e-7)
        assert torch.equal(X, before)  # the sample call's input is not modified
        sweep = res["sweep"]
        assert len(sweep) == len(tune.CHEM_CANDIDATES) and all(r["ms"] > 0 for r in sweep)
        best = min(sweep, key=lambda r: r["ms"])
        base = [r for r in sweep if (r["blocks_per_sm"], r["coop_min_bucket"]) == tune.CHEM_DEFAULT][0]
        if best["ms"] >= (1.0 - tune.MARGIN) * base["ms"]:
            best = base  # the default stays unless a candidate beats it by the margin
        assert res["best"] == (best["blocks_per_sm"], best["coop_min_bucket"]) == tune.get_chem_tuning(gpu)
        # the cooperative phase runs for a low threshold and never for 16
        assert any(r["coop_cells"] > 0 for r in sweep if r["coop_min_bucket"] <= 4)
        assert all(r["coop_cells"] == 0 for r in sweep if r["coop_min_bucket"] == 16)
    finally:
        tune.set_chem_tuning(gpu, *default)
    assert tune.get_chem_tuning(gpu) == default


def test_flux_tuner_times_both_forms(gpu):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import tune, workloads as W
    U, lvd = W.det2d(seed=2, diluent="N2", nx=256, ny=64, hot_columns=16)
    lv = hf.make_level(**lvd)
    st = hf.Stepper(gpu, lv, torch.from_numpy(U).cuda(), flux="plain", chem="batched")
    dt = st.cfl_dt(0.5)
    res = tune.tune_flux(gpu, lv, st.state(), dt)
    st.close()
    assert set(res["ms"]) == {"plain", "fused"} and res["best"] in res["ms"]
    assert all(np.isfinite(v) and v > 0 for v in res["ms"].values())


def test_stepper_tuner_times_whole_steps(gpu):
    """tune_stepper: each candidate from a fresh stepper over whole graph steps; the
    default (no cooperative phase) stays unless a candidate beats it by the margin, and the
    cooperative candidate's queue engages on the stiff 1D detonation."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import tune, workloads as W
    U, lvd = W.det1d(diluent="N2", nx=400)
    lv = hf.make_level(**lvd)
    default = tune.get_chem_tuning(gpu)
    try:
        res = tune.tune_stepper(gpu, lv, torch.from_numpy(U).cuda(), 0.5, warm=10, steps=10,
                                candidates=[tune.CHEM_DEFAULT, (4, 3)])
        sweep = res["sweep"]
        assert [(r["blocks_per_sm"], r["coop_min_bucket"]) for r in sweep] == [tune.CHEM_DEFAULT, (4, 3)]
        assert all(r["ms_per_step"] > 0 for r in sweep)
        assert sweep[0]["coop_cells"] == 0 and sweep[1]["coop_cells"] > 0
        base, other = sweep
        want = (4, 3) if other["ms_per_step"] < (1 - tune.MARGIN) * base["ms_per_step"] else tune.CHEM_DEFAULT
        assert res["best"] == want == tune.get_chem_tuning(gpu)
    finally:
        tune.set_chem_tuning(gpu, *default)
