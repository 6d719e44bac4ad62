"""The oracle on the reference's case configurations and blast checks, against the
outcomes the reference records for them (tests/golden/reference_records.json):
- HyperFlow_V3/docs/case_checks.json:7,12,38,43: Sun-CJ takes 25 steps to 1e-7 s and
  Teng case 1 takes 5 steps to 2e-9 s, neither with a retry.  The final states pass the
  checks of HyperFlow_V3/tests/check_cases.py:43-48,58,68.
- HyperFlow_V3/docs/amr_checks.json:35,52,101: the moving entropy wave takes 58 steps to
  4e-6 s, the inert blast 37 steps to 2e-6 s, and the reacting blast ends with a peak
  Y_H + Y_O + Y_OH of 1.4893699370443747e-07; the uniform chemistry run makes 5824
  chemistry cell calls over 1456 leaf cells, 4 steps.

The reference ran both cases on its AMR hierarchy.  Here each case is one level at the
finest resolution.  The step is the CFL step of the largest wave rate over all levels
(BlockAMR.cpp:335-346), which the finest level sets where it covers the hot spot or the
wedge tip.  So the step sequence, and with it the step count, is the same.  The count
pins the sound speeds and wave speeds of the hot and shocked gas within a few per cent:
Sun-CJ's 24th step ends 2.5 per cent short of 1e-7 s, Teng's 4th step 2.3 per cent short
of 2e-9 s.  The peak radical fraction of the reacting blast pins far more: the induction
chemistry at 1500 K / 10 atm over 2e-7 s, with the slight cooling that the flux scheme
brings to the disc centre (a 0D reactor alone gives 5.5e-5 more)."""
import numpy as np
import pytest

import helpers as H

REC = H.reference_records()


def run(oracle, U, lvd, case):
    """BlockAMR::run on one level (BlockAMR.cpp:400-416): the CFL step shortened to land
    on each output time; returns (final interior state, step sizes, rollbacks)."""
    bc = {"reflecting": 0, "transmissive": 1, "inflow": 2, "wedge": 3}
    g = oracle.make_grid(lvd["nx"], lvd["ny"], lvd["dx"], lvd["dy"], xlo=lvd.get("xlo", 0.0),
                         ylo=lvd.get("ylo", 0.0), periodic=lvd["periodic"],
                         bc_lo=tuple(bc[b] for b in lvd["boundary_lo"]),
                         bc_hi=tuple(bc[b] for b in lvd["boundary_hi"]), inlet=lvd["inlet"],
                         wedge_start=lvd.get("wedge_start", 0.0))
    Ug = oracle.fill_ghosts(g, oracle.ghosted(np.ascontiguousarray(U.transpose(1, 2, 0))))
    t, dts, rollbacks = 0.0, [], 0
    for target in case.get("output_times", [case["end_time"]]):
        while t < target:
            dt = min(target - t, oracle.cfl_dt(g, Ug, case["cfl"]))
            Ug, dta, st, _ = oracle.strang_step(g, Ug, dt, chemistry=case.get("chemistry", True))
            assert st == 0
            rollbacks += dta != dt
            t = target if dta >= target - t else t + dta
            dts.append(dta)
    assert t == case["end_time"]
    return Ug[2:-2, 2:-2], dts, rollbacks


def final_checks(oracle, F):
    """check_cases.py:45-48: finite, Y_k >= 0 summing to 1 within 1e-12, rho, p, T > 0."""
    q = F.reshape(-1, F.shape[-1])
    assert np.all(np.isfinite(q))
    rho = q[:, :9].sum(1)
    Y = q[:, :9] / rho[:, None]
    assert np.min(Y) >= 0 and np.max(np.abs(Y.sum(1) - 1)) < 1e-12
    p, _, T, st = oracle.properties(q)
    assert not np.any(st)
    assert rho.min() > 0 and p.min() > 0 and T.min() > 0


@pytest.fixture(scope="module")
def W():
    from hyperflow_gb300 import workloads
    return workloads


def test_sun_cj_smoke_case(oracle, W):
    """The leading 6 mm of the 0.5 m domain (the disturbance reaches 2.44 mm)."""
    U, lvd, case = W.sun_cj(nx=300, ny=2)
    F, dts, rollbacks = run(oracle, U, lvd, case)
    assert len(dts) == REC["sun_cj"]["steps"] and rollbacks == REC["sun_cj"]["retries"]
    final_checks(oracle, F)
    T0 = oracle.properties(U.transpose(1, 2, 0).reshape(-1, 12))[2]
    hot = np.isclose(T0, 3000.0, rtol=1e-10)
    # check_cases.py:58: the hot spot is 0.002 m^3 per unit depth (2 mm x 1 m)
    assert abs(hot.sum() * lvd["dx"] * lvd["dy"] - REC["sun_cj"]["initial_hotspot_volume_m3"]) < 1e-14
    # check_cases.py:68: mass and energy relative change (closed but for the far right
    # face, where the gas is at rest)
    a = U.transpose(1, 2, 0).reshape(-1, 12).sum(0)
    b = F.reshape(-1, 12).sum(0)
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11
    assert abs(b[11] / a[11] - 1) < 1e-9
    # the cut: every cell past the disturbance holds the far-field state
    far = np.nonzero(np.any(F != F[:, -1:], axis=(0, 2)))[0].max()
    assert (far + 1) * lvd["dx"] < 0.003


def test_teng_case1_smoke_case(oracle, W):
    U, lvd, case = W.teng_case1()
    assert (lvd["nx"], lvd["ny"]) == (576, 256) and abs(lvd["dx"] - 4e-6) < 1e-18
    F, dts, rollbacks = run(oracle, U, lvd, case)
    assert len(dts) == REC["teng_case1"]["steps"] and rollbacks == REC["teng_case1"]["retries"]
    final_checks(oracle, F)


def test_blast2d_inert_check(oracle, W):
    """validate.py:122-137: 37 steps, no retry, mass and energy within 1e-11, a pressure
    field symmetric under the transpose."""
    U, lvd, case = W.blast2d(reacting=False)
    F, dts, rollbacks = run(oracle, U, lvd, case)
    assert len(dts) == REC["blast2d_inert"]["steps"] and rollbacks == 0
    final_checks(oracle, F)
    a, b = U.transpose(1, 2, 0).reshape(-1, 12).sum(0), F.reshape(-1, 12).sum(0)
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
    p = oracle.properties(F.reshape(-1, 12))[0].reshape(F.shape[:2])
    assert np.mean(np.abs(p - p.T)) / np.mean(p) < 1e-12


def test_blast2d_reacting_peak_radicals(oracle, W):
    """validate.py:174-191: two steps of 1e-7 s, no retry, and the peak of
    Y_H + Y_O + Y_OH recorded as 1.4893699370443747e-07 (the oracle: 4.6e-7 below it;
    the reference integrates with CVODE on an AMR hierarchy)."""
    U, lvd, case = W.blast2d(reacting=True)
    F, dts, rollbacks = run(oracle, U, lvd, case)
    assert dts == [1e-7] * REC["blast2d_reacting"]["steps"] and rollbacks == REC["blast2d_reacting"]["retries"]
    final_checks(oracle, F)
    q = F.reshape(-1, 12)
    S = oracle.SPECIES
    peak = np.max((q[:, S.index("H")] + q[:, S.index("O")] + q[:, S.index("OH")]) / q[:, :9].sum(1))
    assert abs(peak / REC["blast2d_reacting"]["peak_radical_mass_fraction"] - 1) < 5e-6


def test_entropy_wave_check(oracle, W):
    """validate.py:104-119: 58 steps, no retry, mass and energy within 1e-11 (periodic)."""
    U, lvd, case = W.entropy_wave()
    F, dts, rollbacks = run(oracle, U, lvd, case)
    assert len(dts) == REC["moving_refine_coarsen"]["steps"] and rollbacks == 0
    final_checks(oracle, F)
    a, b = U.transpose(1, 2, 0).reshape(-1, 12).sum(0), F.reshape(-1, 12).sum(0)
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11


def test_uniform_chemistry_check(oracle):
    """validate.py:140-158 (the uniform-chemistry run of the BASE config at 1500 K / 5 atm
    to 2e-7 s) on its finest level: the reference records 5824 chemistry cell calls over
    1456 leaf cells (docs/amr_checks.json), i.e. 4 steps; the oracle takes 4 CFL steps."""
    from hyperflow_gb300 import case
    c = dict(problem="uniform", base_cells=[16, 16], length=[.01, .01], max_level=2, periodic=[1, 1],
             chemistry=True, cfl=.6, end_time=2e-7, T0=1500., P0=5 * 101325.)
    U, lvd, run_opts = case.load(c, refine=2)
    F, dts, rollbacks = run(oracle, U, lvd, dict(run_opts, chemistry=True))
    rec = REC["zero_dimensional_cvode"]
    assert rec["chemistry_cell_calls"] == rec["expected_leaf_calls"]
    assert len(dts) == rec["chemistry_cell_calls"] // REC["uniform_local_amr"]["leaf_cells"] and rollbacks == 0
    final_checks(oracle, F)
    T = oracle.properties(F.reshape(-1, 12))[2]
    assert np.ptp(T) == 0.0  # a uniform state stays uniform (validate.py:95-97)
