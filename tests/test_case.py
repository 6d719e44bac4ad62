"""The case loader (hyperflow_gb300/case.py) on CPU: the reference's two smoke case
configurations (tests/golden/reference_cases.json, extracted from
HyperFlow_V3/cases/*/smoke.json) and the configs of its blast and moving-refinement checks
(HyperFlow_V3/tests/validate.py:19-24,104-108,122-128,174-178, restated) give, at their
finest resolution, exactly the initial states, levels and run options of the workloads
the oracle and GPU tests run."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

# validate.py:19-24
BASE = dict(problem="uniform", base_cells=[16, 16], length=[.01, .01], max_level=2, blocking_factor=4,
            max_grid_size=16, tag_buffer=1, tag_mode="box", tag_box=[.003, .007, .003, .007], periodic=[1, 1],
            chemistry=False, cfl=.6, end_time=2e-7, regrid_interval=2)


@pytest.fixture(scope="module")
def cases():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
        return json.load(f)


def same_level(a, b):
    for k in ("nx", "ny", "dx", "dy", "periodic", "boundary_lo", "boundary_hi"):
        assert tuple(np.atleast_1d(a[k])) == tuple(np.atleast_1d(b[k])), k
    for k in ("xlo", "ylo", "wedge_start"):  # make_level's defaults: 0
        assert a.get(k, 0.0) == b.get(k, 0.0), k
    assert np.array_equal(a["inlet"], b["inlet"])


def test_sun_cj_smoke_case(cases):
    from hyperflow_gb300 import case, workloads as W
    U, lv, run = case.load(cases["sun_cj"], refine=2)
    Uw, lw, cw = W.sun_cj()
    assert np.array_equal(U, Uw)
    same_level(lv, lw)
    assert run["cfl"] == cw["cfl"] and run["end_time"] == cw["end_time"] and run["output_times"] == [1e-7]
    assert run["chemistry"] and run["max_level"] == 2 and run["regrid_interval"] == 16 and run["tag_buffer"] == 2
    assert run["tags"]["box"] == (0.0, 0.002, 0.0, 1.0) and not run["tags"]["box_only"]
    assert run["block"] is None  # 2 base rows: no block of 8 or more cells fits


def test_teng_case1_smoke_case(cases):
    from hyperflow_gb300 import case, workloads as W
    U, lv, run = case.load(cases["teng_case1"], refine=2)
    Uw, lw, cw = W.teng_case1()
    assert np.array_equal(U, Uw)
    same_level(lv, lw)
    assert run["cfl"] == cw["cfl"] and run["end_time"] == cw["end_time"]
    assert run["block"] == 8 and run["tags"]["temperature_tag"] == 0.06


@pytest.mark.parametrize("reacting", [False, True])
def test_blast_checks(reacting):
    from hyperflow_gb300 import case, workloads as W
    c = dict(BASE)
    if reacting:  # validate.py:174-178
        c.update(problem="blast2d", chemistry=True, max_level=1, center=[.005, .005], radius=.0015,
                 tag_mode="physics", periodic=[0, 0], boundary_hi=["reflecting", "reflecting"], end_time=2e-7,
                 output_times=[1e-7, 2e-7], regrid_interval=2)
    else:  # validate.py:122-128
        c.update(problem="blast2d", base_cells=[24, 24], length=[.02, .02], center=[.01, .01], radius=.002,
                 periodic=[0, 0], boundary_lo=["reflecting", "reflecting"], boundary_hi=["reflecting", "reflecting"],
                 tag_mode="physics", pressure_tag=.06, temperature_tag=.06, end_time=2e-6, output_times=[1e-6, 2e-6],
                 regrid_interval=4)
    c.pop("tag_box")
    U, lv, run = case.load(c, refine=c["max_level"])
    Uw, lw, cw = W.blast2d(reacting=reacting)
    assert np.array_equal(U, Uw)
    same_level(lv, lw)
    assert run["output_times"] == cw["output_times"] and run["chemistry"] == cw["chemistry"]


def test_moving_refinement_check():
    from hyperflow_gb300 import case, workloads as W
    c = dict(BASE)  # validate.py:104-108
    c.update(problem="entropy_wave", center=[.003, .004], sigma=.0007, tag_box=[.002, .004, .003, .005],
             tag_velocity=[300., 200.], u0=300., v0=200., end_time=4e-6, output_times=[2e-6, 4e-6], regrid_interval=4)
    U, lv, run = case.load(c, refine=2)
    Uw, lw, cw = W.entropy_wave()
    assert np.allclose(U, Uw, rtol=1e-14, atol=0)
    assert lv["periodic"] == (1, 1) and lv["nx"] == 64 and lv["dx"] == lw["dx"]
    assert run["tags"]["box_only"] and run["tags"]["velocity"] == (300.0, 200.0) and run["block"] == 8


def test_rejections():
    from hyperflow_gb300 import case
    with pytest.raises(ValueError):
        case.load(dict(BASE, problem="nozzle"))
    with pytest.raises(ValueError):
        case.load(dict(BASE, cfl=0.9))
    with pytest.raises(ValueError):
        case.load(dict(BASE, problem="teng_osw", inflow_speed=2000.0, wedge_angle_deg=95.0))


@pytest.mark.parametrize("problem", ["uniform", "sod_x", "sod_y", "example6", "example7", "entropy_wave", "blast2d"])
def test_every_problem_loads_admissible_states(oracle, problem):
    """Every initial condition of BlockAMR::initial (BlockAMR.cpp:84-121) on a small grid:
    admissible cells, and the shape of each problem's initial field."""
    from hyperflow_gb300 import case
    c = dict(problem=problem, base_cells=[16, 8], length=[1.0, 0.5] if problem.startswith("example") else [.01, .005],
             end_time=1e-7)
    U, lv, run = case.load(c)
    q = U.reshape(12, -1).T
    p, _, T, st = oracle.properties(np.ascontiguousarray(q))
    assert not np.any(st)
    fresh, hot = case.states(c)
    if problem == "uniform":
        assert np.all(U == fresh[:, None, None])
    elif problem == "sod_x":       # hot left of the interface at x = L/2, fresh right of it
        assert np.allclose(U[:, :, :8], hot[:, None, None], rtol=1e-12, atol=0)
        assert np.allclose(U[:, :, 8:], fresh[:, None, None], rtol=1e-12, atol=0)
    elif problem == "sod_y":       # (the cell fractions at the interface round to 1 +- 1 ulp)
        assert np.allclose(U[:, :4, :], hot[:, None, None], rtol=1e-12, atol=0)
        assert np.allclose(U[:, 4:, :], fresh[:, None, None], rtol=1e-12, atol=0)
    elif problem == "example6":    # hot (moving at 800 m/s) up to x = 0.4
        rho = U[:9].sum(0)
        assert np.allclose(U[9, :, :6] / rho[:, :6], 800.0) and np.all(U[9, :, 7:] == 0.0)
    elif problem == "example7":    # hot (2000 m/s) left of x = max(0.5, 0.25 + distance to a wall)
        hot_cols = (U[9] != 0).sum(1)
        assert hot_cols[3] >= hot_cols[0] and hot_cols.min() >= 8
    elif problem == "entropy_wave":  # the temperature dip is centred at (0.3 L, 0.5 H)
        j, i = np.unravel_index(np.argmin(T.reshape(8, 16)), (8, 16))
        assert (j, i) in ((3, 4), (4, 4), (3, 5), (4, 5))
    else:                          # the hot disc at (0.3 L, 0.5 H), radius 0.1 H
        assert T.max() > 1000.0 and T.reshape(8, 16)[0, -1] == pytest.approx(300.0, rel=1e-12)
