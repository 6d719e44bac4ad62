"""Multi-step runs on the GPU against the CPU oracle, and the reference's output files.

The 1D planar detonation (2000 x 2 cells on 0.1 m in the benchmark; a 400 x 2 cut of it
here, N2 diluent so the oracle's 9-species mechanism applies): a driver of 20 cells at
40 atm / 3000 K, reflecting left, transmissive right, reflecting top and bottom.
"""
import os

import numpy as np
import pytest
import torch

import helpers as H

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_det1d_steps_match_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det1d(diluent="N2", nx=400)
    lv = hf.make_level(**lvd)
    g = oracle.make_grid(400, 2, lvd["dx"], lvd["dy"], periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    st = hf.Stepper(gpu, lv, cuda(U), flux="fused", chem="plain")
    for _ in range(12):
        dt = oracle.cfl_dt(g, Ug, 0.5)
        Ug, dta, ok, _ = oracle.strang_step(g, Ug, dt)
        assert ok == 0
        assert st.step(dt=dta) == dta
    got = st.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, 12)
    ref = Ug[2:-2, 2:-2].reshape(-1, 12)
    Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
    assert np.max(np.abs(Tg - Tr) / Tr) < 1e-6
    assert np.max(np.abs(got[:, :9] - ref[:, :9]) / ref[:, :9].sum(1, keepdims=True)) < 1e-8


def test_run_case_writes_reference_files(gpu, tmp_path):
    """state_N.csv / boxes_N.csv / history.csv / summary.json as BlockAMR writes them,
    read back the way tests/validate.py reads them; conservation with closed walls."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import output, workloads as W
    U, lvd = W.det1d(diluent="N2", nx=200)
    lvd.update(boundary_hi=("reflecting", "reflecting"))
    lv = hf.make_level(**lvd)
    summary = output.run_case(gpu, lv, cuda(U), 2e-8, str(tmp_path), flux="fused", chem="batched")
    names = sorted(os.listdir(tmp_path))
    assert names == ["boxes_0.csv", "boxes_1.csv", "history.csv", "state_0.csv", "state_1.csv", "summary.json"]
    data = np.genfromtxt(tmp_path / "state_1.csv", names=True, delimiter=",")
    assert len(data) == 400
    Y = np.column_stack([data[n] for n in data.dtype.names if n.startswith("Y_")])
    assert np.min(Y) >= 0 and np.max(np.abs(Y.sum(1) - 1)) < 1e-12
    assert abs(data["t"][0] - 2e-8) < 1e-20 and summary["final_time"] == 2e-8
    s = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(s["initial_conserved_integrals"]), np.array(s["final_conserved_integrals"])
    assert abs(b[:9].sum() - a[:9].sum()) / a[:9].sum() < 1e-13
    assert abs(b[11] - a[11]) / abs(a[11]) < 1e-12
    hist = np.genfromtxt(tmp_path / "history.csv", names=True, delimiter=",")
    assert len(hist) == s["steps"] + 1


def _final_checks(data):
    """HyperFlow_V3/tests/check_cases.py:45-48 on a state_N.csv read back."""
    assert all(np.isfinite(data[n]).all() for n in data.dtype.names)
    Y = np.column_stack([data[n] for n in data.dtype.names if n.startswith("Y_")])
    assert np.min(Y) >= 0 and np.max(np.abs(Y.sum(1) - 1)) < 1e-12
    assert all(np.min(data[n]) > 0 for n in ["rho", "p", "T"])


def test_sun_cj_smoke_case(gpu, oracle, tmp_path):
    """The reference's Sun-CJ smoke case on its finest level (25000 x 8 cells): 25 steps to
    1e-7 s with no retry (HyperFlow_V3/docs/case_checks.json:7,12) and the final checks of
    tests/check_cases.py:43-48,58,68; then its leading 6 mm against the oracle."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import output, workloads as W
    U, lvd, case = W.sun_cj()
    s = output.run_case(gpu, hf.make_level(**lvd), cuda(U), case["end_time"], str(tmp_path), cfl=case["cfl"],
                        flux="plain", chem="batched")
    R = H.reference_records()["sun_cj"]
    assert s["steps"] == R["steps"] and s["retries"] == R["retries"] and s["final_time"] == R["final_time_s"]
    first = np.genfromtxt(tmp_path / "state_0.csv", names=True, delimiter=",")
    final = np.genfromtxt(tmp_path / "state_1.csv", names=True, delimiter=",")
    _final_checks(final)
    volume = first["dx"] * first["dy"]
    hot = np.isclose(first["T"], 3000.0, rtol=1e-10)
    assert abs(volume.sum() - 0.5) < 1e-13 and abs(volume[hot].sum() - R["initial_hotspot_volume_m3"]) < 1e-14
    a, b = np.array(json.loads((tmp_path / "summary.json").read_text())["initial_conserved_integrals"]), \
        np.array(s["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-9

    U, lvd, case = W.sun_cj(nx=300, ny=2)
    st = hf.Stepper(gpu, hf.make_level(**lvd), cuda(U), flux="plain", chem="batched")
    g = oracle.make_grid(300, 2, lvd["dx"], lvd["dy"], bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.fill_ghosts(g, oracle.ghosted(np.ascontiguousarray(U.transpose(1, 2, 0))))
    t = 0.0
    while t < case["end_time"]:
        dt = min(case["end_time"] - t, oracle.cfl_dt(g, Ug, case["cfl"]))
        Ug, dta, ok, _ = oracle.strang_step(g, Ug, dt)
        assert ok == 0 and st.step(dt=dta) == dta
        t = case["end_time"] if dta >= case["end_time"] - t else t + dta
    got = st.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, 12)
    ref = Ug[2:-2, 2:-2].reshape(-1, 12)
    Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
    assert np.max(np.abs(Tg - Tr) / Tr) < 1e-6
    assert np.max(np.abs(got[:, :9] - ref[:, :9]) / ref[:, :9].sum(1, keepdims=True)) < 1e-8
    st.close()


def test_teng_case1_smoke_case(gpu, oracle, tmp_path):
    """The reference's Teng case-1 smoke case on its finest level (576 x 256 cells, wedge
    bottom, inflow left and top): 5 steps to 2e-9 s with no retry
    (HyperFlow_V3/docs/case_checks.json:38,43), the final checks of
    tests/check_cases.py:43-48, and the final state against the oracle's run."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import output, workloads as W
    U, lvd, case = W.teng_case1()
    s = output.run_case(gpu, hf.make_level(**lvd), cuda(U), case["end_time"], str(tmp_path), cfl=case["cfl"],
                        flux="plain", chem="batched")
    R = H.reference_records()["teng_case1"]
    assert s["steps"] == R["steps"] and s["retries"] == R["retries"] and s["final_time"] == R["final_time_s"]
    final = np.genfromtxt(tmp_path / "state_1.csv", names=True, delimiter=",")
    _final_checks(final)
    assert len(final) == 576 * 256
    bc = {"reflecting": 0, "transmissive": 1, "inflow": 2, "wedge": 3}
    g = oracle.make_grid(lvd["nx"], lvd["ny"], lvd["dx"], lvd["dy"], xlo=lvd["xlo"],
                         bc_lo=tuple(bc[x] for x in lvd["boundary_lo"]), bc_hi=tuple(bc[x] for x in lvd["boundary_hi"]),
                         inlet=lvd["inlet"], wedge_start=0.0)
    Ug = oracle.fill_ghosts(g, oracle.ghosted(np.ascontiguousarray(U.transpose(1, 2, 0))))
    st = hf.Stepper(gpu, hf.make_level(**lvd), cuda(U), flux="plain", chem="batched")
    t = 0.0
    while t < case["end_time"]:
        dt = min(case["end_time"] - t, oracle.cfl_dt(g, Ug, case["cfl"]))
        Ug, dta, ok, _ = oracle.strang_step(g, Ug, dt)
        assert ok == 0 and st.step(dt=dta) == dta
        t = case["end_time"] if dta >= case["end_time"] - t else t + dta
    got = st.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, 12)
    ref = Ug[2:-2, 2:-2].reshape(-1, 12)
    Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
    assert np.max(np.abs(Tg - Tr) / Tr) < 1e-6
    assert np.max(np.abs(got[:, :9] - ref[:, :9]) / ref[:, :9].sum(1, keepdims=True)) < 1e-8
    st.close()


def _stepper_run(gpu, U, lvd, case):
    """BlockAMR::run (BlockAMR.cpp:400-416) on the GPU stepper: the device CFL step
    shortened to land on each output time; returns (final state (ny*nx, NV), step sizes)."""
    import hyperflow_gb300 as hf
    st = hf.Stepper(gpu, hf.make_level(**lvd), cuda(U), chemistry=case["chemistry"], flux="plain", chem="batched")
    t, dts = 0.0, []
    for target in case["output_times"]:
        while t < target:
            dt = st.step(dt=min(target - t, st.cfl_dt(case["cfl"])), cfl=case["cfl"])
            t = target if dt >= target - t else t + dt
            dts.append(dt)
    out = st.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, U.shape[0])
    st.close()
    return out, dts


def test_blast2d_checks(gpu, oracle):
    """The reference's blast checks on one level at their finest resolution: the inert
    blast takes 37 steps to 2e-6 s and the reacting blast ends with a peak Y_H + Y_O + Y_OH
    of 1.4893699370443747e-07 (HyperFlow_V3/docs/amr_checks.json:52,101); both against
    the oracle's runs."""
    from hyperflow_gb300 import workloads as W
    R = H.reference_records()
    for reacting in (False, True):
        U, lvd, case = W.blast2d(reacting=reacting)
        got, dts = _stepper_run(gpu, U, lvd, case)
        g = oracle.make_grid(lvd["nx"], lvd["ny"], lvd["dx"], lvd["dy"], bc_lo=(0, 0), bc_hi=(0, 0))
        Ug = oracle.fill_ghosts(g, oracle.ghosted(np.ascontiguousarray(U.transpose(1, 2, 0))))
        for dt in dts:
            Ug, dta, ok, _ = oracle.strang_step(g, Ug, dt, chemistry=reacting)
            assert ok == 0 and dta == dt
        ref = Ug[2:-2, 2:-2].reshape(-1, 12)
        Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
        assert np.max(np.abs(Tg - Tr) / Tr) < 1e-6
        assert np.max(np.abs(got[:, :9] - ref[:, :9]) / ref[:, :9].sum(1, keepdims=True)) < 1e-8
        if reacting:
            assert dts == [1e-7] * R["blast2d_reacting"]["steps"]
            S = oracle.SPECIES
            peak = np.max((got[:, S.index("H")] + got[:, S.index("O")] + got[:, S.index("OH")]) / got[:, :9].sum(1))
            assert abs(peak / R["blast2d_reacting"]["peak_radical_mass_fraction"] - 1) < 5e-6
        else:
            assert len(dts) == R["blast2d_inert"]["steps"]


def test_entropy_wave_check(gpu, oracle):
    """The reference's moving-refinement check on one 64 x 64 level: 58 steps to 4e-6 s
    (HyperFlow_V3/docs/amr_checks.json:35), against the oracle's run."""
    from hyperflow_gb300 import workloads as W
    U, lvd, case = W.entropy_wave()
    got, dts = _stepper_run(gpu, U, lvd, case)
    assert len(dts) == H.reference_records()["moving_refine_coarsen"]["steps"]
    g = oracle.make_grid(64, 64, lvd["dx"], lvd["dy"], periodic=(1, 1))
    Ug = oracle.fill_ghosts(g, oracle.ghosted(np.ascontiguousarray(U.transpose(1, 2, 0))))
    for dt in dts:
        Ug, dta, ok, _ = oracle.strang_step(g, Ug, dt, chemistry=False)
        assert ok == 0 and dta == dt
    ref = Ug[2:-2, 2:-2].reshape(-1, 12)
    assert H.comp_err(got, ref) < 1e-10


def test_amr_regrid_run_matches_composite_oracle(gpu, oracle):
    """A two-level periodic AMR run whose box tags move 8 coarse cells in 4 steps, with a
    regrid after every step (and hf_amr_create's initial one): after each step the active
    blocks equal the composite oracle's (oracle/amr.py), and at the end both levels agree
    with it to 1e-10 of each component's physical scale (flux path only)."""
    import amr
    import hyperflow_gb300 as hf
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=7)
    g = oracle.make_grid(nx, ny, dx / 2, dx / 2, periodic=(1, 1))
    dt = 0.5 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(U0)), 1.0)
    tags = dict(box=(0.0004, 0.0008, -1.0, 1.0), box_only=True, velocity=(8 * dx / (4 * dt), 0.0))
    lv = hf.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    m = hf.AmrStepper(gpu, lv, cuda(U0.transpose(2, 0, 1)), max_level=1, block=B, tag_buffer=1, regrid_interval=1,
                      chemistry=False, tags=tags)
    o = amr.AmrOracle.from_base(U0, dx, dx, B, amr.criteria(chemistry=False, **tags), tag_buffer=1,
                                regrid_interval=1, chemistry=False)
    assert np.array_equal(m.level(1)[1], o.active)
    first = o.active.copy()
    for _ in range(4):
        assert m.step(dt=dt) == dt
        o.step(dt)
        assert np.array_equal(m.level(1)[1], o.active)
    assert not np.array_equal(first, o.active)
    G0 = m.level(0)[0].cpu().numpy().transpose(1, 2, 0)
    G1 = m.level(1)[0].cpu().numpy().transpose(1, 2, 0)
    pairs = [(G0.reshape(-1, 12), o.level(0).reshape(-1, 12))]
    for bj, bi in zip(*np.nonzero(o.active)):
        sl = (slice(bj * B, (bj + 1) * B), slice(bi * B, (bi + 1) * B))
        pairs.append((G1[sl].reshape(-1, 12), o.level(1)[sl].reshape(-1, 12)))
    ref_all = np.concatenate([r for _, r in pairs])
    rho = ref_all[:, :9].sum(1).max()
    scale = np.array([rho] * 9 + [rho * 1000.0] * 2 + [np.abs(ref_all[:, 11]).max()])
    for got, ref in pairs:
        assert np.max(np.abs(got - ref) / scale) < 1e-10
    m.close()


def test_run_amr_case_writes_reference_files(gpu, tmp_path):
    """BlockAMR::run on three levels through run_amr_case: the reference's files at t = 0
    and two output times, each state file a tiling of the domain by leaf cells
    (validate.py:64-78), mass and energy conserved on the periodic box to 1e-11
    (validate.py:133), one history row per step."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import output, workloads as W
    from test_output_amr import check_geometry
    U, lvd = W.det2d(seed=6, diluent="N2", nx=32, ny=16, hot_columns=6)
    lvd = dict(lvd, periodic=(1, 1))
    lv = hf.make_level(**lvd)
    s = output.run_amr_case(gpu, lv, cuda(U), 2e-8, str(tmp_path), cfl=0.5, output_times=[1e-8, 2e-8], max_level=2,
                            block=16, tag_buffer=1, regrid_interval=2, chem="batched",
                            tags=dict(pressure_tag=0.08, temperature_tag=0.08, density_tag=0.05))
    names = sorted(os.listdir(tmp_path))
    assert names == ["boxes_0.csv", "boxes_1.csv", "boxes_2.csv", "history.csv", "state_0.csv", "state_1.csv",
                     "state_2.csv", "summary.json"]
    # the composite oracle takes 5 steps here without a retry (tests/test_output_amr.py)
    assert s["completed"] and s["final_time"] == 2e-8 and s["retries"] == 0 and s["finest_level"] >= 1
    assert s["steps"] == 5
    for k in range(3):
        data = np.genfromtxt(tmp_path / ("state_%d.csv" % k), names=True, delimiter=",")
        check_geometry(data, (32, 16), (32 * lvd["dx"], 16 * lvd["dy"]), int(data["level"].max()))
        Y = np.column_stack([data[n] for n in data.dtype.names if n.startswith("Y_")])
        assert np.min(Y) >= 0 and np.max(np.abs(Y.sum(1) - 1)) < 1e-12
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
    hist = np.genfromtxt(tmp_path / "history.csv", names=True, delimiter=",")
    assert len(hist) == s["steps"] + 1 and hist["regrids"][-1] == s["regrids"]
    assert np.all(hist["leaf_cells"] > 0)


def test_amr_three_level_wedge_matches_composite_oracle(gpu, oracle):
    """The oblique-detonation wedge (inflow left and top, wedge bottom from x = 0,
    transmissive right) on three levels from the uniform free stream, density tags,
    a regrid every 2 steps, flux path only: after each of 6 graph-captured steps the
    active blocks of levels 1 and 2 equal the composite oracle's (oracle/amr.py, fed
    the GPU's step sizes), and at the end every level agrees with it to 1e-9 of each
    component's physical scale."""
    import amr
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.wedge(nx=64, ny=32)
    tags = dict(density_tag=0.05)
    m = hf.AmrStepper(gpu, hf.make_level(**lvd), cuda(U), max_level=2, block=16, tag_buffer=1, regrid_interval=2,
                      chemistry=False, tags=tags)
    o = amr.Hierarchy.from_base(U.transpose(1, 2, 0), lvd, 16, amr.criteria(chemistry=False, **tags), max_level=2,
                                tag_buffer=1, regrid_interval=2, chemistry=False)
    for _ in range(6):
        o.step(m.step(cfl=0.5))
        for lev in (1, 2):
            assert np.array_equal(m.level(lev)[1], o.acts[lev] if lev <= o.finest else np.zeros_like(o.acts[lev]))
    assert o.finest == 2 and m.info(0)["finest"] == 2
    pairs = [(m.level(0)[0].cpu().numpy().transpose(1, 2, 0).reshape(-1, 12), o.level(0).reshape(-1, 12))]
    for lev in (1, 2):
        G = m.level(lev)[0].cpu().numpy().transpose(1, 2, 0)
        R = o.level(lev)
        for bj, bi in zip(*np.nonzero(o.acts[lev])):
            sl = (slice(bj * 16, (bj + 1) * 16), slice(bi * 16, (bi + 1) * 16))
            pairs.append((G[sl].reshape(-1, 12), R[sl].reshape(-1, 12)))
    ref_all = np.concatenate([r for _, r in pairs])
    rho = ref_all[:, :9].sum(1).max()
    scale = np.array([rho] * 9 + [rho * 1000.0] * 2 + [np.abs(ref_all[:, 11]).max()])
    for got, ref in pairs:
        assert np.max(np.abs(got - ref) / scale) < 1e-9
    m.close()


def test_amr_rollback_matches_composite_oracle(gpu, oracle):
    """Two periodic levels with part of level 1 active, one step of 8 times the CFL step
    on the host-driven path: the GPU stepper and the composite oracle roll back and
    halve to the same step, and their levels agree to 1e-10 of each component's physical
    scale (flux path only)."""
    import amr
    import hyperflow_gb300 as hf
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=7)
    crit = dict(box=(0.0008, 0.0016, -1.0, 1.0), box_only=True)
    m = hf.AmrStepper(gpu, hf.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1)), cuda(U0.transpose(2, 0, 1)),
                      max_level=1, block=B, tag_buffer=1, regrid_interval=0, chemistry=False, tags=crit)
    o = amr.AmrOracle.from_base(U0, dx, dx, B, amr.criteria(chemistry=False, **crit), tag_buffer=1, chemistry=False)
    assert np.array_equal(m.level(1)[1], o.active) and 0 < o.active.sum() < o.active.size
    dt = 8.0 * m.cfl_dt(1.0)
    h = m.step(dt=dt)
    assert h < dt and o.step(dt) == h
    pairs = [(m.level(0)[0].cpu().numpy().transpose(1, 2, 0).reshape(-1, 12), o.level(0).reshape(-1, 12))]
    G1, R1 = m.level(1)[0].cpu().numpy().transpose(1, 2, 0), o.level(1)
    for bj, bi in zip(*np.nonzero(o.active)):
        sl = (slice(bj * B, (bj + 1) * B), slice(bi * B, (bi + 1) * B))
        pairs.append((G1[sl].reshape(-1, 12), R1[sl].reshape(-1, 12)))
    ref_all = np.concatenate([r for _, r in pairs])
    rho = ref_all[:, :9].sum(1).max()
    scale = np.array([rho] * 9 + [rho * 1000.0] * 2 + [np.abs(ref_all[:, 11]).max()])
    for got, ref in pairs:
        assert np.max(np.abs(got - ref) / scale) < 1e-10
    m.close()


def test_flux_adjoint_matches_oracle_fd(gpu, oracle):
    """hf_flux_adjoint (one Euler stage, walls left and at the top and bottom, periodic
    nowhere, transmissive right): J^T w against kink-free central differences of
    <w, stage(U)> from the oracle's stage at 24 sampled entries, the entries weighted by
    the component's physical scale: 1e-5 relative (2-norm) and 1e-4 for each entry."""
    import hyperflow_gb300 as hf
    from test_gpu_flow_adjoint import clean_difference, scales
    nx, ny, dx = 24, 12, 1e-4
    A = H.smooth_field(nx, ny, seed=21)                  # (ny, nx, NV)
    U = np.ascontiguousarray(A.transpose(2, 0, 1))       # (NV, ny, nx)
    lvd = dict(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
               boundary_hi=("transmissive", "reflecting"))
    level = hf.make_level(**lvd)
    g = oracle.make_grid(nx, ny, dx, dx, periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0))
    h = 0.3 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(A)), 1.0)
    sc = scales(U)
    w = np.random.default_rng(5).uniform(-1.0, 1.0, U.shape) / sc[:, None, None]
    pa = hf.PatchArray(12, nx, ny)
    pa.interior().copy_(cuda(U))
    hf.fill(gpu, level, pa)
    wb = pa.like()
    wb.interior().copy_(cuda(w))
    G = hf.flux_adjoint(gpu, level, pa, wb, h).interior().cpu().numpy()

    def J(V):
        o, _, _, st = oracle.euler_stage(g, oracle.fill_ghosts(g, oracle.ghosted(V.transpose(1, 2, 0))), h)
        assert st == 0
        return float(np.sum(w * o[2:-2, 2:-2].transpose(2, 0, 1)))

    J0 = J(U)
    rng = np.random.default_rng(9)
    got, want = [], []
    while len(got) < 24:
        n, j, i = int(rng.integers(0, 12)), int(rng.integers(0, ny)), int(rng.integers(0, nx))
        i = [0, 1, nx - 2, nx - 1, i][int(rng.integers(0, 5))]  # boundary cells too
        if n < 9 and U[n, j, i] <= 1e-5 * sc[n]:
            continue  # a step of 1e-6 of the scale would make the partial density negative
        fd = clean_difference(J, U, n, j, i, sc[n], J0, floor=1.0 / sc[n])
        got.append(G[n, j, i] * sc[n])
        want.append(fd * sc[n])
    got, want = np.array(got), np.array(want)
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
    assert np.all(np.abs(got - want) <= 1e-4 * np.maximum(np.abs(want), 1.0))


def test_reference_blast_config_through_the_amr_stepper(gpu, oracle, tmp_path):
    """The reference's reacting blast check (tests/validate.py:174-191) on the block-AMR
    stepper through case.load / case.levels and run_amr_case, the fine level built from
    the initial condition at its resolution (hf_amr_create_levels): two steps of 1e-7 s
    without a retry, mass and energy within 1e-11, and the recorded peak
    Y_H + Y_O + Y_OH 1.4893699370443747e-07 within 5e-6 relative (docs/amr_checks.json:101)."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import case, output
    from test_output_amr import check_geometry
    c = dict(problem="blast2d", base_cells=[16, 16], length=[.01, .01], max_level=1, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="physics", periodic=[0, 0], chemistry=True, cfl=.6,
             end_time=2e-7, output_times=[1e-7, 2e-7], regrid_interval=2, center=[.005, .005], radius=.0015,
             boundary_hi=["reflecting", "reflecting"])
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    s = output.run_amr_case(gpu, hf.make_level(**lvd), cuda(U0), run["end_time"], str(tmp_path), cfl=run["cfl"],
                            output_times=run["output_times"], max_level=run["max_level"], block=run["block"],
                            tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"], chemistry=True,
                            tags=run["tags"], U_levels=[cuda(u) for u in lv[1:]])
    assert s["steps"] == 2 and s["retries"] == 0
    data = np.genfromtxt(tmp_path / "state_2.csv", names=True, delimiter=",")
    check_geometry(data, (16, 16), (.01, .01), int(data["level"].max()))
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
    peak = float(np.max(data["Y_H"] + data["Y_O"] + data["Y_OH"]))
    assert abs(peak / H.reference_records()["blast2d_reacting"]["peak_radical_mass_fraction"] - 1) < 5e-6


def test_reference_inert_blast_config_through_the_amr_stepper(gpu, tmp_path):
    """The reference's inert blast check (tests/validate.py:122-137) on three levels of the
    block-AMR stepper through case.load / case.levels and run_amr_case: 37 steps to
    2e-6 s as recorded (docs/amr_checks.json:52), no retry, leaf cells tiling the domain,
    mass and energy within 1e-11."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import case, output
    from test_output_amr import check_geometry
    c = dict(problem="blast2d", base_cells=[24, 24], length=[.02, .02], max_level=2, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="physics", periodic=[0, 0], chemistry=False, cfl=.6,
             end_time=2e-6, output_times=[1e-6, 2e-6], regrid_interval=4, center=[.01, .01], radius=.002,
             boundary_lo=["reflecting", "reflecting"], boundary_hi=["reflecting", "reflecting"], pressure_tag=.06,
             temperature_tag=.06)
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    s = output.run_amr_case(gpu, hf.make_level(**lvd), cuda(U0), run["end_time"], str(tmp_path), cfl=run["cfl"],
                            output_times=run["output_times"], max_level=run["max_level"], block=run["block"],
                            tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"], chemistry=False,
                            tags=run["tags"], U_levels=[cuda(u) for u in lv[1:]])
    assert s["steps"] == H.reference_records()["blast2d_inert"]["steps"] and s["retries"] == 0
    for k in range(3):
        data = np.genfromtxt(tmp_path / ("state_%d.csv" % k), names=True, delimiter=",")
        check_geometry(data, (24, 24), (.02, .02), int(data["level"].max()))
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11


def test_reference_moving_refinement_config_through_the_amr_stepper(gpu, tmp_path):
    """The reference's moving-refinement check (tests/validate.py:104-119) on three levels
    of the block-AMR stepper through case.load / case.levels and run_amr_case: 58 steps
    to 4e-6 s as recorded (docs/amr_checks.json:35), no retry, mass and energy within
    1e-11 on the periodic box."""
    import json
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import case, output
    c = dict(problem="entropy_wave", base_cells=[16, 16], length=[.01, .01], max_level=2, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="box", tag_box=[.002, .004, .003, .005], periodic=[1, 1],
             chemistry=False, cfl=.6, end_time=4e-6, output_times=[2e-6, 4e-6], regrid_interval=4,
             center=[.003, .004], sigma=.0007, tag_velocity=[300., 200.], u0=300., v0=200.)
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    s = output.run_amr_case(gpu, hf.make_level(**lvd), cuda(U0), run["end_time"], str(tmp_path), cfl=run["cfl"],
                            output_times=run["output_times"], max_level=run["max_level"], block=run["block"],
                            tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"], chemistry=False,
                            tags=run["tags"], U_levels=[cuda(u) for u in lv[1:]])
    assert s["steps"] == H.reference_records()["moving_refine_coarsen"]["steps"] and s["retries"] == 0
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
