"""The multi-level output writers (hyperflow_gb300/output.py) on CPU: the leaf cells of
a block hierarchy tile the domain once (the geometry check of
HyperFlow_V3/tests/validate.py:64-78), their conserved sums are the hierarchy's leaf
totals, and state_N.csv / boxes_N.csv read back the way the reference's scripts read
them.  The hierarchy comes from the composite AMR oracle, which also stands in for the
GPU stepper to check run_amr_case's host logic (output times, regrid cadence, history,
summary)."""
import numpy as np
import pytest

import helpers as H


def check_geometry(data, base_cells, length, max_level):
    """validate.py:64-78, restated: cell sizes per level, total area, every finest pixel
    covered by exactly one leaf cell."""
    level = data["level"].astype(int)
    base_dx = np.array(length) / np.array(base_cells)
    assert np.allclose(data["dx"], base_dx[0] / 2.0 ** level, rtol=1e-13, atol=0)
    assert np.allclose(data["dy"], base_dx[1] / 2.0 ** level, rtol=1e-13, atol=0)
    assert abs(np.sum(data["dx"] * data["dy"]) / np.prod(length) - 1) < 1e-13
    full = np.zeros(np.array(base_cells) * 2 ** max_level, dtype=np.int8)
    for q in data:
        r = 2 ** (max_level - int(q["level"]))
        i, j = int(q["i"]) * r, int(q["j"]) * r
        full[i:i + r, j:j + r] += 1
    assert np.all(full == 1), "leaf cells overlap or leave a hole"
    return len(data)


@pytest.fixture(scope="module")
def out():
    from hyperflow_gb300 import output
    return output


def test_leaf_masks_tile_three_levels(out):
    """Level 1 blocks 0-2 of row 0 and block (1, 1); level 2 blocks inside them."""
    nx, ny, B = 16, 8, 8
    act1 = np.zeros((2, 4), np.uint8)
    act1[0, :3] = 1
    act1[1, 1] = 1
    act2 = np.zeros((4, 8), np.uint8)
    act2[0, 1:4] = 1
    act2[1, 2] = 1
    acts, shapes = [None, act1, act2], [(ny, nx), (2 * ny, 2 * nx), (4 * ny, 4 * nx)]
    masks = out.leaf_masks(acts, shapes, B)
    full = np.zeros((4 * ny, 4 * nx), np.int8)
    for l, m in enumerate(masks):
        r = 2 ** (2 - l)
        for j, i in zip(*np.nonzero(m)):
            full[j * r:(j + 1) * r, i * r:(i + 1) * r] += 1
    assert np.all(full == 1)
    boxes = out.amr_boxes(acts, shapes, B)
    assert boxes[0] == (0, 0, 0, nx - 1, ny - 1) and len(boxes) == 1 + 4 + 4


def test_state_rows_of_the_oracle_hierarchy(oracle, out, tmp_path):
    import amr
    from hyperflow_gb300 import solver as S
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=5)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=6)
    active = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    active[:, 2:5] = 1
    active[1, 6] = 1
    a = amr.AmrOracle(U0, U1, active, dx, dx, B)
    base = S.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    Qs = [a.level(0).transpose(2, 0, 1), a.level(1).transpose(2, 0, 1)]
    acts, shapes = [None, a.active], [(ny, nx), (2 * ny, 2 * nx)]

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    rows = out.amr_state_rows(Qs, out.leaf_masks(acts, shapes, B), base, 1e-7, props)
    ns = U0.shape[2] - 3
    out.write_rows(tmp_path / "state_1.csv", rows, ns)
    out.write_amr_boxes(tmp_path / "boxes_1.csv", out.amr_boxes(acts, shapes, B), base)
    data = np.genfromtxt(tmp_path / "state_1.csv", names=True, delimiter=",")
    n = check_geometry(data, (nx, ny), (nx * dx, ny * dx), 1)
    assert n == nx * ny - int(active.sum()) * (B // 2) ** 2 + int(active.sum()) * B * B
    # conserved sums of the rows = the hierarchy's leaf totals
    vol = data["dx"] * data["dy"]
    Y = np.column_stack([data["Y_" + s] for s in out.SPECIES[:ns]])
    got = np.concatenate([(data["rho"][:, None] * Y * vol[:, None]).sum(0),
                          [(data["rho"] * data["u"] * vol).sum(), (data["rho"] * data["v"] * vol).sum(),
                           (data["rhoE"] * vol).sum()]])
    want = a.totals()
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    boxes = np.genfromtxt(tmp_path / "boxes_1.csv", names=True, delimiter=",")
    assert len(boxes) == 1 + int(active.sum())
    assert abs(np.sum((boxes["x_right"] - boxes["x_left"]) * (boxes["y_top"] - boxes["y_bottom"])
                      * (boxes["level"] == 1)) - active.sum() * (B * dx / 2) ** 2) < 1e-18


class OracleAmr:
    """AmrStepper's interface over the composite oracle (regrids driven by the caller)."""

    def __init__(self, oracle, amr, U0, lvd, block, crit, max_level, tag_buffer, chemistry=False, levels=None):
        self.o, self.B = oracle, block
        self.h = amr.Hierarchy.from_base(U0, lvd, block, crit, max_level=max_level, tag_buffer=tag_buffer,
                                         regrid_interval=0, chemistry=chemistry, levels=levels)

    def info(self, lev):
        h = self.h
        (ny, nx), (nby, nbx) = h.shape[lev], h.nb[lev]
        leaf = int(h.leaf_mask(lev).sum()) if lev <= h.finest else 0
        return dict(nx=nx, ny=ny, nbx=nbx, nby=nby, finest=h.finest, leaf_cells=leaf)

    def level(self, lev):
        import torch
        h = self.h
        act = h.acts[lev] if lev <= h.finest else np.zeros_like(h.acts[lev])
        return torch.from_numpy(np.ascontiguousarray(h.level(lev).transpose(2, 0, 1))), act.copy()

    def cfl_dt(self, cfl):
        h, o, B = self.h, self.o, self.B
        dts = [o.cfl_dt(h.g[0], o.fill_ghosts(h.g[0], h.X[0].copy()), cfl)]
        for lev in range(1, h.finest + 1):
            for bi, bj in h.blocks(lev):
                win = h.X[lev][bj * B:bj * B + B + 4, bi * B:bi * B + B + 4]
                dts.append(o.cfl_dt(h._grid(lev, bi * B, bj * B, B, B), win, cfl))
        return min(dts)

    def step(self, dt=0.0, cfl=0.5):
        return self.h.step(dt)

    def regrid(self):
        self.h.regrid()

    def totals(self):
        return self.h.totals()

    def close(self):
        pass


class CountingCtx:
    """The counters run_amr_case reads, taken from the composite oracle behind the stepper."""

    def __init__(self, stepper):
        self.h = stepper.h

    def counters(self):
        h = self.h
        return {"retries": h.retries, "first_order_stages": h.first_order_stages,
                "roundoff_repairs": h.roundoff_repairs, "chem_cell_calls": 0}


def test_run_amr_case_host_logic(oracle, out, tmp_path):
    """run_amr_case over the composite oracle: the reference's files at t = 0 and at two
    output times, leaf cells tiling the domain on three levels, one history row per
    step, a regrid after every second step except one that reached the end time
    (BlockAMR.cpp:420), and conserved totals on the periodic box."""
    import json
    import amr
    import torch
    from hyperflow_gb300 import solver as S
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=15)
    lvd = dict(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    g = oracle.make_grid(4 * nx, 4 * ny, dx / 4, dx / 4, periodic=(1, 1))
    dt = 0.5 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(np.kron(U0, np.ones((4, 4, 1))))), 1.0)
    kw = dict(box=(0.0008, 0.0016, 0.0004, 0.0012), box_only=True, velocity=(2 * dx / (2 * dt), 0.0))
    stepper = OracleAmr(oracle, amr, U0, lvd, B, amr.criteria(chemistry=False, **kw), 2, 1)

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    end = 5.5 * dt
    s = out.run_amr_case(CountingCtx(stepper), S.make_level(**lvd), torch.from_numpy(U0.transpose(2, 0, 1).copy()), end,
                         str(tmp_path), cfl=0.5, output_times=[2.5 * dt, end], max_level=2, block=B, tag_buffer=1,
                         regrid_interval=2, chemistry=False, stepper=stepper, props=props)
    import os
    assert sorted(os.listdir(tmp_path)) == ["boxes_0.csv", "boxes_1.csv", "boxes_2.csv", "history.csv",
                                            "state_0.csv", "state_1.csv", "state_2.csv", "summary.json"]
    assert s["final_time"] == end and s["finest_level"] == 2
    steps = s["steps"]
    assert s["regrids"] == sum(1 for k in range(1, steps) if k % 2 == 0)
    for k in range(3):
        data = np.genfromtxt(tmp_path / ("state_%d.csv" % k), names=True, delimiter=",")
        check_geometry(data, (nx, ny), (nx * dx, ny * dx), 2)
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
    hist = np.genfromtxt(tmp_path / "history.csv", names=True, delimiter=",")
    assert len(hist) == steps + 1 and hist["regrids"][-1] == s["regrids"] and hist["finest_level"][-1] == 2
    assert abs(hist["t"][-1] - end) == 0 and np.all(np.diff(hist["t"]) > 0)


def test_reference_blast_config_through_the_amr_runner(oracle, out, tmp_path):
    """The reference's reacting blast check (tests/validate.py:174-191: config, then the
    peak Y_H + Y_O + Y_OH of the last state file) through case.load / case.levels and
    run_amr_case, with the composite oracle standing in for the GPU stepper: two steps of
    1e-7 s without a retry, and the recorded peak 1.4893699370443747e-07 within 5e-6
    relative (docs/amr_checks.json:101)."""
    import amr
    import torch
    from hyperflow_gb300 import case, solver as S
    c = dict(problem="blast2d", base_cells=[16, 16], length=[.01, .01], max_level=1, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="physics", periodic=[0, 0], chemistry=True, cfl=.6,
             end_time=2e-7, output_times=[1e-7, 2e-7], regrid_interval=2, center=[.005, .005], radius=.0015,
             boundary_hi=["reflecting", "reflecting"])
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    crit = amr.criteria(chemistry=run["chemistry"], **run["tags"])
    stepper = OracleAmr(oracle, amr, U0.transpose(1, 2, 0), lvd, run["block"], crit, run["max_level"], run["tag_buffer"],
                        chemistry=True, levels=[u.transpose(1, 2, 0) for u in lv[1:]])

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    s = out.run_amr_case(CountingCtx(stepper), S.make_level(**lvd), torch.from_numpy(U0), run["end_time"], str(tmp_path),
                         cfl=run["cfl"], output_times=run["output_times"], max_level=run["max_level"],
                         block=run["block"], tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"],
                         chemistry=True, stepper=stepper, props=props)
    assert s["steps"] == 2 and s["retries"] == 0 and s["regrids"] == 0
    data = np.genfromtxt(tmp_path / "state_2.csv", names=True, delimiter=",")
    check_geometry(data, (16, 16), (.01, .01), int(data["level"].max()))
    peak = float(np.max(data["Y_H"] + data["Y_O"] + data["Y_OH"]))
    assert abs(peak / H.reference_records()["blast2d_reacting"]["peak_radical_mass_fraction"] - 1) < 5e-6


def test_reference_inert_blast_config_through_the_amr_runner(oracle, out, tmp_path):
    """The reference's inert blast check (tests/validate.py:122-137) on three levels
    through case.load / case.levels and run_amr_case, the composite oracle standing in
    for the GPU stepper: 37 steps to 2e-6 s as recorded (docs/amr_checks.json:52), no
    retry, leaf cells tiling the domain, mass and energy within 1e-11."""
    import json
    import amr
    import torch
    from hyperflow_gb300 import case, solver as S
    c = dict(problem="blast2d", base_cells=[24, 24], length=[.02, .02], max_level=2, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="physics", periodic=[0, 0], chemistry=False, cfl=.6,
             end_time=2e-6, output_times=[1e-6, 2e-6], regrid_interval=4, center=[.01, .01], radius=.002,
             boundary_lo=["reflecting", "reflecting"], boundary_hi=["reflecting", "reflecting"], pressure_tag=.06,
             temperature_tag=.06)
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    crit = amr.criteria(chemistry=False, **run["tags"])
    stepper = OracleAmr(oracle, amr, U0.transpose(1, 2, 0), lvd, run["block"], crit, run["max_level"],
                        run["tag_buffer"], levels=[u.transpose(1, 2, 0) for u in lv[1:]])

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    s = out.run_amr_case(CountingCtx(stepper), S.make_level(**lvd), torch.from_numpy(U0), run["end_time"], str(tmp_path),
                         cfl=run["cfl"], output_times=run["output_times"], max_level=run["max_level"],
                         block=run["block"], tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"],
                         chemistry=False, stepper=stepper, props=props)
    assert s["steps"] == H.reference_records()["blast2d_inert"]["steps"] and s["retries"] == 0
    assert s["finest_level"] == 2
    for k in range(3):
        data = np.genfromtxt(tmp_path / ("state_%d.csv" % k), names=True, delimiter=",")
        check_geometry(data, (24, 24), (.02, .02), int(data["level"].max()))
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11


def test_reference_moving_refinement_config_through_the_amr_runner(oracle, out, tmp_path):
    """The reference's moving-refinement check (tests/validate.py:104-119: the entropy wave
    with box tags moving at (300, 200) m/s, three levels, a regrid every 4 steps) through
    case.load / case.levels and run_amr_case over the composite oracle: 58 steps to 4e-6 s
    as recorded (docs/amr_checks.json:35), no retry, refinement both gained and lost,
    mass and energy within 1e-11 on the periodic box."""
    import json
    import amr
    import torch
    from hyperflow_gb300 import case, solver as S
    c = dict(problem="entropy_wave", base_cells=[16, 16], length=[.01, .01], max_level=2, blocking_factor=4,
             max_grid_size=16, tag_buffer=1, tag_mode="box", tag_box=[.002, .004, .003, .005], periodic=[1, 1],
             chemistry=False, cfl=.6, end_time=4e-6, output_times=[2e-6, 4e-6], regrid_interval=4,
             center=[.003, .004], sigma=.0007, tag_velocity=[300., 200.], u0=300., v0=200.)
    U0, lvd, run = case.load(c)
    lv = case.levels(c)
    stepper = OracleAmr(oracle, amr, U0.transpose(1, 2, 0), lvd, run["block"],
                        amr.criteria(chemistry=False, **run["tags"]), run["max_level"], run["tag_buffer"],
                        levels=[u.transpose(1, 2, 0) for u in lv[1:]])
    first = stepper.h.acts[2].copy()

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    s = out.run_amr_case(CountingCtx(stepper), S.make_level(**lvd), torch.from_numpy(U0), run["end_time"], str(tmp_path),
                         cfl=run["cfl"], output_times=run["output_times"], max_level=run["max_level"],
                         block=run["block"], tag_buffer=run["tag_buffer"], regrid_interval=run["regrid_interval"],
                         chemistry=False, stepper=stepper, props=props)
    assert s["steps"] == H.reference_records()["moving_refine_coarsen"]["steps"] and s["retries"] == 0
    last = stepper.h.acts[2]
    assert np.any(last & (1 - first)) and np.any(first & (1 - last))
    summ = json.loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11


def test_reacting_detonation_through_the_amr_runner_takes_no_retry(oracle, out, tmp_path):
    """The three-level reacting detonation of the GPU runner test (32 x 16 periodic, N2
    diluent, blocks of 16, regrid every 2 steps) over the composite oracle: with the
    roundoff repair after reflux over every level's leaf cells (BlockAMR.cpp:257), no step
    is rolled back.  A repair level by level before the reflux leaves a coarse trace
    species a few ulp below zero next to a fine block, which fails validation at any step
    size until the step is small enough to change nothing."""
    import amr
    import torch
    from hyperflow_gb300 import solver as S, workloads as W
    U, lvd = W.det2d(seed=6, diluent="N2", nx=32, ny=16, hot_columns=6)
    lvd = dict(lvd, periodic=(1, 1))
    tags = dict(pressure_tag=0.08, temperature_tag=0.08, density_tag=0.05)
    stepper = OracleAmr(oracle, amr, U.transpose(1, 2, 0), lvd, 16, amr.criteria(chemistry=True, **tags), 2, 1,
                        chemistry=True)

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    s = out.run_amr_case(CountingCtx(stepper), S.make_level(**lvd), torch.from_numpy(U), 2e-8, str(tmp_path), cfl=0.5,
                         output_times=[1e-8, 2e-8], max_level=2, block=16, tag_buffer=1, regrid_interval=2,
                         chemistry=True, stepper=stepper, props=props)
    assert s["completed"] and s["retries"] == 0 and s["finest_level"] == 2 and s["steps"] == 5
    summ = __import__("json").loads((tmp_path / "summary.json").read_text())
    a, b = np.array(summ["initial_conserved_integrals"]), np.array(summ["final_conserved_integrals"])
    assert abs(b[:9].sum() / a[:9].sum() - 1) < 1e-11 and abs(b[11] / a[11] - 1) < 1e-11
