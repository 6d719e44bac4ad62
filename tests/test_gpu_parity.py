"""GPU parity: every kernel against the CPU oracle on the same seeded inputs.

Tolerances: EOS / HLLC / Euler stage results within 1e-12 relative (per component,
relative to that component's field maximum); ghost fill exact; chemistry within
T rel 1e-6 and Y abs 1e-8 of the oracle run at the same tolerances.
"""
import numpy as np
import pytest
import torch

import helpers as H

pytestmark = pytest.mark.gpu

TOL_FLUX = 1e-12


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# ------------------------------------------------------------------ EOS / HLLC
def test_properties_match_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    q = H.random_states(400, seed=1)
    bad = q[:8].copy()
    bad[0, 3] = -1e-12          # negative partial density
    bad[1, 0] = np.nan          # non-finite
    bad[2, :9] = 0.0            # zero density
    bad[3, 11] = -1e9           # energy far below the EOS range
    allq = np.vstack([q, bad])
    p, a, T, st = hf.properties(gpu, cuda(allq.T))
    po, ao, To, sto = oracle.properties(allq)
    st = st.cpu().numpy()
    assert np.array_equal(st, sto), (st[-8:], sto[-8:])
    ok = sto == 0
    for g, o in ((p, po), (a, ao), (T, To)):
        assert H.rel_err(g.cpu().numpy()[ok], o[ok]) < TOL_FLUX


@pytest.mark.parametrize("direction", [0, 1])
def test_hllc_matches_oracle(gpu, oracle, direction):
    import hyperflow_gb300 as hf
    n = 300
    L = H.random_states(n, seed=2)
    R = H.random_states(n, seed=3)
    # include near-identical pairs and supersonic pairs (both sides fast, same direction)
    R[:20] = L[:20] * (1 + 1e-3)
    L[20:40] = H.random_states(20, seed=4, T=(300.0, 600.0), speed=1.0)
    R[20:40] = L[20:40]
    for k in range(20, 40):
        sgn = 1.0 if k % 2 else -1.0
        for q in (L, R):
            rho = q[k, :9].sum()
            q[k, 11] += 0.5 * rho * 3000.0 ** 2
            q[k, 9 + direction] = sgn * rho * 3000.0
    pl = np.stack(oracle.properties(L)[:3])
    pr = np.stack(oracle.properties(R)[:3])
    f = hf.hllc(gpu, cuda(L.T), cuda(R.T), cuda(pl), cuda(pr), direction).cpu().numpy().T
    fo = np.array([oracle.hllc(L[k], R[k], 9 + direction, pl[:, k], pr[:, k]) for k in range(n)])
    assert H.comp_err(f, fo) < TOL_FLUX


# ------------------------------------------------------------------ ghost fill
def test_boundary_known_answers(gpu):
    """HyperFlow_V3/tests/boundary_check.cpp:15-36: 8x4 box on [-0.002, 0.006] x [0, 0.004],
    value(i,j,n) = 1000 n + 10 j + i + 1, inflow left/bottom(wedge)/top, outflow right,
    wedge tip at x = 0; exact ghost values."""
    import hyperflow_gb300 as hf
    nv = 12
    pa = hf.PatchArray(nv, 8, 4, 2)
    g = np.full((nv, 8, 12), -1e100)
    for n in range(nv):
        for j in range(4):
            for i in range(8):
                g[n, j + 2, i + 2] = 1000.0 * n + 10.0 * j + i + 1.0
    pa.data[:, :, :12] = cuda(g)
    inlet = [20000.0 + n for n in range(nv)]
    lv = hf.make_level(8, 4, 0.001, 0.001, xlo=-0.002, ylo=0.0, periodic=(0, 0),
                       boundary_lo=("inflow", "wedge"), boundary_hi=("transmissive", "inflow"),
                       inlet=inlet, wedge_start=0.0)
    hf.fill(gpu, lv, pa)
    a = pa.ghosted().cpu().numpy()
    at = lambda i, j, n: a[n, j + 2, i + 2]  # noqa: E731
    value = lambda i, j, n: 1000.0 * n + 10.0 * j + i + 1.0  # noqa: E731
    for n in range(nv):
        assert at(-1, 1, n) == inlet[n] and at(3, 4, n) == inlet[n]
        assert at(-1, -1, n) == inlet[n] and at(8, 2, n) == value(7, 2, n)
        assert at(0, -1, n) == value(0, 0, n) and at(0, -2, n) == value(0, 0, n)
        sign = -1.0 if n == 10 else 1.0
        assert at(3, -1, n) == sign * value(3, 0, n) and at(3, -2, n) == sign * value(3, 1, n)


BC_CASES = [
    ((0, 0), ("reflecting", "reflecting"), ("transmissive", "reflecting")),
    ((0, 1), ("reflecting", "reflecting"), ("transmissive", "reflecting")),
    ((1, 1), ("reflecting", "reflecting"), ("reflecting", "reflecting")),
    ((1, 0), ("transmissive", "inflow"), ("transmissive", "reflecting")),
    ((0, 0), ("inflow", "wedge"), ("transmissive", "inflow")),
    ((0, 0), ("transmissive", "transmissive"), ("inflow", "transmissive")),
]


@pytest.mark.parametrize("case", range(len(BC_CASES)))
def test_fill_matches_oracle(gpu, oracle, case):
    import hyperflow_gb300 as hf
    periodic, lo, hi = BC_CASES[case]
    nx, ny = 13, 7
    rng = np.random.default_rng(case)
    interior = rng.uniform(0.5, 2.0, (ny, nx, 12))
    inlet = rng.uniform(3.0, 4.0, 12)
    Ug = oracle.ghosted(interior)
    kinds = {"reflecting": 0, "transmissive": 1, "inflow": 2, "wedge": 3}
    g = oracle.make_grid(nx, ny, 1e-3, 1e-3, xlo=-0.004, periodic=periodic, bc_lo=[kinds[k] for k in lo],
                         bc_hi=[kinds[k] for k in hi], inlet=inlet, wedge_start=0.0)
    ref = oracle.fill_ghosts(g, Ug.copy())
    pa = H.to_patch(gpu, Ug)
    lv = hf.make_level(nx, ny, 1e-3, 1e-3, xlo=-0.004, periodic=periodic, boundary_lo=lo, boundary_hi=hi,
                       inlet=inlet, wedge_start=0.0)
    hf.fill(gpu, lv, pa)
    got = H.from_patch(pa)
    assert np.array_equal(got, ref)


# ------------------------------------------------------------------ Euler stage / flow
STAGE_CASES = [
    ((0, 1), ("reflecting", "reflecting"), ("transmissive", "reflecting")),
    ((0, 0), ("reflecting", "reflecting"), ("transmissive", "reflecting")),
    ((1, 1), ("reflecting", "reflecting"), ("reflecting", "reflecting")),
    ((0, 0), ("inflow", "wedge"), ("transmissive", "inflow")),
]


def _stage_setup(oracle, case, nx=37, ny=19, seed=0):
    periodic, lo, hi = STAGE_CASES[case]
    field = H.smooth_field(nx, ny, seed=seed)
    inlet = field[ny // 2, 0]
    kinds = {"reflecting": 0, "transmissive": 1, "inflow": 2, "wedge": 3}
    dx = 1e-4
    g = oracle.make_grid(nx, ny, dx, dx, xlo=-0.001, periodic=periodic, bc_lo=[kinds[k] for k in lo],
                         bc_hi=[kinds[k] for k in hi], inlet=inlet, wedge_start=0.0)
    Ug = oracle.fill_ghosts(g, oracle.ghosted(field))
    h = 0.3 * oracle.cfl_dt(g, Ug, 1.0)
    return periodic, lo, hi, field, inlet, g, Ug, h, dx


@pytest.mark.parametrize("form", ["plain", "fused"])
@pytest.mark.parametrize("case", range(len(STAGE_CASES)))
@pytest.mark.parametrize("first_order", [False, True])
def test_euler_stage_matches_oracle(gpu, oracle, form, case, first_order):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    periodic, lo, hi, field, inlet, g, Ug, h, dx = _stage_setup(oracle, case)
    out, fx, fy, st = oracle.euler_stage(g, Ug, h, first_order)
    assert st == 0
    lv = hf.make_level(g.nx, g.ny, dx, dx, xlo=-0.001, periodic=periodic, boundary_lo=lo, boundary_hi=hi,
                       inlet=inlet, wedge_start=0.0)
    pin = H.to_patch(gpu, Ug if form == "plain" else oracle.ghosted(field))
    pout = pin.like()
    if form == "plain":
        gfx, gfy = hf.euler_stage(gpu, lv, pin, pout, h, first_order, form=L.HF_FLUX_PLAIN, faces=True)
        assert H.comp_err(gfx.cpu().numpy().transpose(1, 2, 0), fx) < TOL_FLUX
        assert H.comp_err(gfy.cpu().numpy().transpose(1, 2, 0), fy) < TOL_FLUX
    else:
        hf.euler_stage(gpu, lv, pin, pout, h, first_order, form=L.HF_FLUX_FUSED)
    got = H.from_patch(pout)[2:-2, 2:-2]
    assert H.comp_err(got, out[2:-2, 2:-2]) < TOL_FLUX


@pytest.mark.parametrize("form", ["plain", "fused"])
def test_heun_flow_matches_oracle(gpu, oracle, form):
    """flow(h): two stages and the Heun combine (BlockAMR.cpp:266-269)."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    periodic, lo, hi, field, inlet, g, Ug, h, dx = _stage_setup(oracle, 0, seed=5)
    ref, st, _ = oracle.flow(g, Ug, h)
    assert st == 0
    lv = hf.make_level(g.nx, g.ny, dx, dx, xlo=-0.001, periodic=periodic, boundary_lo=lo, boundary_hi=hi,
                       inlet=inlet, wedge_start=0.0)
    f = L.HF_FLUX_PLAIN if form == "plain" else L.HF_FLUX_FUSED
    u0 = H.to_patch(gpu, oracle.ghosted(field))
    u1, u2 = u0.like(), u0.like()
    if form == "plain":
        hf.fill(gpu, lv, u0)
    hf.euler_stage(gpu, lv, u0, u1, h, form=f)
    if form == "plain":
        hf.fill(gpu, lv, u1)
    hf.euler_stage(gpu, lv, u1, u2, h, u_old=u0, form=f)
    got = H.from_patch(u2)[2:-2, 2:-2]
    assert H.comp_err(got, ref[2:-2, 2:-2]) < TOL_FLUX


def test_cfl_matches_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    periodic, lo, hi, field, inlet, g, Ug, h, dx = _stage_setup(oracle, 0, seed=7)
    lv = hf.make_level(g.nx, g.ny, dx, dx, periodic=periodic, boundary_lo=lo, boundary_hi=hi, inlet=inlet)
    dt = hf.cfl_dt(gpu, lv, H.to_patch(gpu, Ug), 0.5)
    assert abs(dt - oracle.cfl_dt(g, Ug, 0.5)) / dt < 1e-13


# ------------------------------------------------------------------ interpolation
def test_conservative_interp_matches_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    nx, ny = 6, 5
    coarse = H.smooth_field(nx + 2, ny + 2, seed=11)  # includes a 1-cell ring used as neighbours
    # force a steep feature so that some theta halving happens
    coarse[3, 3, :9] *= 40.0
    c = hf.PatchArray(12, nx, ny, 2, ilo=0, jlo=0)
    gc = np.zeros((12, ny + 4, nx + 4))
    gc[:, 1:ny + 3, 1:nx + 3] = coarse.transpose(2, 0, 1)
    c.data[:, :, :nx + 4] = cuda(gc)
    f = hf.PatchArray(12, 2 * nx, 2 * ny, 2, ilo=0, jlo=0)
    hf.ConservativeInterp(gpu).interp(c, f, (0, 0, 2 * nx - 1, 2 * ny - 1))
    got = f.interior().cpu().numpy()
    for cj in range(ny):
        for ci in range(nx):
            q = coarse[cj + 1, ci + 1]
            ch, _ = oracle.interp_cell(q, coarse[cj + 1, ci], coarse[cj + 1, ci + 2], coarse[cj, ci + 1],
                                       coarse[cj + 2, ci + 1])
            for b in range(2):
                for a in range(2):
                    g = got[:, 2 * cj + b, 2 * ci + a]
                    assert H.rel_err(g, ch[b * 2 + a]) < 1e-13


# ------------------------------------------------------------------ chemistry
def _chem_cells(n, seed):
    from hyperflow_gb300 import workloads as W
    U, dt = W.chem_batch(n, seed=seed, diluent="N2")
    return U, dt


def _compare_chem(got, ref):
    """T rel and Y abs errors between AoS state batches."""
    import oracle as o
    Tg = o.properties(got)[2]
    Tr = o.properties(ref)[2]
    rho = ref[:, :9].sum(1)
    t_err = float(np.max(np.abs(Tg - Tr) / Tr))
    y_err = float(np.max(np.abs(got[:, :9] - ref[:, :9]) / rho[:, None]))
    return t_err, y_err


@pytest.mark.parametrize("form", ["plain", "persistent", "batched"])
def test_chemistry_matches_oracle(gpu, oracle, form):
    import hyperflow_gb300 as hf
    U, dt = _chem_cells(96, seed=3)
    ref, bad, steps = oracle.chem_batch(U.T, 0.0, dt_cell=dt)
    assert bad == -1
    field = cuda(U)
    hf.ChemistryBatch(gpu, form).advance(field, 0.0, dt_cell=cuda(dt))
    got = field.cpu().numpy().T
    t_err, y_err = _compare_chem(got, ref)
    assert t_err < 1e-6 and y_err < 1e-8, (t_err, y_err)


def test_chemistry_forms_identical(gpu):
    """Each cell runs the same step sequence in both forms: bitwise equal results."""
    import hyperflow_gb300 as hf
    U, dt = _chem_cells(300, seed=4)
    a, b = cuda(U), cuda(U)
    hf.ChemistryBatch(gpu, "plain").advance(a, 0.0, dt_cell=cuda(dt))
    hf.ChemistryBatch(gpu, "persistent").advance(b, 0.0, dt_cell=cuda(dt))
    assert torch.equal(a, b)


def test_batched_history_and_screen(gpu, oracle):
    """Batched form over two consecutive intervals (warm-started step sizes, cost-ordered
    queue) on a mix of frozen cold cells and igniting hot cells, against the oracle."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0, 0, 0, 0, 0, 0, 3.76]) / 6.76
    cells = [M.primitive(298.0, 101325.0, X=X, ns=9), M.primitive(3000.0, 40 * 101325.0, X=X, ns=9),
             M.primitive(1100.0, 2e5, X=X, ns=9), M.primitive(2400.0, 1e5, X=X, ns=9)]
    U = np.array([cells[k % 4] for k in range(64)])
    ref = U.copy()
    field = cuda(U.T.copy())
    cb = hf.ChemistryBatch(gpu, "batched")
    for _ in range(2):
        ref, bad, _ = oracle.chem_batch(ref, 1e-8)
        assert bad == -1
        cb.advance(field, 1e-8)
    t_err, y_err = _compare_chem(field.cpu().numpy().T, ref)
    assert t_err < 1e-6 and y_err < 1e-8, (t_err, y_err)
    cost = cb.history[1].cpu().numpy()
    assert cost[0] == 0 and cost[1] > 10   # cold cell screened, hot cell integrated


def test_chemistry_zero_dimensional_against_tight(gpu, oracle):
    """validate.py:140-159 analogue: 1500 K, 5 atm stoichiometric H2/air over 2e-7 s;
    rtol 1e-8/atol 1e-15 against the rtol 1e-12 oracle: T rel < 1e-7, Y abs < 1e-8."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0, 0, 0, 0, 0, 0, 3.76]) / 6.76
    q = M.primitive(1500.0, 5 * 101325.0, X=X, ns=9)
    U = np.tile(q, (8, 1))
    tight, bad, _ = oracle.chem_batch(U, 2e-7, rtol=1e-12, atol=1e-20)
    assert bad == -1
    field = cuda(U.T.copy())
    hf.ChemistryBatch(gpu, "persistent").advance(field, 2e-7)
    t_err, y_err = _compare_chem(field.cpu().numpy().T, tight)
    assert t_err < 1e-7 and y_err < 1e-8


def test_chemistry_all_or_nothing(gpu):
    """chemistry_batch.cpp:40-49: on failure the field is unchanged and the lowest
    failing index is reported."""
    import hyperflow_gb300 as hf
    U, dt = _chem_cells(64, seed=5)
    U[:, 17] = U[:, 3]
    U[4, 17] = -1.0   # negative partial density: properties() throws for cell 17
    U[4, 40] = -1.0
    field = cuda(U)
    before = field.clone()
    with pytest.raises(RuntimeError) as e:
        hf.ChemistryBatch(gpu, "persistent").advance(field, 1e-7)
    assert e.value.first_failed == 17
    assert torch.equal(field, before)


# ------------------------------------------------------------------ full step
def test_strang_step_matches_oracle(gpu, oracle):
    """One Strang step (flow, react, flow) on a small 2D detonation (N2 diluent)."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=1, diluent="N2", nx=48, ny=12, hot_columns=6)
    lv = hf.make_level(**lvd)
    g = oracle.make_grid(48, 12, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    dt = oracle.cfl_dt(g, Ug, 0.5)
    ref, dt_acc, st, _ = oracle.strang_step(g, Ug, dt)
    assert st == 0 and dt_acc == dt
    for flux, chem in (("plain", "plain"), ("fused", "persistent")):
        s = hf.Stepper(gpu, lv, cuda(U), flux=flux, chem=chem)
        d = s.step(dt=dt)
        assert d == dt
        got = s.state().cpu().numpy().transpose(1, 2, 0)
        t_err, y_err = _compare_chem(got.reshape(-1, 12), ref[2:-2, 2:-2].reshape(-1, 12))
        assert t_err < 1e-6 and y_err < 1e-8, (flux, t_err, y_err)
        s.close()


@pytest.mark.parametrize("flux,chem", [("fused", "batched"), ("plain", "batched"), ("plain", "plain")])
def test_graph_step_equals_host_step(gpu, flux, chem):
    """The CUDA-graph Strang step (device dt, one status read per step) gives the same
    states, bit for bit, as the host-controlled path on the same inputs, with either
    chemistry form inside the graph."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=2, diluent="N2", nx=96, ny=24, hot_columns=8)
    lv = hf.make_level(**lvd)
    a = hf.Stepper(gpu, lv, cuda(U), flux=flux, chem=chem)
    b = hf.Stepper(gpu, lv, cuda(U), flux=flux, chem=chem)
    b.set_graph(False)
    for _ in range(3):
        da = a.step(cfl=0.5)
        db = b.step(cfl=0.5)
        assert da == db
    assert a.stats()["graph_steps"] == 3 and b.stats()["graph_steps"] == 0
    assert torch.equal(a.state(), b.state())
    assert a.time == b.time


def test_graph_step_phase_flags(gpu):
    """hf_stepper_graph_info: an accepted graph step has no flag at any of its four phase
    boundaries; a graph step at 8 times the CFL number fails on the device (and is re-run
    with host control), and its flags only accumulate from phase to phase up to the
    step's final flags."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=2, diluent="N2", nx=96, ny=24, hot_columns=8)
    lv = hf.make_level(**lvd)
    s = hf.Stepper(gpu, lv, cuda(U), flux="plain", chem="batched")
    s.step(cfl=0.5)
    info = s.graph_info()
    assert s.stats()["graph_steps"] == 1
    assert info == {"last_flags": 0, "capture_error": 0, "phase_flags": [0, 0, 0, 0]}
    s.step(cfl=8.0)
    info = s.graph_info()
    assert s.stats()["host_steps"] == 1 and info["capture_error"] == 0
    ph = info["phase_flags"]
    assert info["last_flags"] != 0 and ph[3] == info["last_flags"]
    assert all((ph[k] & ph[k + 1]) == ph[k] for k in range(3))
    s.close()


@pytest.mark.parametrize("flux,cfl,chem", [("fused", 0.5, "batched"), ("fused", 8.0, "batched"),
                                          ("plain", 0.5, "batched"), ("plain", 8.0, "batched"),
                                          ("plain", 0.5, "plain"), ("plain", 8.0, "plain")])
def test_device_resident_run_equals_steps(gpu, flux, cfl, chem):
    """hf_stepper_run (graph steps launched back to back, one record read per batch)
    gives the states, times and step kinds of the same number of step() calls.  At CFL
    8 graph steps fail: the run stops on the device at the failed step and re-runs it
    with host control (rollback, dt halving), like step() does."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=3, diluent="N2", nx=96, ny=24, hot_columns=8)
    lv = hf.make_level(**lvd)
    a = hf.Stepper(gpu, lv, cuda(U), flux=flux, chem=chem)
    b = hf.Stepper(gpu, lv, cuda(U), flux=flux, chem=chem)
    assert a.run(5, cfl=cfl) == 5
    for _ in range(5):
        b.step(cfl=cfl)
    assert torch.equal(a.state(), b.state())
    assert a.time == b.time
    assert a.stats() == b.stats()
    if cfl > 1:
        assert a.stats()["host_steps"] > 0
    else:
        assert a.stats()["graph_steps"] == 5
