"""The CPU oracle against the reference's known answers and against identities.

The only exact known-answer vectors the reference holds for this path are the
ghost values of HyperFlow_V3/tests/boundary_check.cpp.  The thermo/kinetics
restatement of Cantera (absent here) is checked by identities and by the tolerances
of the reference's own tests (validate.py:140-159, docs/amr_checks.json) in this
file, and against the reference's recorded run outcomes in test_oracle_cases.py.
"""
import numpy as np

import helpers as H


def test_boundary_known_answers(oracle):
    """boundary_check.cpp:15-36, exact."""
    nv = 12
    interior = np.zeros((4, 8, nv))
    for n in range(nv):
        for j in range(4):
            for i in range(8):
                interior[j, i, n] = 1000.0 * n + 10.0 * j + i + 1.0
    U = oracle.ghosted(interior)
    U[np.isnan(U)] = -1e100
    inlet = [20000.0 + n for n in range(nv)]
    g = oracle.make_grid(8, 4, 0.001, 0.001, xlo=-0.002, periodic=(0, 0), bc_lo=(2, 3), bc_hi=(1, 2),
                         inlet=inlet, wedge_start=0.0)
    a = oracle.fill_ghosts(g, U)
    at = lambda i, j, n: a[j + 2, i + 2, n]  # noqa: E731
    value = lambda i, j, n: 1000.0 * n + 10.0 * j + i + 1.0  # noqa: E731
    for n in range(nv):
        assert at(-1, 1, n) == inlet[n] and at(3, 4, n) == inlet[n]
        assert at(-1, -1, n) == inlet[n] and at(8, 2, n) == value(7, 2, n)
        assert at(0, -1, n) == value(0, 0, n) and at(0, -2, n) == value(0, 0, n)
        sign = -1.0 if n == 10 else 1.0
        assert at(3, -1, n) == sign * value(3, 0, n) and at(3, -2, n) == sign * value(3, 1, n)


def test_rodas4_fourth_order(oracle):
    """Rodas4 coefficients: global error ratio ~16 per step halving on a nonlinear
    system with a closed-form solution."""
    y0 = np.array([0.3, 0.1])
    r0, th0 = np.hypot(*y0), np.arctan2(y0[1], y0[0])
    r = 1 / np.sqrt(1 + (1 / r0 ** 2 - 1) * np.exp(-2.0))
    exact = np.array([r * np.cos(th0 + 1), r * np.sin(th0 + 1)])
    errs = [np.max(np.abs(oracle.rodas4_circle(y0, 1.0, n) - exact)) for n in (10, 20, 40, 80)]
    orders = [np.log2(errs[k] / errs[k + 1]) for k in range(3)]
    assert all(3.8 < o < 4.3 for o in orders), orders


def test_uv_round_trip(oracle):
    """T -> e(T) -> properties() recovers T to rounding."""
    from hyperflow_gb300 import mechanism as M
    rng = np.random.default_rng(0)
    for T in np.concatenate([rng.uniform(250, 4000, 40), [999.999, 1000.0, 1000.001]]):
        X = rng.uniform(0, 1, 9)
        q = M.primitive(T, 2e5, X=X / X.sum(), u=100.0, ns=9)
        p, a, Tq, st = oracle.properties(q)
        assert st[0] == 0 and abs(Tq[0] - T) / T < 1e-13


def test_nasa_continuity(oracle):
    """h/RT and cp/R of each species nearly continuous at T_mid (data property)."""
    lo = oracle.species_thermo(1000.0)
    hi = oracle.species_thermo(1000.0 * (1 + 1e-12))
    assert np.max(np.abs(lo[1] - hi[1]) / np.abs(lo[1])) < 1e-3
    assert np.max(np.abs(lo[0] - hi[0]) / np.abs(lo[0])) < 1e-2


def test_element_conservation(oracle):
    """Net production conserves H, O, N atoms to rounding."""
    elem = np.array([[2, 0, 0], [0, 2, 0], [2, 1, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [1, 2, 0], [2, 2, 0],
                     [0, 0, 2]], dtype=float)
    rng = np.random.default_rng(1)
    for _ in range(20):
        C = rng.uniform(0, 1e-2, 9)
        T = rng.uniform(600, 3000)
        w = oracle.net_production(T, C)
        scale = np.max(np.abs(w)) + 1e-300
        assert np.max(np.abs(elem.T @ w)) / scale < 1e-12


def test_detailed_balance_at_equilibrium(oracle):
    """Integrate a closed cell to equilibrium: every reversible reaction balances,
    which checks Kc (Gibbs energies, units, p0) of all 21 reactions."""
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0, 0, 0, 0, 0, 0, 3.76])
    q = M.primitive(2500.0, 101325.0, X=X / X.sum(), ns=9)
    u, st, _ = oracle.chem_advance(q, 1e-2, rtol=1e-12, atol=1e-25, max_steps=200000)
    assert st == 0
    p, a, T, _ = oracle.properties(u)
    C = u[:9] / oracle.molecular_weights()
    kf, kr, qf, qr = oracle.progress(T[0], C)
    rel = np.abs(qf - qr) / np.maximum(qf, qr)
    assert np.max(rel) < 1e-6, rel


def test_jacobian_analytic_vs_fd(oracle):
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0.1, 0.01, 0.01, 0.02, 0.001, 0.001, 3.76])
    for T in (900.0, 1500.0, 2800.0):
        q = M.primitive(T, 3e5, X=X / X.sum(), ns=9)
        rho = q[:9].sum()
        e = q[11] / rho
        y = q[:8] / rho
        Ja, _ = oracle.chem_jac(rho, e, y, T)
        Jf, _ = oracle.chem_jac(rho, e, y, T, fd=True)
        assert np.max(np.abs(Ja - Jf)) / np.max(np.abs(Ja)) < 1e-5


def test_zero_dimensional_against_tight(oracle):
    """validate.py:140-159 tolerances: rtol 1e-8 vs the rtol 1e-12 oracle."""
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0, 0, 0, 0, 0, 0, 3.76])
    q = M.primitive(1500.0, 5 * 101325.0, X=X / X.sum(), ns=9)
    a, sa, _ = oracle.chem_advance(q, 2e-7)
    b, sb, _ = oracle.chem_advance(q, 2e-7, rtol=1e-12, atol=1e-20)
    assert sa == 0 and sb == 0
    Ta, Tb = oracle.properties(a)[2][0], oracle.properties(b)[2][0]
    assert abs(Ta - Tb) / Tb < 1e-7
    assert np.max(np.abs(a[:9] - b[:9])) / a[:9].sum() < 1e-8


def test_batch_thread_invariance_and_failure(oracle):
    """chemistry_parallel (validate.py:163-170): 1 vs 4 threads bit-identical;
    all-or-nothing with the lowest failing index."""
    from hyperflow_gb300 import workloads as W
    U, dt = W.chem_batch(64, seed=2, diluent="N2")
    a, ba, _ = oracle.chem_batch(U.T, 0.0, dt_cell=dt, threads=1)
    b, bb, _ = oracle.chem_batch(U.T, 0.0, dt_cell=dt, threads=4)
    assert ba == bb == -1 and np.array_equal(a, b)
    V = U.T.copy()
    V[9, 2] = -1.0
    V[30, 2] = -1.0
    c, bc, _ = oracle.chem_batch(V, 1e-7)
    assert bc == 9 and np.array_equal(c, V)


def test_flow_conserves_periodic(oracle):
    """Periodic flow: mass and energy sums conserved to rounding (uniform_local_amr analogue)."""
    field = H.smooth_field(24, 16, seed=3)
    g = oracle.make_grid(24, 16, 1e-4, 1e-4, periodic=(1, 1))
    Ug = oracle.ghosted(field)
    dt = oracle.cfl_dt(g, Ug, 0.5)
    out, st, _ = oracle.flow(g, Ug, dt)
    assert st == 0
    a, b = field.reshape(-1, 12), out[2:-2, 2:-2].reshape(-1, 12)
    assert abs(b[:, :9].sum() - a[:, :9].sum()) / a[:, :9].sum() < 1e-13
    assert abs(b[:, 11].sum() - a[:, 11].sum()) / np.abs(a[:, 11]).sum() < 1e-13


def test_uniform_state_stays_uniform(oracle):
    """uniform_local_amr (validate.py:91-102): a uniform state stays uniform to 1e-12
    under flow and reflecting walls."""
    from hyperflow_gb300 import mechanism as M
    X = np.array([2.0, 1.0, 0, 0, 0, 0, 0, 0, 3.76])
    q = M.primitive(300.0, 101325.0, X=X / X.sum(), ns=9)
    field = np.tile(q, (8, 10, 1))
    g = oracle.make_grid(10, 8, 1e-3, 1e-3, periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0))
    Ug = oracle.ghosted(field)
    out, st, _ = oracle.flow(g, Ug, 1e-7)
    assert st == 0
    dev = np.max(np.abs(out[2:-2, 2:-2] - field) / np.maximum(np.abs(field), 1.0))
    assert dev < 1e-12


def test_transpose_symmetry(oracle):
    """blast2d transpose symmetry (validate.py:121-138): x/y swap commutes with a step."""
    field = H.smooth_field(12, 12, seed=4)
    field = 0.5 * (field + field.transpose(1, 0, 2)[:, :, [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 9, 11]])
    g = oracle.make_grid(12, 12, 1e-4, 1e-4, periodic=(0, 0), bc_lo=(0, 0), bc_hi=(0, 0))
    out, st, _ = oracle.flow(g, oracle.ghosted(field), 2e-9)
    assert st == 0
    o = out[2:-2, 2:-2]
    ot = o.transpose(1, 0, 2)[:, :, [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 9, 11]]
    assert np.max(np.abs(o - ot) / np.maximum(np.abs(o), 1e-30)) < 1e-12


def test_hot_band_step_runs(oracle):
    """A Strang step of the detonation workload (small) completes without retries."""
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=0, diluent="N2", nx=24, ny=4, hot_columns=3)
    g = oracle.make_grid(24, 4, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    dt = oracle.cfl_dt(g, Ug, 0.5)
    out, dta, st, stats = oracle.strang_step(g, Ug, dt)
    assert st == 0 and stats.retries == 0


def test_reflux_makes_composite_update_conservative(oracle):
    """With arbitrary face fluxes on a periodic coarse level and two fine boxes, the
    composite sum (uncovered coarse cells + fine cells) of a flux-divergence update is
    conserved only once the coarse cells next to the fine boxes are refluxed."""
    rng = np.random.default_rng(5)
    nxc, nyc, nv = 12, 10, 12
    dxc, dyc, h = 2e-4, 1e-4, 1e-8
    Uc = rng.uniform(1, 2, (nyc, nxc, nv))
    fxc = rng.normal(size=(nyc, nxc + 1, nv))
    fxc[:, -1] = fxc[:, 0]   # periodic: the domain's two x faces are one face
    fyc = rng.normal(size=(nyc + 1, nxc, nv))
    fyc[-1] = fyc[0]
    boxes = [(4, 4, 9, 9), (16, 0, 23, 3)]
    cover = np.zeros((nyc, nxc), bool)
    fine_old, fine_new, fxs, fys = [], [], [], []
    for (i0, j0, i1, j1) in boxes:
        cover[j0 // 2:(j1 + 1) // 2, i0 // 2:(i1 + 1) // 2] = True
        nxf, nyf = i1 - i0 + 1, j1 - j0 + 1
        fx = rng.normal(size=(nyf, nxf + 1, nv))
        fy = rng.normal(size=(nyf + 1, nxf, nv))
        uf = rng.uniform(1, 2, (nyf, nxf, nv))
        fine_old.append(uf)
        fine_new.append(uf - h / (dxc / 2) * (fx[:, 1:] - fx[:, :-1]) - h / (dyc / 2) * (fy[1:] - fy[:-1]))
        fxs.append(fx)
        fys.append(fy)
    new_c = Uc - h / dxc * (fxc[:, 1:] - fxc[:, :-1]) - h / dyc * (fyc[1:] - fyc[:-1])
    refl = oracle.reflux(new_c, fxc, fyc, boxes, fxs, fys, h, dxc, dyc, periodic=(1, 1))
    vc, vf = dxc * dyc, dxc * dyc / 4

    def composite(c, fs):
        return c[~cover].sum(0) * vc + sum(f.sum((0, 1)) for f in fs) * vf

    before = composite(Uc, fine_old)
    assert np.max(np.abs(composite(new_c, fine_new) - before)) > 1e-12 * np.max(np.abs(before))
    assert np.max(np.abs(composite(refl, fine_new) - before)) < 1e-13 * np.max(np.abs(before))


def test_sensitivity_fd_frozen_and_adaptive_agree(oracle):
    # d(ignition delay)/d ln(multiplier_r) of H2/air cells by central differences
    # (step 1e-6): replaying the unperturbed accepted steps (the map a discrete adjoint
    # differentiates) and re-running the adaptive integrator give the same derivative
    # to far better than the 1e-5 bar of the adjoint checks
    from hyperflow_gb300 import workloads as W
    U = W.ignition_batch(4, seed=1).T.copy()
    J, Gf, bad = oracle.chem_sens_fd(U, 1e-6, 40, "ignition_delay", frozen=True)
    assert bad == -1
    _, Ga, _ = oracle.chem_sens_fd(U, 1e-6, 40, "ignition_delay", frozen=False)
    ok = ~np.isnan(J)
    assert ok.sum() >= 2
    scale = np.abs(Gf[ok]).max(1, keepdims=True)
    assert np.max(np.abs(Gf[ok] - Ga[ok]) / scale) < 1e-6
    # H + O2 <=> O + OH dominates and shortens the delay
    assert np.all(np.argmax(np.abs(Gf[ok]), 1) == 0) and np.all(Gf[ok][:, 0] < 0)


def test_frozen_run_replay(oracle):
    # a recorded run of Strang steps replays bit for bit with its chemistry step
    # sequences frozen, and a rate multiplier changes the replayed result smoothly
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det1d(diluent="N2", nx=40)
    g = oracle.make_grid(40, 2, lvd["dx"], lvd["dy"], periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    V, dts = Ug.copy(), []
    for _ in range(6):
        dt = oracle.cfl_dt(g, V, 0.5)
        dts.append(dt)
        V, dta, st, _ = oracle.strang_step(g, V, dt)
        assert st == 0 and dta == dt
    fr = oracle.FrozenRun(g, Ug, dts)
    try:
        assert np.array_equal(fr.U[2:-2, 2:-2], V[2:-2, 2:-2])
        assert np.array_equal(fr.replay(Ug)[2:-2, 2:-2], V[2:-2, 2:-2])
        m = np.ones(21)
        m[0] = np.exp(1e-6)
        oracle.set_rate_mult(m)
        try:
            W1 = fr.replay(Ug)[2:-2, 2:-2]
        finally:
            oracle.set_rate_mult(None)
        d = np.abs(W1 - V[2:-2, 2:-2]).max()
        assert 0 < d < 1e-3 * np.abs(V[2:-2, 2:-2]).max()
    finally:
        fr.close()


def test_threaded_flux_loops_bitwise_equal(oracle):
    # the OpenMP flux/update/validation loops (CPU baseline) give the serial loops' bits
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=1, diluent="N2", nx=64, ny=8, hot_columns=8)
    g = oracle.make_grid(64, 8, lvd["dx"], lvd["dy"], periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0),
                         inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    dt = oracle.cfl_dt(g, Ug, 0.5)
    out = []
    for ft in (1, 4):
        oracle.set_flux_threads(ft)
        try:
            V, dta, st, _ = oracle.strang_step(g, Ug, dt, chemistry=False)
        finally:
            oracle.set_flux_threads(1)
        assert st == 0
        out.append(V)
    assert np.array_equal(out[0], out[1])
