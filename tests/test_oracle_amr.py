"""The CPU oracle of the block-AMR composite step (oracle/amr.py) on its own: with every
block active it is the one-level run of the finest grid bit for bit (periodic, walled
and wedge/inflow domains, two and three levels), with none it is the one-level run of
the coarse grid, and with part of the hierarchy active it conserves mass, momentum and
energy over the leaf cells (reflux and average_down); regrids follow the tags, nest the
levels and conserve."""
import numpy as np
import pytest

import helpers as H


@pytest.fixture(scope="module")
def amr_oracle(oracle):
    import amr
    return amr


def one_level(oracle, U, dx, dy, dt, nsteps):
    ny, nx, _ = U.shape
    g = oracle.make_grid(nx, ny, dx, dy, periodic=(1, 1))
    Ug = oracle.fill_ghosts(g, oracle.ghosted(U))
    for _ in range(nsteps):
        Ug, dta, st, _ = oracle.strang_step(g, Ug, dt)
        assert st == 0 and dta == dt
    return Ug[2:-2, 2:-2]


def fine_dt(oracle, U1, dx, dy, cfl=0.3):
    ny, nx, _ = U1.shape
    g = oracle.make_grid(nx, ny, dx / 2, dy / 2, periodic=(1, 1))
    return oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(U1)), cfl)


def test_full_refinement_is_the_fine_run(oracle, amr_oracle):
    nx, ny, B, dx = 16, 8, 8, 1e-4
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=3)
    U0 = oracle.average_down(U1)
    dt = fine_dt(oracle, U1, dx, dx)
    a = amr_oracle.AmrOracle(U0, U1, np.ones((2 * ny // B, 2 * nx // B), np.uint8), dx, dx, B)
    for _ in range(2):
        a.step(dt)
    ref = one_level(oracle, U1, dx / 2, dx / 2, dt, 2)
    assert np.array_equal(a.level(1), ref)
    assert np.array_equal(a.level(0), oracle.average_down(a.level(1)))


def test_no_refinement_is_the_coarse_run(oracle, amr_oracle):
    nx, ny, B, dx = 16, 8, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=4)
    dt = 0.3 * oracle.cfl_dt(oracle.make_grid(nx, ny, dx, dx, periodic=(1, 1)),
                             oracle.fill_ghosts(oracle.make_grid(nx, ny, dx, dx, periodic=(1, 1)),
                                                oracle.ghosted(U0)), 1.0)
    a = amr_oracle.AmrOracle(U0, np.zeros((2 * ny, 2 * nx, U0.shape[2])), np.zeros((2 * ny // B, 2 * nx // B),
                                                                                    np.uint8), dx, dx, B)
    for _ in range(2):
        a.step(dt)
    assert np.array_equal(a.level(0), one_level(oracle, U0, dx, dx, dt, 2))


def test_partial_refinement_conserves(oracle, amr_oracle):
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=5)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=6)
    active = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    active[:, 2:5] = 1        # a band of fine blocks: coarse-fine faces on both sides
    active[1, 6] = 1          # and an isolated block (corner regions)
    a = amr_oracle.AmrOracle(U0, U1, active, dx, dx, B)
    assert len(a.regions) > 0
    dt = fine_dt(oracle, U1, dx, dx)
    t0 = a.totals()
    for _ in range(2):
        a.step(dt)
    t1 = a.totals()
    ns = U0.shape[2] - 3
    mass = t0[:ns].sum()
    assert abs(t1[:ns].sum() - mass) <= 1e-14 * mass
    for n, sc in ((ns, mass * 1000.0), (ns + 1, mass * 1000.0), (ns + 2, abs(t0[ns + 2]))):
        assert abs(t1[n] - t0[n]) <= 1e-12 * sc, n
    # the fine level moved and stays consistent with level 0 under it
    lv1 = a.level(1)
    assert not np.array_equal(lv1[:, 16:40], U1[:, 16:40])


def test_regrid_follows_a_moving_box_and_conserves(oracle, amr_oracle):
    """Box tags moving across a periodic level (8 coarse cells in 4 steps): the initial
    hierarchy holds the blocks whose grown footprint meets the box, every regrid moves
    them along, the new blocks are ConservativeInterp of level 0, and the leaf totals are
    conserved."""
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=7)
    g = oracle.make_grid(nx, ny, dx / 2, dx / 2, periodic=(1, 1))
    dt = 0.5 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(U0)), 1.0)
    crit = amr_oracle.criteria(box=(0.0004, 0.0008, -1.0, 1.0), box_only=True, velocity=(8 * dx / (4 * dt), 0.0),
                               chemistry=False)
    a = amr_oracle.AmrOracle.from_base(U0, dx, dx, B, crit, tag_buffer=1, regrid_interval=1, chemistry=False)
    # cells 4..7 tagged, grown by 1: footprints of 4 cells meet 3..8 -> blocks 0..2
    assert a.active[:, :3].all() and not a.active[:, 3:].any()
    # a new block's children average to their coarse cell
    lv0, lv1 = a.level(0), a.level(1)
    assert np.allclose(oracle.average_down(lv1[:, :24]), lv0[:, :12], rtol=1e-13, atol=0)
    t0 = a.totals()
    seen = [a.active.copy()]
    for _ in range(4):
        a.step(dt)
        seen.append(a.active.copy())
    # the box moved 0.8 mm = 8 coarse cells: the blocks followed it
    assert a.regrids == 4 and not np.array_equal(seen[0], seen[-1])
    assert seen[-1][:, 2:5].all() and not seen[-1][:, :2].any()
    t1 = a.totals()
    ns = U0.shape[2] - 3
    mass = t0[:ns].sum()
    assert abs(t1[:ns].sum() - mass) <= 1e-13 * mass
    assert abs(t1[ns + 2] - t0[ns + 2]) <= 1e-12 * abs(t0[ns + 2])


def test_regrid_twice_changes_nothing(oracle, amr_oracle):
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=8)
    crit = amr_oracle.criteria(box=(0.001, 0.002, 0.0, 0.0008), box_only=True, chemistry=False)
    a = amr_oracle.AmrOracle.from_base(U0, dx, dx, B, crit, tag_buffer=2, chemistry=False)
    act, l0, l1 = a.active.copy(), a.level(0), a.level(1)
    a.regrid()
    # (cells of inactive blocks hold ghost-frame values of the fill, not state)
    m = np.kron(act, np.ones((B, B), np.uint8)).astype(bool)
    assert np.array_equal(a.active, act) and np.array_equal(a.level(0), l0) and np.array_equal(a.level(1)[m], l1[m])


def _grid_run(oracle, g, U, dt, nsteps):
    Ug = oracle.fill_ghosts(g, oracle.ghosted(U))
    for _ in range(nsteps):
        Ug, dta, st, _ = oracle.strang_step(g, Ug, dt)
        assert st == 0 and dta == dt
    return Ug[2:-2, 2:-2]


def _coarsen(F, times):
    for _ in range(times):
        F = (((F[0::2, 0::2] + F[0::2, 1::2]) + F[1::2, 0::2]) + F[1::2, 1::2]) * 0.25
    return F


@pytest.mark.parametrize("case", ["periodic", "walls", "wedge"])
def test_three_levels_fully_refined_are_the_finest_run(oracle, amr_oracle, case):
    """Every level-1 and level-2 block active: level 2 is the one-level run of the finest
    grid bit for bit; the wall and wedge cases check that a block face is a wall face
    exactly where it lies on the domain's wall."""
    from hyperflow_gb300 import workloads as W
    nx, ny, B = 8, 4, 8
    if case == "wedge":
        _, lvd = W.wedge(nx=nx, ny=ny, length=0.004, x_tip=0.001)
        U2 = np.tile(lvd["inlet"], (4 * ny, 4 * nx, 1))
        U2 *= (1.0 + 0.05 * np.sin(np.arange(4 * nx) / 3.0))[None, :, None]  # density waves
        dx = lvd["dx"]
    else:
        dx = 1e-4
        U2 = H.smooth_field(4 * nx, 4 * ny, seed=11)
        lvd = dict(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1) if case == "periodic" else (0, 0),
                   boundary_lo=("reflecting", "reflecting"), boundary_hi=("reflecting", "reflecting"))
    dom = dict(lvd)
    U1, U0 = _coarsen(U2, 1), _coarsen(U2, 2)
    acts = [None, np.ones((2 * ny // B, 2 * nx // B), np.uint8), np.ones((4 * ny // B, 4 * nx // B), np.uint8)]
    h = amr_oracle.Hierarchy([U0, U1, U2], acts, dom, B, chemistry=(case != "wedge"))
    g2 = h.g[2]
    dt = 0.3 * oracle.cfl_dt(g2, oracle.fill_ghosts(g2, oracle.ghosted(U2)), 1.0)
    for _ in range(2):
        h.step(dt)
    ref = U2
    Ug = oracle.fill_ghosts(g2, oracle.ghosted(U2))
    for _ in range(2):
        Ug, dta, st, _ = oracle.strang_step(g2, Ug, dt, chemistry=(case != "wedge"))
        assert st == 0 and dta == dt
    ref = Ug[2:-2, 2:-2]
    assert np.array_equal(h.level(2), ref)
    assert np.array_equal(h.level(1), _coarsen(ref, 1))
    assert np.array_equal(h.level(0), _coarsen(h.level(1), 1))


def test_three_levels_partial_refinement_conserves(oracle, amr_oracle):
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=12)
    crit = amr_oracle.criteria(box=(0.0008, 0.0016, 0.0004, 0.0012), box_only=True, chemistry=False)
    dom = dict(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    h = amr_oracle.Hierarchy.from_base(U0, dom, B, crit, max_level=2, tag_buffer=1, chemistry=True)
    assert h.finest == 2 and 0 < h.acts[2].sum() < h.acts[2].size
    # proper nesting: every level-2 block's footprint grown by 2 lies in active level-1 cells
    a1 = np.kron(h.acts[1], np.ones((B, B), np.uint8)).astype(bool)
    for bj, bi in zip(*np.nonzero(h.acts[2])):
        rows = np.arange(bj * B // 2 - 2, (bj + 1) * B // 2 + 2) % a1.shape[0]
        cols = np.arange(bi * B // 2 - 2, (bi + 1) * B // 2 + 2) % a1.shape[1]
        assert a1[np.ix_(rows, cols)].all()
    g = oracle.make_grid(4 * nx, 4 * ny, dx / 4, dx / 4, periodic=(1, 1))
    dt = 0.3 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(np.kron(U0, np.ones((4, 4, 1))))), 1.0)
    t0 = h.totals()
    for _ in range(2):
        h.step(dt)
    t1 = h.totals()
    ns = U0.shape[2] - 3
    mass = t0[:ns].sum()
    assert abs(t1[:ns].sum() - mass) <= 1e-13 * mass
    assert abs(t1[ns + 2] - t0[ns + 2]) <= 1e-12 * abs(t0[ns + 2])


def test_walled_partial_refinement_conserves(oracle, amr_oracle):
    """Reflecting walls on all sides and level-1 blocks on two of them: mass and energy
    stay, the wall faces of the blocks carry no mass flux."""
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=13)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=14)
    act = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    act[0, :3] = 1      # along the bottom wall from the left wall
    act[3, 5:] = 1      # along the top wall to the right wall
    dom = dict(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
               boundary_hi=("reflecting", "reflecting"))
    h = amr_oracle.Hierarchy([U0, U1], [None, act], dom, B, chemistry=True)
    g = oracle.make_grid(2 * nx, 2 * ny, dx / 2, dx / 2)
    dt = 0.3 * oracle.cfl_dt(g, oracle.fill_ghosts(g, oracle.ghosted(U1)), 1.0)
    t0 = h.totals()
    for _ in range(2):
        h.step(dt)
    t1 = h.totals()
    ns = U0.shape[2] - 3
    mass = t0[:ns].sum()
    assert abs(t1[:ns].sum() - mass) <= 1e-13 * mass
    assert abs(t1[ns + 2] - t0[ns + 2]) <= 1e-12 * abs(t0[ns + 2])


def test_composite_repair_of_roundoff_negatives(oracle, amr_oracle):
    """repairRoundoff over the leaf cells of both levels (BlockAMR.cpp:299-334): a species a
    few ulp below zero on a level-1 block and on an uncovered level-0 cell is zeroed, the
    deficit taken from the leaf cell holding the most mass of it (value x volume, over
    both levels), so the leaf total is kept; a negative under a fine block is not a leaf
    and stays; one far below zero fails."""
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=5)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=6)
    active = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    active[:, 2:5] = 1
    a = amr_oracle.AmrOracle(U0, U1, active, dx, dx, B)
    X = [x.copy() for x in a.X]
    l0, l1 = X[0][2:-2, 2:-2], X[1][2:-2, 2:-2]
    m0, m1 = a.leaf_mask(0), a.leaf_mask(1)
    vol = [dx * dx, dx * dx / 4]

    def leaf_total(n):
        return (l0[m0][:, n].sum() * vol[0]) + (l1[m1][:, n].sum() * vol[1])

    peak = max(l0[m0][:, 5].max(), l1[m1][:, 5].max())
    l1[3, 20, 5] = -2e-16 * peak      # leaf on level 1, within 64 ulp
    l0[2, 1, 5] = -1e-16 * peak       # leaf on level 0
    l0[4, 10, 5] = -1e-3 * peak       # covered by the level-1 block over columns 8..19: not a leaf
    assert m1[3, 20] and m0[2, 1] and not m0[4, 10]
    total = leaf_total(5)
    ok, count = a.repair(X)
    assert ok and count == 2 and a.roundoff_repairs == 2
    assert l1[3, 20, 5] == 0.0 and l0[2, 1, 5] == 0.0 and l0[4, 10, 5] < 0
    assert abs(leaf_total(5) - total) <= 1e-14 * abs(total)
    l1[5, 22, 5] = -1e-3 * peak       # materially negative leaf value
    ok, _ = a.repair(X)
    assert not ok


def test_rollback_halves_like_the_one_level_run(oracle, amr_oracle):
    """Fully refined, a step 8 times the CFL step fails and is retried with half the step
    until it passes (BlockAMR.cpp:411-419): the step taken and the fine level equal the
    one-level oracle's run of the fine grid bit for bit."""
    nx, ny, B, dx = 16, 8, 8, 1e-4
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=3)
    U0 = oracle.average_down(U1)
    a = amr_oracle.AmrOracle(U0, U1, np.ones((2 * ny // B, 2 * nx // B), np.uint8), dx, dx, B, chemistry=False)
    dt = 8.0 * fine_dt(oracle, U1, dx, dx, cfl=1.0)
    h = a.step(dt)
    g = oracle.make_grid(2 * nx, 2 * ny, dx / 2, dx / 2, periodic=(1, 1))
    Ug, dta, st, _ = oracle.strang_step(g, oracle.fill_ghosts(g, oracle.ghosted(U1)), dt, chemistry=False)
    assert st == 0 and h == dta < dt and a.retries >= 1
    assert np.array_equal(a.level(1), Ug[2:-2, 2:-2])
