"""The CPU oracle of the block-AMR composite step (oracle/amr.py) on its own: with every
level-1 block active it is the one-level run of the fine grid bit for bit, with none it
is the one-level run of the coarse grid, and with part of level 1 active it conserves
mass, momentum and energy over the leaf cells (reflux and average_down)."""
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
    assert np.array_equal(a.active, act) and np.array_equal(a.level(0), l0) and np.array_equal(a.level(1), l1)
