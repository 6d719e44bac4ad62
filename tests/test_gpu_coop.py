"""The batched chemistry's cooperative phase (hyperflow_gb300/csrc/hf_chem_coop.cuh), set
on here (hf_set_chem_tuning): cells whose previous call took at least 31 step attempts
are integrated by groups of 8 lanes,
the rest one per lane.  Results stay within the chemistry parity bar against the oracle
(T relative 1e-6, Y absolute 1e-8 of the cell's density), with the file's 9 species and
with the inert AR extension, in a chemistry batch and inside the stepper's graph steps."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def cooperative(gpu):
    """The cooperative phase for cells of at least 31 attempts (off by default)."""
    from hyperflow_gb300 import tune
    before = tune.get_chem_tuning(gpu)
    tune.set_chem_tuning(gpu, 0, 5)
    yield
    tune.set_chem_tuning(gpu, *before)


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def errors(oracle, got, ref, ns):
    Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
    rho = ref[:, :ns].sum(1)
    return float(np.max(np.abs(Tg - Tr) / Tr)), float(np.max(np.abs(got[:, :ns] - ref[:, :ns]) / rho[:, None]))


@pytest.mark.parametrize("ns", [9, 10])
def test_cooperative_cells_match_oracle(gpu, oracle, ns):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    ctx = gpu if ns == 9 else hf.Context("H2_Li+AR")
    U, dt = W.chem_batch(1024, seed=21, diluent="N2" if ns == 9 else "AR")
    cb = hf.ChemistryBatch(ctx, "batched")
    first = cuda(U)
    cb.advance(first, 0.0, dt_cell=cuda(dt))  # one cell per lane; records each cell's attempts
    cost = cb.history[1].cpu().numpy()
    assert (cost >= 31).sum() >= 8
    c0 = ctx.counters()["chem_coop_cells"]
    second = cuda(U)
    cb.advance(second, 0.0, dt_cell=cuda(dt))  # the costliest cells in groups of 8 lanes
    ncoop = ctx.counters()["chem_coop_cells"] - c0
    # whole cost buckets from the top, at most 4 cells per warp of the launch (16 blocks of 2 warps)
    assert 0 < ncoop <= 16 * 2 * 4
    try:
        oracle.set_species(ns)
        ref, bad, _ = oracle.chem_batch(U.T, 0.0, dt_cell=dt)
        assert bad == -1
        for got in (first, second):
            t_err, y_err = errors(oracle, got.cpu().numpy().T, ref, ns)
            assert t_err < 1e-6 and y_err < 1e-8, (t_err, y_err)
    finally:
        oracle.set_species(9)


def test_graph_steps_with_cooperative_chemistry_match_oracle(gpu, oracle):
    """Four CFL Strang steps of a small detonation through the stepper's graph path with
    the batched chemistry (cooperative from the second step on, where the hot band's
    igniting cells took many attempts) against the oracle's steps of the same sizes."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=4, diluent="N2", nx=64, ny=16, hot_columns=8)
    lv = hf.make_level(**lvd)
    s = hf.Stepper(gpu, lv, cuda(U), flux="plain", chem="batched")
    g = oracle.make_grid(64, 16, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    c0 = gpu.counters()["chem_coop_cells"]
    for _ in range(4):
        dt = s.step(cfl=0.5)
        Ug, dta, st, _ = oracle.strang_step(g, Ug, dt)
        assert st == 0 and dta == dt
    assert gpu.counters()["chem_coop_cells"] > c0
    assert s.stats()["graph_steps"] == 4
    got = s.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, 12)
    t_err, y_err = errors(oracle, got, Ug[2:-2, 2:-2].reshape(-1, 12), 9)
    assert t_err < 1e-6 and y_err < 1e-8, (t_err, y_err)
    s.close()
