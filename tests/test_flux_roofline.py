"""The flux path's roofline inputs: the oracle's counted FP64 flops of a face, a cell
update and a Heun combine (oracle.flux_flops), and the bench's per-step arithmetic
(bench.flux_roofline)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.join(os.path.dirname(__file__), "..")


@pytest.fixture(scope="module")
def oracle10():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    oracle.set_species(10)
    yield oracle
    oracle.set_species(9)


def stencil():
    from hyperflow_gb300 import workloads as W
    U, _ = W.det2d(seed=0, diluent="AR", nx=256, ny=4)
    return U[:, 0, 128:132].T.copy()


def test_counts_follow_the_newton_iterations(oracle10):
    a = oracle10.flux_flops(stencil(), 0, 3)
    b = oracle10.flux_flops(stencil(), 0, 4)
    per_solve = b["cell"] - a["cell"]       # one EOS solve per cell update (validation)
    assert per_solve > 0
    assert b["face"] - a["face"] == 2 * per_solve  # two EOS solves per face (L and R)
    assert a["combine"] == b["combine"] == 3 * 13  # 0.5 a + 0.5 b per component
    assert a["face_transcendental"] == 0
    # the face's EOS solves dominate, HLLC and MUSCL are the rest
    assert 2 * (a["cell"] - 6 * 13) < a["face"] < 3 * a["cell"]


def test_y_direction_same_work(oracle10):
    s = stencil()
    assert oracle10.flux_flops(s, 1, 3)["face"] == oracle10.flux_flops(s, 0, 3)["face"]


def test_bench_flux_roofline_arithmetic():
    sys.path.insert(0, ROOT)
    import bench
    ff = {"face": 2000.0, "cell": 1000.0, "combine": 39.0}
    r = bench.flux_roofline(ff, 13, 1 << 20, 20.0, 1250.0, 6800.0)
    flops = 4 * (2 * 2000 + 1000) + 2 * 39
    assert r["fp64"]["flops_per_cell_step"] == flops
    assert r["hbm"]["bytes_per_cell_step"] == 2 * 5 * 13 * 8 == 1040
    assert np.isclose(r["fp64"]["achieved"], flops * (1 << 20) / 0.020 / 1e9)
    assert np.isclose(r["hbm"]["frac"], 1040 * (1 << 20) / 0.020 / 1e9 / 6800.0)
    assert r["bound"] == "fp64"
