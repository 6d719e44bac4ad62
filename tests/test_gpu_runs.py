"""Multi-step runs on the GPU against the CPU oracle, and the reference's output files.

The 1D planar detonation (2000 x 2 cells on 0.1 m in the benchmark; a 400 x 2 cut of it
here, N2 diluent so the oracle's 9-species mechanism applies): a driver of 20 cells at
40 atm / 3000 K, reflecting left, transmissive right, reflecting top and bottom.
"""
import os

import numpy as np
import pytest
import torch

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
