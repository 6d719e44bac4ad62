"""The C host program on the GPU: the same steps as the Python stepper, bit for bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_host_program_equals_python_stepper(gpu, tmp_path):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    from hyperflow_gb300 import hostcase
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=2, diluent="N2", nx=96, ny=24, hot_columns=8)
    case, out = str(tmp_path / "case"), str(tmp_path / "result")
    hostcase.write_case(case, U, nsteps=3, mechanism="H2_Li", flux=L.HF_FLUX_PLAIN, chem=L.HF_CHEM_PERSISTENT,
                        **lvd)
    r = hostcase.run(case, out)
    assert r.returncode == 0, r.stderr
    taken, t, dts, Uh = hostcase.read_result(out, U.shape[0], lvd["ny"], lvd["nx"], 3)
    st = hf.Stepper(gpu, hf.make_level(**lvd), torch.from_numpy(U).cuda(), flux="plain", chem="batched")
    ref_dts = [st.step(cfl=0.5) for _ in range(3)]
    assert taken == 3 and list(dts) == ref_dts and t == st.time
    assert np.array_equal(Uh, st.state().cpu().numpy())
    st.close()
