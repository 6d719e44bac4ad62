"""The allocation-free chemistry entry point, hf_chem_advance_noalloc.

Some callers of this library cannot call cudaMalloc: an application that hands its
whole device-memory budget to its own pool before loading the library (a library
allocation would fail or break that budget), or host code that must not take the
device-wide synchronisation cudaMalloc and cudaFree can imply.  This entry point needs
no context and keeps its scratch in a fixed device array of HF_NOALLOC_MAX_CELLS cells.
Its results must equal those of the allocating entry point hf_chem_advance (plain form)
on the same cells, over two calls in a row (the shared array keeps the previous call's
contents).  The comparison runs twice: in a fresh process, where the first call comes
before any context exists (so the entry point loads the rate constants itself), and in
this process after the other tests.  This file is collected last.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

HF_OK, HF_ERR_ARG, HF_CHEM_PLAIN = 0, 4, 0
MAX_CELLS = 16384
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from hyperflow_gb300 import build
    lib = ctypes.CDLL(build.build())
    vp, i64, d = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
    lib.hf_chem_advance_noalloc.restype = ctypes.c_int32
    lib.hf_chem_advance_noalloc.argtypes = [ctypes.c_int, vp, i64, vp, i64, d, vp, d, d, ctypes.POINTER(i64), vp]
    return lib


def _T(states_aos):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.set_species(9)
    return oracle.properties(states_aos)[2]


def compare(context_first):
    """Two allocation-free calls, then the same two intervals through the allocating entry
    point, on 3000 cells of uneven stiffness; context_first creates the context (which
    loads the unscaled rate constants) before the allocation-free calls."""
    from hyperflow_gb300 import workloads as W
    import hyperflow_gb300 as hf
    lib = _lib()
    ctx = hf.Context("H2_Li") if context_first else None
    U, dt = W.chem_batch(3000, seed=7, diluent="N2")
    n = U.shape[1]
    a = torch.from_numpy(U.copy()).cuda()
    dtc = torch.from_numpy(dt).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    first = ctypes.c_int64(-1)
    for _ in range(2):
        st = lib.hf_chem_advance_noalloc(9, ctypes.c_void_p(a.data_ptr()), n, None, n, 0.0,
                                         ctypes.c_void_p(dtc.data_ptr()), 1e-8, 1e-15, ctypes.byref(first), stream)
        torch.cuda.synchronize()
        assert st == HF_OK and first.value == -1
    ctx = ctx or hf.Context("H2_Li")
    b = torch.from_numpy(U.copy()).cuda()
    cb = hf.ChemistryBatch(ctx, "plain")
    for _ in range(2):
        cb.advance(b, 0.0, dt_cell=dtc)
    ga, gb = a.cpu().numpy().T, b.cpu().numpy().T
    Ta, Tb = _T(ga), _T(gb)
    # the tolerances of the chemistry parity tests: T relative 1e-6, Y absolute 1e-8
    assert np.max(np.abs(Ta - Tb) / Tb) < 1e-6
    rho = gb[:, :9].sum(1, keepdims=True)
    assert np.max(np.abs(ga[:, :9] - gb[:, :9]) / rho) < 1e-8
    assert np.array_equal(ga[:, 9:], gb[:, 9:])  # momentum and energy untouched


def test_noalloc_matches_allocating_entry_point_in_a_fresh_process():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    code = ("import sys; sys.path[:0] = [%r, %r]; import test_zz_no_alloc as t; t.compare(False); print('ok')"
            % (ROOT, os.path.join(ROOT, "tests")))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-3000:]


def test_noalloc_matches_allocating_entry_point_after_other_tests():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    compare(True)


def test_noalloc_rejects_oversized_batch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib()
    n = MAX_CELLS + 1
    a = torch.ones(12, n, dtype=torch.float64, device="cuda")
    before = a.clone()
    first = ctypes.c_int64(0)
    st = lib.hf_chem_advance_noalloc(9, ctypes.c_void_p(a.data_ptr()), n, None, n, 1e-7, None, 1e-8, 1e-15,
                                     ctypes.byref(first), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == HF_ERR_ARG and first.value == -1
    assert torch.equal(a, before)
