"""Edge cases of the C ABI on the GPU: empty batches, argument errors returned as status
codes (before any device work, the context stays usable), inadmissible states reported
with their cell index, and a one-cell periodic grid."""
import ctypes

import numpy as np
import pytest
import torch

import helpers as H

pytestmark = pytest.mark.gpu


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_empty_chemistry_batch(gpu):
    # ChemistryBatch::advance with count 0 does nothing (chemistry_batch.cpp:21-50)
    import hyperflow_gb300 as hf
    field = torch.empty(gpu.nv, 0, dtype=torch.float64, device="cuda")
    for form in ("plain", "persistent", "batched"):
        hf.ChemistryBatch(gpu, form).advance(field, 1e-7)


def test_argument_errors_are_status_codes(gpu):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    lib, h = gpu.lib, gpu.h
    nx, ny = 16, 8
    lv = hf.make_level(nx, ny, 1e-3, 1e-3, periodic=(1, 1))
    pin = H.to_patch(gpu, H.ghosted_field(nx, ny, seed=1))
    pout = pin.like()
    bad = ctypes.c_int64()

    def flux(patch, npatch, uin, uout, hh, form=L.HF_FLUX_PLAIN):
        return lib.hf_flux_update(h, ctypes.byref(lv), ctypes.byref(patch), npatch, _p(uin), None, _p(uout), None,
                                  None, hh, 0, form, ctypes.byref(bad), _s())

    assert flux(pin.patch, 0, pin.data, pout.data, 1e-9) == L.HF_ERR_ARG          # no patch
    assert flux(pin.patch, 1, pin.data, pout.data, 0.0) == L.HF_ERR_ARG           # h <= 0
    assert flux(pin.patch, 1, pin.data, pin.data, 1e-9) == L.HF_ERR_ARG           # in place
    thin = L.Patch.from_buffer_copy(pin.patch)
    thin.ng = 1
    assert flux(thin, 1, pin.data, pout.data, 1e-9) == L.HF_ERR_ARG               # 1 ghost layer
    part = L.Patch.from_buffer_copy(pin.patch)
    part.nx = nx // 2
    assert flux(part, 1, pin.data, pout.data, 1e-9, L.HF_FLUX_FUSED) == L.HF_ERR_ARG  # fused: whole domain only
    assert (lib.hf_last_error(h) or b"") != b""
    # chemistry: extent, interval, tolerances, form
    f = torch.from_numpy(H.chem_cells(4, seed=2)).cuda()
    first = ctypes.c_int64()
    chem = lambda n, dt, rtol, form: lib.hf_chem_advance(h, _p(f), f.shape[1], None, n, dt, None, rtol, 1e-15,
                                                         form, ctypes.byref(first), _s())
    assert chem(-1, 1e-7, 1e-8, L.HF_CHEM_PLAIN) == L.HF_ERR_ARG
    assert chem(4, 0.0, 1e-8, L.HF_CHEM_PLAIN) == L.HF_ERR_ARG
    assert chem(4, 1e-7, 0.0, L.HF_CHEM_PLAIN) == L.HF_ERR_ARG
    assert chem(4, 1e-7, 1e-8, 7) == L.HF_ERR_ARG
    assert chem(8, 1e-7, 1e-8, L.HF_CHEM_PLAIN) == L.HF_ERR_ARG                # beyond the component stride
    # interpolation region outside the fine patch's ghosted box
    fine = pin.like()
    reg = (ctypes.c_int32 * 4)(0, 0, nx + 4, 3)
    assert lib.hf_interp_coarse_to_fine(h, ctypes.byref(pin.patch), _p(pin.data), ctypes.byref(fine.patch),
                                        _p(fine.data), reg, _s()) == L.HF_ERR_ARG
    # block-AMR options: odd block size
    with pytest.raises(hf.HyperFlowError) as e:
        hf.AmrStepper(gpu, lv, pin.interior().contiguous(), max_level=1, block=15)
    assert e.value.status == L.HF_ERR_ARG
    # the context is still usable
    hf.euler_stage(gpu, lv, pin, pout, 1e-9)
    assert torch.isfinite(pout.interior()).all()


def test_inadmissible_states_reported(gpu):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    q = torch.from_numpy(H.chem_cells(6, seed=3)).cuda()
    q[0, 2] = -1e-3                 # negative partial density
    q[gpu.nv - 1, 4] = float("nan")  # energy not finite
    ok = hf.admissible(gpu, q).cpu().numpy()
    assert list(ok) == [True, True, False, True, False, True]
    # validate() reports the lowest bad cell of the patch (row-major interior index)
    nx, ny = 12, 6
    lv = hf.make_level(nx, ny, 1e-3, 1e-3, periodic=(1, 1))
    pa = H.to_patch(gpu, H.ghosted_field(nx, ny, seed=4))
    pa.interior()[0, 3, 7] = -1.0
    pa.interior()[0, 4, 2] = -1.0
    bad = ctypes.c_int64(-1)
    st = gpu.lib.hf_validate(gpu.h, ctypes.byref(lv), ctypes.byref(pa.patch), 1, _p(pa.data), ctypes.byref(bad), _s())
    assert st == L.HF_ERR_INADMISSIBLE
    assert bad.value == 3 * nx + 7


def test_one_cell_periodic_grid(gpu, oracle):
    # both faces of the only cell see the cell itself: the fluxes cancel exactly
    import hyperflow_gb300 as hf
    field = H.smooth_field(1, 1, seed=5)
    field[0, 0, 9] = 0.3 * field[0, 0, :9].sum()   # moving gas (rho u)
    g = oracle.make_grid(1, 1, 1e-3, 1e-3, periodic=(1, 1))
    Ug = oracle.fill_ghosts(g, oracle.ghosted(field))
    out, _, _, st = oracle.euler_stage(g, Ug, 1e-8, False)
    assert st == 0
    lv = hf.make_level(1, 1, 1e-3, 1e-3, periodic=(1, 1))
    pin = H.to_patch(gpu, Ug)
    pout = pin.like()
    hf.euler_stage(gpu, lv, pin, pout, 1e-8)
    got = H.from_patch(pout)[2:-2, 2:-2]
    assert np.array_equal(got, out[2:-2, 2:-2])
    assert np.array_equal(got, field)
