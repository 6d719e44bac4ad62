"""GPU parity of the block-AMR level operations against the CPU oracle: conserved
totals (BlockAMR.cpp:347-355), average_down (:157-159), reflux (:247-255) and
ErrorEst tagging (:170-200), on multi-patch levels packed in one device buffer."""
import numpy as np
import pytest
import torch

import helpers as H

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_totals_match_long_double(gpu, oracle):
    import hyperflow_gb300 as hf
    ps = hf.PatchSet(12, [(0, 0, 9, 5), (10, 0, 19, 5), (0, 6, 19, 8)])
    rng = np.random.default_rng(0)
    cells = []
    for k in range(len(ps)):
        v = rng.normal(size=tuple(ps.interior(k).shape)) * 10.0 ** rng.uniform(-3, 3, size=(12, 1, 1))
        ps.interior(k).copy_(cuda(v))
        cells.append(v.reshape(12, -1).T)
    cells = np.vstack(cells)
    mask = (rng.uniform(size=len(cells)) < 0.7).astype(np.uint8)
    for absolute in (False, True):
        got = np.array(hf.totals(gpu, ps, 2.5e-9, leaf_mask=cuda(mask), absolute=absolute))
        ref = oracle.totals(cells, 2.5e-9, mask=mask, absolute=absolute)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-15


def test_average_down_matches_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    fine = hf.PatchSet(12, [(4, 2, 11, 9), (12, 2, 15, 5)])
    coarse = hf.PatchSet(12, [(0, 0, 11, 7)])
    rng = np.random.default_rng(1)
    for k in range(len(fine)):
        fine.interior(k).copy_(cuda(rng.uniform(0.5, 2.0, size=tuple(fine.interior(k).shape))))
    before = coarse.interior(0).cpu().numpy().copy()
    hf.average_down(gpu, fine, coarse)
    got = coarse.interior(0).cpu().numpy()
    expect = before.copy()
    for k, (i0, j0, i1, j1) in enumerate(fine.boxes):
        avg = oracle.average_down(fine.interior(k).cpu().numpy().transpose(1, 2, 0))
        expect[:, j0 // 2:(j1 + 1) // 2, i0 // 2:(i1 + 1) // 2] = avg.transpose(2, 0, 1)
    assert np.array_equal(got, expect)


@pytest.mark.parametrize("periodic", [(0, 0), (1, 1)])
def test_reflux_matches_oracle(gpu, oracle, periodic):
    import hyperflow_gb300 as hf
    nxc, nyc, nv = 16, 12, 12
    dxc, dyc, h = 2e-4, 1e-4, 3e-9
    rng = np.random.default_rng(2)
    coarse = hf.PatchSet(nv, [(0, 0, nxc - 1, nyc - 1)])
    Uc = rng.uniform(1.0, 2.0, size=(nv, nyc, nxc))
    coarse.interior(0).copy_(cuda(Uc))
    fxc = rng.normal(size=(nv, nyc, nxc + 1))
    fyc = rng.normal(size=(nv, nyc + 1, nxc))
    boxes = [(4, 4, 11, 11), (24, 0, 31, 7), (12, 16, 19, 23)]  # the second touches x-hi, the third y-hi
    fine = hf.PatchSet(nv, boxes)
    fx_list, fy_list = [], []
    for (i0, j0, i1, j1) in boxes:
        nxf, nyf = i1 - i0 + 1, j1 - j0 + 1
        fx_list.append(rng.normal(size=(nv, nyf, nxf + 1)))
        fy_list.append(rng.normal(size=(nv, nyf + 1, nxf)))
    lv = hf.make_level(nxc, nyc, dxc, dyc, periodic=periodic)
    fxf = cuda(np.concatenate([a.ravel() for a in fx_list]))
    fyf = cuda(np.concatenate([a.ravel() for a in fy_list]))
    hf.reflux(gpu, lv, coarse, cuda(fxc.ravel()), cuda(fyc.ravel()), fine, fxf, fyf, h)
    got = coarse.interior(0).cpu().numpy()
    ref = oracle.reflux(Uc.transpose(1, 2, 0), fxc.transpose(1, 2, 0), fyc.transpose(1, 2, 0), boxes,
                        [a.transpose(1, 2, 0) for a in fx_list], [a.transpose(1, 2, 0) for a in fy_list], h, dxc, dyc,
                        periodic=periodic).transpose(2, 0, 1)
    assert not np.array_equal(ref, Uc)
    assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-13


def test_tagging_matches_oracle(gpu, oracle):
    import hyperflow_gb300 as hf
    nx, ny = 40, 24
    field = H.smooth_field(nx, ny, seed=9, amp=0.6)
    field[8:12, 20:26] *= 1.5   # a density/pressure feature
    g = oracle.make_grid(nx, ny, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0))
    Ug = oracle.fill_ghosts(g, oracle.ghosted(field))
    crit = oracle.TagCriteria()
    crit.pressure_tag, crit.temperature_tag, crit.fuel_rate_tag, crit.density_tag = 0.08, 0.06, 50.0, 0.05
    crit.chemistry, crit.box_only, crit.has_box = 1, 0, 1
    for k, v in enumerate((0.0005, 0.001, 0.0, 0.0008)):
        crit.box[k] = v
    crit.velocity[0], crit.velocity[1] = 300.0, 0.0
    ref, st = oracle.tag(g, Ug, 1e-7, crit)
    assert st == 0 and 0 < ref.sum() < nx * ny
    ps = hf.PatchSet(12, [(0, 0, nx - 1, ny - 1)])
    ps.view(0)[:, :, :nx + 4] = cuda(Ug.transpose(2, 0, 1))
    lv = hf.make_level(nx, ny, 1e-4, 1e-4, periodic=(0, 1))
    got = hf.tag_cells(gpu, lv, ps, 1e-7, pressure_tag=0.08, temperature_tag=0.06, fuel_rate_tag=50.0,
                       density_tag=0.05, chemistry=True, box=(0.0005, 0.001, 0.0, 0.0008), velocity=(300.0, 0.0))
    assert np.array_equal(got.cpu().numpy().reshape(ny, nx), ref)


def test_multi_patch_launches_equal_single_patch(gpu):
    """One launch over every patch of a level (the multi-patch face/update, validation and
    CFL kernels) gives the bits of one call per patch."""
    import ctypes
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import _lib as L
    lib, hh = gpu.lib, gpu.h
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    nx, ny, nv = 48, 24, 12
    boxes = [(0, 0, 15, 11), (16, 0, 47, 11), (0, 12, 31, 23), (32, 12, 47, 23)]  # the whole domain
    lv = hf.make_level(nx, ny, 1e-4, 1e-4, periodic=(1, 1))
    field = H.smooth_field(nx, ny, seed=9)
    src = hf.PatchSet(nv, boxes)
    for k, (i0, j0, i1, j1) in enumerate(boxes):
        src.interior(k).copy_(cuda(field[j0:j1 + 1, i0:i1 + 1].transpose(2, 0, 1)))
    gpu.check(lib.hf_fill_ghosts(hh, ctypes.byref(lv), src.patches, len(boxes), p(src.data), s), "fill")
    dt = ctypes.c_double()
    gpu.check(lib.hf_cfl_dt(hh, ctypes.byref(lv), src.patches, len(boxes), p(src.data), 0.5, ctypes.byref(dt), s),
              "cfl")
    one = []
    for k in range(len(boxes)):
        d = ctypes.c_double()
        gpu.check(lib.hf_cfl_dt(hh, ctypes.byref(lv), ctypes.byref(src.patches[k]), 1, p(src.data), 0.5,
                                ctypes.byref(d), s), "cfl")
        one.append(d.value)
    assert dt.value == min(one)
    bad = ctypes.c_int64()
    out_all = hf.PatchSet(nv, boxes)
    out_one = hf.PatchSet(nv, boxes)
    gpu.check(lib.hf_flux_update(hh, ctypes.byref(lv), src.patches, len(boxes), p(src.data), None, p(out_all.data),
                                 None, None, 0.5 * dt.value, 0, L.HF_FLUX_PLAIN, ctypes.byref(bad), s), "flux")
    for k in range(len(boxes)):
        gpu.check(lib.hf_flux_update(hh, ctypes.byref(lv), ctypes.byref(src.patches[k]), 1, p(src.data), None,
                                     p(out_one.data), None, None, 0.5 * dt.value, 0, L.HF_FLUX_PLAIN,
                                     ctypes.byref(bad), s), "flux")
    assert torch.equal(out_all.data, out_one.data)
    assert not torch.equal(out_all.interior(0), src.interior(0))
    # validation: the bad cell's index counts the cells of the patches before it
    out_all.interior(2)[0, 5, 7] = -1.0
    b_all, b_one = ctypes.c_int64(-1), ctypes.c_int64(-1)
    assert lib.hf_validate(hh, ctypes.byref(lv), out_all.patches, len(boxes), p(out_all.data), ctypes.byref(b_all),
                           s) == L.HF_ERR_INADMISSIBLE
    assert lib.hf_validate(hh, ctypes.byref(lv), ctypes.byref(out_all.patches[2]), 1, p(out_all.data),
                           ctypes.byref(b_one), s) == L.HF_ERR_INADMISSIBLE
    before = sum(out_all.patches[k].nx * out_all.patches[k].ny for k in range(2))
    assert b_one.value == 5 * out_all.patches[2].nx + 7
    assert b_all.value == before + b_one.value
