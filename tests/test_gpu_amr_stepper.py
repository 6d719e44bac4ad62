"""Multi-level block AMR stepper (hf_amr_*): BlockAMR::run with max_level > 0.

- Full refinement: with every level-1 block active, level 1 is a one-level run of the
  fine grid (its ghosts are physical or in place) and level 0 its average: the fine
  level must equal the one-level stepper's result bit for bit.
- Partial refinement on a periodic box: reflux, average_down, the leaf-cell chemistry
  and the regrid's conservative interpolation keep the composite totals.
- Regrid: the active blocks are the deterministic function of the ErrorEst tags
  (tagged footprint grown by tag_buffer, proper nesting) restated here in Python.
- The oblique-detonation wedge (three levels) runs and refines along the shock.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def small_det(nx=32, ny=16, periodic=(0, 1)):
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=6, diluent="N2", nx=nx, ny=ny, hot_columns=6)
    lvd = dict(lvd, periodic=periodic)
    return U, lvd


def coarsen(F):
    """average_down of a whole level: the four children summed row by row (j, i),
    (j, i+1), (j+1, i), (j+1, i+1), times 1/4 (AMReX avgdown order)."""
    return (((F[:, 0::2, 0::2] + F[:, 0::2, 1::2]) + F[:, 1::2, 0::2]) + F[:, 1::2, 1::2]) * 0.25


def test_amr_full_refinement_equals_fine_run(gpu):
    import hyperflow_gb300 as hf
    U, lvd = small_det()
    lv = hf.make_level(**lvd)
    box = (-1.0, 1.0, -1.0, 1.0)  # every cell tagged: level 1 covers the domain
    amr = hf.AmrStepper(gpu, lv, cuda(U), max_level=1, block=16, tags=dict(box=box, box_only=True))
    assert amr.info(0)["finest"] == 1
    F0, act = amr.level(1)
    assert act.all()
    fine = hf.make_level(**dict(lvd, nx=2 * lvd["nx"], ny=2 * lvd["ny"], dx=lvd["dx"] / 2, dy=lvd["dy"] / 2))
    st = hf.Stepper(gpu, fine, F0.contiguous(), flux="plain", chem="batched")
    for _ in range(4):
        dt = amr.step(cfl=0.5)
        assert st.step(dt=dt) == dt
    F, _ = amr.level(1)
    assert torch.equal(F, st.state())
    C, _ = amr.level(0)
    assert np.array_equal(C.cpu().numpy(), coarsen(F.cpu().numpy()))
    st.close()
    amr.close()


def test_amr_partial_refinement_conserves(gpu):
    import hyperflow_gb300 as hf
    U, lvd = small_det(periodic=(1, 1))
    lv = hf.make_level(**lvd)
    x0, x1 = lvd["dx"] * 4, lvd["dx"] * 14  # refine a band over the hot columns and beyond
    amr = hf.AmrStepper(gpu, lv, cuda(U), max_level=1, block=16, tag_buffer=1, regrid_interval=3,
                        tags=dict(box=(x0, x1, -1.0, 1.0), box_only=True))
    _, act = amr.level(1)
    assert 0 < act.sum() < act.size
    t0 = amr.totals()
    ns = U.shape[0] - 3
    mag = np.abs(U).reshape(U.shape[0], -1).sum(1) * lvd["dx"] * lvd["dy"]
    for _ in range(7):  # two regrids on the way
        amr.step(cfl=0.5)
    t1 = amr.totals()
    mass0, mass1 = t0[:ns].sum(), t1[:ns].sum()
    assert abs(mass1 - mass0) <= 1e-13 * mass0
    # momenta start at zero: their scale is the mass times 3000 m/s
    scale = [mass0 * 3000.0, mass0 * 3000.0, mag[ns + 2]]
    for n, sc in zip((ns, ns + 1, ns + 2), scale):
        assert abs(t1[n] - t0[n]) <= 1e-12 * sc, n


def test_amr_regrid_blocks_follow_tags(gpu):
    import hyperflow_gb300 as hf
    U, lvd = small_det(nx=64, ny=32)
    lv = hf.make_level(**lvd)
    tags = dict(pressure_tag=0.08, temperature_tag=0.08, density_tag=0.05)
    amr = hf.AmrStepper(gpu, lv, cuda(U), max_level=1, block=16, tag_buffer=2, tags=tags)
    _, act = amr.level(1)
    # ErrorEst on the base level (one patch, ghosts filled) and the block rule restated
    import ctypes
    ps = hf.PatchSet(U.shape[0], [(0, 0, lvd["nx"] - 1, lvd["ny"] - 1)], device="cuda")
    ps.interior(0).copy_(cuda(U))
    gpu.check(gpu.lib.hf_fill_ghosts(gpu.h, ctypes.byref(lv), ps.patches, 1, ctypes.c_void_p(ps.data.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "fill")
    t = hf.tag_cells(gpu, lv, ps, 0.0, chemistry=True, **tags).cpu().numpy().reshape(lvd["ny"], lvd["nx"])
    half, buf = 8, 2
    nby, nbx = act.shape
    want = np.zeros_like(act)
    for bj in range(nby):
        for bi in range(nbx):
            i0, j0 = bi * half, bj * half
            # the footprint grown by tag_buffer: cut at the x edges, wrapped in y (periodic)
            rows = np.arange(j0 - buf, j0 + half + buf) % lvd["ny"]
            sub = t[rows][:, max(i0 - buf, 0):min(i0 + half + buf, lvd["nx"])]
            want[bj, bi] = 1 if sub.any() else 0  # nesting holds: level 0 is all active
    assert want.any() and not want.all()
    assert np.array_equal(act, want)
    amr.close()


def test_amr_wedge_three_levels(gpu):
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    ctx = gpu
    U, lvd = W.wedge(nx=64, ny=32)
    lv = hf.make_level(**lvd)
    amr = hf.AmrStepper(ctx, lv, cuda(U), max_level=2, block=16, tag_buffer=2, regrid_interval=4,
                        tags=dict(density_tag=0.05))
    t = 0.0
    for _ in range(12):
        t += amr.step(cfl=0.5)
    assert abs(amr.time - t) <= 1e-15 * t
    info = [amr.info(l) for l in range(3)]
    assert info[0]["finest"] == 2
    assert info[2]["leaf_cells"] > 0
    # the refinement follows the shock off the wedge surface: level-1 blocks sit over
    # the wedge (x >= 0), none far upstream of the tip in the free stream at the top left
    _, act1 = amr.level(1)
    assert act1.sum() > 0
    assert act1[-1, 0] == 0
    for l in range(3):
        F, a = amr.level(l)
        blk = 16
        for bj, bi in zip(*np.nonzero(a)):
            Fb = F[:, bj * blk:(bj + 1) * blk, bi * blk:(bi + 1) * blk]
            assert torch.isfinite(Fb).all()
            assert (Fb[:9] >= 0).all()
    amr.close()


@pytest.mark.parametrize("case", ["periodic", "wedge"])
def test_amr_graph_steps_equal_host_steps(gpu, case):
    """The graph-captured multi-level step (device dt, one status read per step,
    recaptured after each regrid) gives the host-driven path's states bit for bit."""
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    if case == "periodic":
        U, lvd = small_det(periodic=(1, 1))
        kw = dict(max_level=1, block=16, tag_buffer=1, regrid_interval=3,
                  tags=dict(box=(lvd["dx"] * 4, lvd["dx"] * 14, -1.0, 1.0), box_only=True))
    else:
        U, lvd = W.wedge(nx=64, ny=32)
        kw = dict(max_level=2, block=16, tag_buffer=2, regrid_interval=4, tags=dict(density_tag=0.05))
    lv = hf.make_level(**lvd)
    a = hf.AmrStepper(gpu, lv, cuda(U), **kw)
    b = hf.AmrStepper(gpu, lv, cuda(U), **kw)
    b.set_graph(False)
    for _ in range(9):  # two or three regrids on the way
        assert a.step(cfl=0.5) == b.step(cfl=0.5)
    assert a.stats()["graph_steps"] == 9 and b.stats()["graph_steps"] == 0
    assert a.time == b.time
    for l in range(kw["max_level"] + 1):
        Fa, acta = a.level(l)
        Fb, actb = b.level(l)
        assert np.array_equal(acta, actb)
        blk = kw["block"]
        for bj, bi in zip(*np.nonzero(acta)):
            sl = (slice(None), slice(bj * blk, (bj + 1) * blk), slice(bi * blk, (bi + 1) * blk))
            assert torch.equal(Fa[sl], Fb[sl]), (l, bj, bi)
    a.close()
    b.close()


@pytest.mark.parametrize("chemistry", [False, True])
def test_amr_step_matches_composite_oracle(gpu, oracle, chemistry):
    """Two-level periodic hierarchy (the GPU's own initial blocks, no regrid), plain
    chemistry: two CFL steps of the GPU stepper against the CPU oracle of the composite
    step (oracle/amr.py) with the same step sizes.  Flux path alone: 1e-10 of each
    component's physical scale (species: the largest density; momenta: that density
    times 1000 m/s; energy: its largest magnitude), since rho v is ~0 in this case and a
    per-component relative measure divides roundoff by it.  With chemistry, the full-run
    bar (T rel 1e-6, Y_k abs 1e-8): the stiff igniting cells amplify the roundoff-level
    differences of the interpolation and averaging order."""
    import amr
    import hyperflow_gb300 as hf
    U, lvd = small_det(periodic=(1, 1))
    lv = hf.make_level(**lvd)
    x0, x1 = lvd["dx"] * 4, lvd["dx"] * 14
    g = hf.AmrStepper(gpu, lv, cuda(U), max_level=1, block=16, tag_buffer=1, regrid_interval=0, chem="plain",
                      chemistry=chemistry, tags=dict(box=(x0, x1, -1.0, 1.0), box_only=True))
    L0, _ = g.level(0)
    L1, act = g.level(1)
    assert 0 < act.sum() < act.size
    o = amr.AmrOracle(L0.cpu().numpy().transpose(1, 2, 0), L1.cpu().numpy().transpose(1, 2, 0), act, lvd["dx"],
                      lvd["dy"], 16, chemistry=chemistry)
    for _ in range(2):
        o.step(g.step(cfl=0.5))
    G0 = g.level(0)[0].cpu().numpy().transpose(1, 2, 0)
    G1 = g.level(1)[0].cpu().numpy().transpose(1, 2, 0)
    pairs = [(G0.reshape(-1, 12), o.level(0).reshape(-1, 12))]
    for bj, bi in zip(*np.nonzero(act)):
        sl = (slice(bj * 16, (bj + 1) * 16), slice(bi * 16, (bi + 1) * 16))
        pairs.append((G1[sl].reshape(-1, 12), o.level(1)[sl].reshape(-1, 12)))
    ref_all = np.concatenate([r for _, r in pairs])
    rho = ref_all[:, :9].sum(1).max()
    scale = np.array([rho] * 9 + [rho * 1000.0] * 2 + [np.abs(ref_all[:, 11]).max()])
    for got, ref in pairs:
        if not chemistry:
            assert np.max(np.abs(got - ref) / scale) < 1e-10
        else:
            Tg, Tr = oracle.properties(got)[2], oracle.properties(ref)[2]
            assert np.max(np.abs(Tg - Tr) / Tr) < 1e-6
            assert np.max(np.abs(got[:, :9] - ref[:, :9]) / ref[:, :9].sum(1, keepdims=True)) < 1e-8
    g.close()
