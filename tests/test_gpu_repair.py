"""GPU parity of the roundoff repair (BlockAMR::repairRoundoff, BlockAMR.cpp:299-334) with
the oracles, bit for bit: one level against the one-level oracle (oracle/hf_oracle.cpp),
and the leaf cells of two levels against the composite oracle (oracle/amr.py).  Values
are planted a few ulp below zero (repaired), beyond 64 ulp or not finite (material), and
under a fine block (not a leaf: left alone)."""
import numpy as np
import pytest
import torch

import helpers as H

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def plant(rng, cells, leaf, species, count, ulps=(1, 60)):
    """Set `count` leaf cells of each species to -k ulp of the species' peak over the
    leaf cells (k uniform in ulps); cells: (..., NV) view, leaf: bool mask of its cells."""
    flat = cells.reshape(-1, cells.shape[-1])
    where = np.nonzero(leaf.reshape(-1))[0]
    for n in species:
        peak = flat[where, n].max()
        for c in rng.choice(where, size=count, replace=False):
            flat[c, n] = -rng.integers(*ulps) * EPS * peak * rng.uniform(0.5, 1.0)
    cells[...] = flat.reshape(cells.shape)


def one_level(seed):
    nx, ny, dx = 40, 24, 1e-4
    F = H.smooth_field(nx, ny, seed=seed)
    return nx, ny, dx, F


@pytest.mark.parametrize("count", [1, 40, 700])
def test_repair_one_level_matches_oracle(gpu, oracle, count):
    """Roundoff negatives of three species on one periodic level: zeroed values, donor
    cells and the deficits taken from them equal the oracle's; past the kernel's ordered
    capacity (2048 entries; 3 x 700 here) the deficits are summed in atomic order and
    agree to rounding."""
    import hyperflow_gb300 as hf
    nx, ny, dx, F = one_level(11)
    rng = np.random.default_rng(count)
    plant(rng, F, np.ones((ny, nx), bool), (2, 5, 8), count)  # H2O, OH, N2 (H, O, HO2 are 0 here)
    g = oracle.make_grid(nx, ny, dx, dx, periodic=(1, 1))
    Ug = oracle.ghosted(F)
    ref, st, n_ref = oracle.repair_roundoff(g, Ug)
    assert st == 0 and n_ref == 3 * count
    pa = H.to_patch(gpu, Ug)
    lv = hf.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    n = hf.repair_roundoff(gpu, [(lv, pa, None)])
    got = H.from_patch(pa)[2:-2, 2:-2]
    assert n == n_ref
    if 3 * count <= 2048:
        assert np.array_equal(got, ref[2:-2, 2:-2])
    else:
        keep = [0, 1, 3, 4, 6, 7, 9, 10, 11]  # components the repair does not touch
        assert np.array_equal(got[..., keep], ref[2:-2, 2:-2, keep])
        assert H.comp_err(got, ref[2:-2, 2:-2]) < 1e-15
    assert np.min(got[..., :9]) >= 0.0


@pytest.mark.parametrize("bad", ["far", "nan"])
def test_repair_one_level_material(gpu, oracle, bad):
    """A value 100 ulp of the peak below zero, or NaN, is material: HF_ERR_NEGATIVE, as the
    oracle's status."""
    import hyperflow_gb300 as hf
    nx, ny, dx, F = one_level(12)
    F[5, 7, 5] = -100 * EPS * F[..., 5].max() if bad == "far" else np.nan
    g = oracle.make_grid(nx, ny, dx, dx, periodic=(1, 1))
    _, st, _ = oracle.repair_roundoff(g, oracle.ghosted(F))
    assert st == 1
    pa = H.to_patch(gpu, oracle.ghosted(F))
    pa.interior()[5, 5, 7] = float(F[5, 7, 5])  # to_patch turns NaN (its ghost filler) into 0
    lv = hf.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    with pytest.raises(hf.DomainError, match="HF_ERR_NEGATIVE"):
        hf.repair_roundoff(gpu, [(lv, pa, None)])


def test_repair_two_levels_matches_composite_oracle(gpu, oracle):
    """Leaf cells of a coarse level and of level-1 blocks: the peak and the donor (largest
    mass, value x volume) are taken over both levels; negatives on leaf cells of either
    level are repaired as the composite oracle repairs them, and a material negative under
    a fine block (not a leaf) is left alone."""
    import amr
    import hyperflow_gb300 as hf
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=5)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=6)
    active = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    active[:, 2:5] = 1
    active[1, 6] = 1
    a = amr.AmrOracle(U0, U1, active, dx, dx, B)
    X = [x.copy() for x in a.X]
    l0, l1 = X[0][2:-2, 2:-2], X[1][2:-2, 2:-2]
    m0, m1 = a.leaf_mask(0), a.leaf_mask(1)
    rng = np.random.default_rng(4)
    plant(rng, l0, m0, (2, 5), 15)
    plant(rng, l1, m1, (2, 5, 8), 15)
    l0[4, 10, 2] = -1e-3 * l0[..., 2].max()  # covered by level 1: not a leaf
    assert not m0[4, 10]
    # the GPU's layout of the same hierarchy: level 0 as one patch, level 1 as its active
    # blocks in row-major order, leaf masks packed patch by patch
    lv0 = hf.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    lv1 = hf.make_level(nx=2 * nx, ny=2 * ny, dx=dx / 2, dy=dx / 2, periodic=(1, 1))
    pa = H.to_patch(gpu, X[0])
    blocks = a.blocks(1)
    ps = hf.PatchSet(12, [(bi * B, bj * B, bi * B + B - 1, bj * B + B - 1) for bi, bj in blocks])
    for k, (bi, bj) in enumerate(blocks):
        ps.interior(k).copy_(cuda(l1[bj * B:(bj + 1) * B, bi * B:(bi + 1) * B].transpose(2, 0, 1)))
    leaf0 = cuda(m0.reshape(-1).astype(np.uint8))
    leaf1 = cuda(np.concatenate([m1[bj * B:(bj + 1) * B, bi * B:(bi + 1) * B].reshape(-1)
                                 for bi, bj in blocks]).astype(np.uint8))
    ok, n_ref = a.repair(X)
    assert ok and n_ref == 2 * 15 + 3 * 15
    n = hf.repair_roundoff(gpu, [(lv0, pa, leaf0), (lv1, ps, leaf1)])
    assert n == n_ref
    assert np.array_equal(H.from_patch(pa)[2:-2, 2:-2], X[0][2:-2, 2:-2])
    for k, (bi, bj) in enumerate(blocks):
        got = ps.interior(k).cpu().numpy().transpose(1, 2, 0)
        assert np.array_equal(got, X[1][2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B])
