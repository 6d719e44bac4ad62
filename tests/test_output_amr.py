"""The multi-level output writers (hyperflow_gb300/output.py) on CPU: the leaf cells of
a block hierarchy tile the domain once (the geometry check of
HyperFlow_V3/tests/validate.py:64-78), their conserved sums are the hierarchy's leaf
totals, and state_N.csv / boxes_N.csv read back the way the reference's scripts read
them.  The hierarchy comes from the composite AMR oracle."""
import numpy as np
import pytest

import helpers as H


def check_geometry(data, base_cells, length, max_level):
    """validate.py:64-78, restated: cell sizes per level, total area, every finest pixel
    covered by exactly one leaf cell."""
    level = data["level"].astype(int)
    base_dx = np.array(length) / np.array(base_cells)
    assert np.allclose(data["dx"], base_dx[0] / 2.0 ** level, rtol=1e-13, atol=0)
    assert np.allclose(data["dy"], base_dx[1] / 2.0 ** level, rtol=1e-13, atol=0)
    assert abs(np.sum(data["dx"] * data["dy"]) / np.prod(length) - 1) < 1e-13
    full = np.zeros(np.array(base_cells) * 2 ** max_level, dtype=np.int8)
    for q in data:
        r = 2 ** (max_level - int(q["level"]))
        i, j = int(q["i"]) * r, int(q["j"]) * r
        full[i:i + r, j:j + r] += 1
    assert np.all(full == 1), "leaf cells overlap or leave a hole"
    return len(data)


@pytest.fixture(scope="module")
def out():
    from hyperflow_gb300 import output
    return output


def test_leaf_masks_tile_three_levels(out):
    """Level 1 blocks 0-2 of row 0 and block (1, 1); level 2 blocks inside them."""
    nx, ny, B = 16, 8, 8
    act1 = np.zeros((2, 4), np.uint8)
    act1[0, :3] = 1
    act1[1, 1] = 1
    act2 = np.zeros((4, 8), np.uint8)
    act2[0, 1:4] = 1
    act2[1, 2] = 1
    acts, shapes = [None, act1, act2], [(ny, nx), (2 * ny, 2 * nx), (4 * ny, 4 * nx)]
    masks = out.leaf_masks(acts, shapes, B)
    full = np.zeros((4 * ny, 4 * nx), np.int8)
    for l, m in enumerate(masks):
        r = 2 ** (2 - l)
        for j, i in zip(*np.nonzero(m)):
            full[j * r:(j + 1) * r, i * r:(i + 1) * r] += 1
    assert np.all(full == 1)
    boxes = out.amr_boxes(acts, shapes, B)
    assert boxes[0] == (0, 0, 0, nx - 1, ny - 1) and len(boxes) == 1 + 4 + 4


def test_state_rows_of_the_oracle_hierarchy(oracle, out, tmp_path):
    import amr
    from hyperflow_gb300 import solver as S
    nx, ny, B, dx = 32, 16, 8, 1e-4
    U0 = H.smooth_field(nx, ny, seed=5)
    U1 = H.smooth_field(2 * nx, 2 * ny, seed=6)
    active = np.zeros((2 * ny // B, 2 * nx // B), np.uint8)
    active[:, 2:5] = 1
    active[1, 6] = 1
    a = amr.AmrOracle(U0, U1, active, dx, dx, B)
    base = S.make_level(nx=nx, ny=ny, dx=dx, dy=dx, periodic=(1, 1))
    Qs = [a.level(0).transpose(2, 0, 1), a.level(1).transpose(2, 0, 1)]
    acts, shapes = [None, a.active], [(ny, nx), (2 * ny, 2 * nx)]

    def props(q):
        p, _, T, st = oracle.properties(np.ascontiguousarray(q.T))
        assert not np.any(st)
        return p, T

    rows = out.amr_state_rows(Qs, out.leaf_masks(acts, shapes, B), base, 1e-7, props)
    ns = U0.shape[2] - 3
    out.write_rows(tmp_path / "state_1.csv", rows, ns)
    out.write_amr_boxes(tmp_path / "boxes_1.csv", out.amr_boxes(acts, shapes, B), base)
    data = np.genfromtxt(tmp_path / "state_1.csv", names=True, delimiter=",")
    n = check_geometry(data, (nx, ny), (nx * dx, ny * dx), 1)
    assert n == nx * ny - int(active.sum()) * (B // 2) ** 2 + int(active.sum()) * B * B
    # conserved sums of the rows = the hierarchy's leaf totals
    vol = data["dx"] * data["dy"]
    Y = np.column_stack([data["Y_" + s] for s in out.SPECIES[:ns]])
    got = np.concatenate([(data["rho"][:, None] * Y * vol[:, None]).sum(0),
                          [(data["rho"] * data["u"] * vol).sum(), (data["rho"] * data["v"] * vol).sum(),
                           (data["rhoE"] * vol).sum()]])
    want = a.totals()
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    boxes = np.genfromtxt(tmp_path / "boxes_1.csv", names=True, delimiter=",")
    assert len(boxes) == 1 + int(active.sum())
    assert abs(np.sum((boxes["x_right"] - boxes["x_left"]) * (boxes["y_top"] - boxes["y_bottom"])
                      * (boxes["level"] == 1)) - active.sum() * (B * dx / 2) ** 2) < 1e-18
