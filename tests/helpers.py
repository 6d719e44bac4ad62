"""Shared test helpers: seeded random states and layout conversions.

The oracle works on the reference's AoS layout, a ghosted level array of shape
(ny+4, nx+4, NV); the GPU path uses SoA patch arrays of shape (NV, ny+4, pitch).
"""
import numpy as np

from hyperflow_gb300 import mechanism as M


def random_states(n, seed=0, ns=9, T=(300.0, 3500.0), p=(0.1, 50.0), speed=1500.0, radicals=True):
    """(n, NV) admissible states with random T, p, composition and velocity."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, ns + 3))
    for k in range(n):
        X = rng.uniform(0.0, 1.0, ns)
        if not radicals:
            X[3:8] = 0.0
        X[rng.uniform(size=ns) < 0.2] = 0.0
        if X.sum() == 0:
            X[0] = 1.0
        X /= X.sum()
        t = rng.uniform(*T)
        pr = 101325.0 * np.exp(rng.uniform(np.log(p[0]), np.log(p[1])))
        u, v = rng.uniform(-speed, speed, 2)
        out[k] = M.primitive(t, pr, X=X, u=u, v=v, ns=ns)
    return out


def smooth_field(nx, ny, seed=0, ns=9, amp=0.3):
    """(ny, nx, NV) smooth random field: Gaussian bumps in T, p, u, v and a varying
    H2O/OH content on a diluted stoichiometric H2/O2 base."""
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)

    def bump():
        cx, cy, s = rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.15, 0.35)
        return np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / s ** 2)

    T = 900.0 * (1 + amp * (bump() - 0.5 * bump()) * 2)
    P = 101325.0 * (1 + amp * (bump() + 0.5 * bump()) * 3)
    U = 400.0 * (bump() - bump())
    V = 400.0 * (bump() - bump())
    h2o = 0.05 * (1 + np.sin(2 * np.pi * (X + 0.5 * Y)))
    oh = 1e-3 * (1 + np.cos(2 * np.pi * (2 * X - Y)))
    base = M.mixture_X(1.0, 0.7, "N2" if ns == 9 else "AR", ns)
    out = np.empty((ny, nx, ns + 3))
    for j in range(ny):
        for i in range(nx):
            Xc = base.copy()
            Xc[2] += h2o[j, i]
            Xc[5] += oh[j, i]
            Xc /= Xc.sum()
            out[j, i] = M.primitive(T[j, i], P[j, i], X=Xc, u=U[j, i], v=V[j, i], ns=ns)
    return out


def to_patch(ctx, aos_ghosted, ng=2):
    """(ny+4, nx+4, NV) ghosted AoS -> PatchArray with the same ghost content."""
    import torch
    from hyperflow_gb300 import PatchArray
    ny4, nx4, nv = aos_ghosted.shape
    pa = PatchArray(nv, nx4 - 2 * ng, ny4 - 2 * ng, ng)
    g = np.nan_to_num(aos_ghosted, nan=0.0)
    pa.data[:, :, :nx4] = torch.from_numpy(np.ascontiguousarray(g.transpose(2, 0, 1))).cuda()
    return pa


def from_patch(pa):
    """PatchArray -> (ny+4, nx+4, NV) ghosted AoS numpy array."""
    return pa.ghosted().cpu().numpy().transpose(1, 2, 0).copy()


def rel_err(a, b, floor=1e-300):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)))


def comp_err(a, b):
    """max over components of |a-b| / max(|b| over the field of that component, tiny)."""
    a, b = np.asarray(a), np.asarray(b)
    nv = a.shape[-1]
    a2, b2 = a.reshape(-1, nv), b.reshape(-1, nv)
    scale = np.maximum(np.max(np.abs(b2), axis=0), 1e-300)
    return float(np.max(np.abs(a2 - b2) / scale))


def ghosted_field(nx, ny, seed=0, ns=9):
    """(ny+4, nx+4, NV) smooth field with periodic ghost layers (no oracle needed)."""
    return np.pad(smooth_field(nx, ny, seed=seed, ns=ns), ((2, 2), (2, 2), (0, 0)), mode="wrap")


def chem_cells(n, seed=0):
    """(NV, n) independent 0D cells of uneven stiffness, N2 diluent (9 species)."""
    from hyperflow_gb300 import workloads as W
    return W.chem_batch(n, seed=seed, diluent="N2")[0]


def reference_records():
    """Run outcomes the reference records for its own checks (tests/golden/
    reference_records.json, written by tests/golden/make_reference_records.py)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_records.json")) as f:
        return json.load(f)
