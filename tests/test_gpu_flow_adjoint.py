"""Discrete adjoint of a run of Strang steps (hf_flow_record / hf_flow_adjoint) against
central differences of the CPU oracle.

Case: the 1D planar detonation (a 60 x 2 cut, N2 diluent: the oracle's 9 species, a
smooth perturbation of every component), 16 CFL steps recorded by the GPU run and
replayed with the same step sizes by the oracle.  Objective: a fixed random linear functional J = <c, U_final> (c scaled per
component), whose gradient is the seed.  Bar: 1e-5 relative (2-norm over the 21
reactions) for dJ/d ln A_r, 1e-5 relative for sampled components of dJ/dU0.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NX, NSTEPS, K = 60, 16, 5


def case():
    """The 1D detonation with a smooth perturbation of every component (a few percent,
    its own phase per component), so that no limiter sits exactly at its kink: on the
    uniform states of the plain case every slope is zero, where minmod has no
    derivative and one-cell differences pick up its piecewise-linear response."""
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det1d(diluent="N2", nx=NX)
    x = (np.arange(NX) + 0.5) / NX
    ns = U.shape[0] - 3
    for n in range(U.shape[0]):
        ph = 0.7 * n + 0.3
        if n < ns or n == ns + 2:
            U[n] *= 1.0 + 0.02 * np.sin(2 * np.pi * 3 * x + ph)[None, :]
        elif n == ns:
            U[n] = U[:ns].sum(0) * 5.0 * np.sin(2 * np.pi * 2 * x + ph)[None, :]
    return U, lvd


def scales(U):
    """Largest magnitude of each component, at least 1e-3 of the largest density for the
    species (most are absent initially); the momenta (zero at rest, rho v zero in 1D)
    take the largest density times 1000 m/s."""
    s = np.abs(U).reshape(U.shape[0], -1).max(1)
    ns = U.shape[0] - 3
    rho = U[:ns].sum(0).max()
    s[:ns] = np.maximum(s[:ns], 1e-3 * rho)
    s[ns] = s[ns + 1] = rho * 1000.0
    return s


def weights(U, seed=7):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, U.shape) / scales(U)[:, None, None]


def oracle_run(oracle, lvd, U0, dts, chemistry=True):
    g = oracle.make_grid(NX, 2, lvd["dx"], lvd["dy"], periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U0.transpose(1, 2, 0))
    for dt in dts:
        Ug, dta, st, _ = oracle.strang_step(g, Ug, dt, chemistry=chemistry)
        assert st == 0 and dta == dt
    return Ug[2:-2, 2:-2].transpose(2, 0, 1)


@pytest.mark.parametrize("chemistry", [True, False])
def test_flow_adjoint_matches_oracle_fd(gpu, oracle, chemistry):
    import hyperflow_gb300 as hf
    U, lvd = case()
    lv = hf.make_level(**lvd)
    fa = hf.FlowAdjoint(gpu, lv, torch.from_numpy(U).cuda(), NSTEPS, checkpoint_every=K, chemistry=chemistry)
    c = weights(U)
    U0b, g = fa.adjoint(torch.from_numpy(c).cuda())
    U0b = U0b.cpu().numpy()
    dts = fa.dts.copy()
    # the recorded run is the oracle's run with the same step sizes
    ref = oracle_run(oracle, lvd, U, dts, chemistry)
    fin = fa.final.cpu().numpy()
    assert np.max(np.abs(fin - ref) / scales(ref)[:, None, None]) < 1e-8
    if chemistry:
        # d/d ln A_r
        h = 1e-6
        fd = np.zeros(21)
        for r in range(21):
            Jpm = []
            for sgn in (1.0, -1.0):
                m = np.ones(21)
                m[r] = np.exp(sgn * h)
                oracle.set_rate_mult(m)
                try:
                    Jpm.append(float((c * oracle_run(oracle, lvd, U, dts)).sum()))
                finally:
                    oracle.set_rate_mult(None)
            fd[r] = (Jpm[0] - Jpm[1]) / (2 * h)
        assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-5, (g, fd)
    else:
        assert np.all(g == 0.0)
    # d/dU0 at sampled cells, for the components present initially (the absent
    # species cannot be perturbed both ways)
    rng = np.random.default_rng(3)

    def run(V):
        return oracle_run(oracle, lvd, V, dts, chemistry)
    for n in (0, 1, 8, 9, 10, 11):  # H2, O2, N2, rho u, rho v, rho E
        i = int(rng.integers(0, NX))
        j = int(rng.integers(0, 2))
        d = 1e-6 * max(abs(U[n, j, i]), np.abs(U[n]).max() * 1e-3)
        Up, Um = U.copy(), U.copy()
        Up[n, j, i] += d
        Um[n, j, i] -= d
        fd0 = ((c * run(Up)).sum() - (c * run(Um)).sum()) / (2 * d)
        assert abs(U0b[n, j, i] - fd0) <= 1e-5 * max(abs(fd0), 1e-3 * np.abs(U0b[n]).max()), (n, U0b[n, j, i], fd0)
    fa.close()


def test_flow_adjoint_checkpoint_interval_invariant(gpu):
    import hyperflow_gb300 as hf
    U, lvd = case()
    lv = hf.make_level(**lvd)
    c = torch.from_numpy(weights(U)).cuda()
    outs = []
    for k in (1, 4, NSTEPS):
        fa = hf.FlowAdjoint(gpu, lv, torch.from_numpy(U).cuda(), 8, checkpoint_every=k)
        outs.append(fa.adjoint(c))
        fa.close()
    for U0b, g in outs[1:]:
        assert torch.equal(U0b, outs[0][0])
        assert np.array_equal(g, outs[0][1])


def test_flow_adjoint_2d_matches_oracle_fd(gpu, oracle):
    # a 2D cut of the cellular detonation (periodic in y, N2 diluent) with a smooth
    # perturbation in x and y: exercises the y faces and the periodic ghost transpose
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    nx, ny, nsteps = 24, 12, 5
    U, lvd = W.det2d(seed=4, diluent="N2", nx=nx, ny=ny, hot_columns=6)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    ns = U.shape[0] - 3
    for n in range(U.shape[0]):
        U[n] *= 1.0 + 0.02 * np.sin(2 * np.pi * (2 * x[None, :] + y[:, None]) + 0.9 * n)
    rho = U[:ns].sum(0)
    U[ns] = rho * 5.0 * np.sin(2 * np.pi * (x[None, :] + 2 * y[:, None]) + 0.4)
    U[ns + 1] = rho * 3.0 * np.sin(2 * np.pi * (2 * x[None, :] - y[:, None]) + 1.1)
    lv = hf.make_level(**lvd)
    fa = hf.FlowAdjoint(gpu, lv, torch.from_numpy(U).cuda(), nsteps, checkpoint_every=2)
    c = weights(U)
    U0b, g = fa.adjoint(torch.from_numpy(c).cuda())
    U0b = U0b.cpu().numpy()
    dts = fa.dts.copy()
    grid = oracle.make_grid(nx, ny, lvd["dx"], lvd["dy"], periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0),
                            inlet=lvd["inlet"])

    def run(V, mult=None):
        oracle.set_rate_mult(mult)
        try:
            Ug = oracle.ghosted(V.transpose(1, 2, 0))
            for dt in dts:
                Ug, dta, st, _ = oracle.strang_step(grid, Ug, dt)
                assert st == 0 and dta == dt
        finally:
            oracle.set_rate_mult(None)
        return Ug[2:-2, 2:-2].transpose(2, 0, 1)
    fin = fa.final.cpu().numpy()
    assert np.max(np.abs(fin - run(U)) / scales(U)[:, None, None]) < 1e-8
    h = 1e-6
    fd = np.zeros(21)
    for r in range(21):
        m = np.ones(21)
        m[r] = np.exp(h)
        Jp = (c * run(U, m)).sum()
        m[r] = np.exp(-h)
        Jm = (c * run(U, m)).sum()
        fd[r] = (Jp - Jm) / (2 * h)
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-5, (g, fd)
    rng = np.random.default_rng(5)
    for n in (0, 1, 8, 9, 10, 11):
        i, j = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        d = 1e-6 * max(abs(U[n, j, i]), np.abs(U[n]).max() * 1e-3)
        Up, Um = U.copy(), U.copy()
        Up[n, j, i] += d
        Um[n, j, i] -= d
        fd0 = ((c * run(Up)).sum() - (c * run(Um)).sum()) / (2 * d)
        assert abs(U0b[n, j, i] - fd0) <= 1e-5 * max(abs(fd0), 1e-3 * np.abs(U0b[n]).max()), (n, U0b[n, j, i], fd0)
    fa.close()
