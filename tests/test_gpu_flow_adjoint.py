"""Discrete adjoint of a run of Strang steps (hf_flow_record / hf_flow_adjoint) against
central differences of the CPU oracle.

Case: the 1D planar detonation (a 60 x 2 cut, N2 diluent: the oracle's 9 species, a
smooth perturbation of every component), 16 CFL steps recorded by the GPU run and
replayed with the same step sizes (and chemistry step sequences) by the oracle.
Objective: a fixed random linear functional J = <c, U_final> (c scaled per component),
whose gradient is the seed.  Bar: 1e-5 relative (2-norm over the 21 reactions) for
dJ/d ln A_r; 1e-5 relative (2-norm, scale-weighted) for sampled components of dJ/dU0
against central differences taken at a step that crosses no kink of the scheme.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NX, NSTEPS, K = 60, 16, 5


def case():
    """The 1D detonation with a smooth perturbation of every component (a few percent,
    its own phase per component and row, small velocities in both directions), so that
    the base run sits on no kink of the scheme.  On the plain case the uniform states
    have zero slopes (minmod has no derivative there) and the two identical rows give
    every y face equal left and right wave speeds (min/max ties in HLLC): central
    differences then average two one-sided derivatives."""
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det1d(diluent="N2", nx=NX)
    x = (np.arange(NX) + 0.5) / NX
    ns = U.shape[0] - 3
    for n in range(U.shape[0]):
        for j in range(U.shape[1]):
            ph = 0.7 * n + 0.3 + 1.3 * j
            if n < ns or n == ns + 2:
                U[n, j] *= 1.0 + 0.02 * np.sin(2 * np.pi * 3 * x + ph)
            elif n == ns:
                U[n, j] = U[:ns, j].sum(0) * 5.0 * np.sin(2 * np.pi * 2 * x + ph)
            else:
                U[n, j] = U[:ns, j].sum(0) * 2.0 * np.sin(2 * np.pi * 2 * x + ph)
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


class Frozen:
    """The oracle's run with the recorded step sizes and, with chemistry, its chemistry
    step sequences frozen (replayed): differences of this map carry no step-size
    selection noise."""

    def __init__(self, oracle, grid, U0, dts, chemistry):
        self.o, self.g, self.dts, self.chem = oracle, grid, dts, chemistry
        self.fr = oracle.FrozenRun(grid, oracle.ghosted(U0.transpose(1, 2, 0)), dts) if chemistry else None

    def __call__(self, V, mult=None):
        self.o.set_rate_mult(mult)
        try:
            Ug = self.o.ghosted(V.transpose(1, 2, 0))
            if self.chem:
                Ug = self.fr.replay(Ug)
            else:
                for dt in self.dts:
                    Ug, dta, st, _ = self.o.strang_step(self.g, Ug, dt, chemistry=False)
                    assert st == 0 and dta == dt
        finally:
            self.o.set_rate_mult(None)
        return Ug[2:-2, 2:-2].transpose(2, 0, 1)

    def close(self):
        if self.fr:
            self.fr.close()


def clean_difference(J, U, n, j, i, scale, J0, floor):
    """Central difference of J at U along entry (n, j, i) at a step that crosses no kink
    of the scheme (minmod slope switches, HLLC wave-speed min/max switches of some face
    somewhere in the run), where one-sided derivatives differ.  Central differences at
    1e-6, 1e-7 and 1e-8 times the component's scale: the first pair of consecutive
    steps whose differences agree to 1e-5 of max(|difference|, floor) gives the
    smaller step's value (a crossed kink changes the difference with the step; smooth
    curvature does not, to second order); with no such pair, the step whose forward and
    backward differences agree best.  A step of 1e-6 of the largest energy density moves
    a cold cell's energy by 1e-4 of its own and crosses such switches."""
    cen, spread = [], []
    for e in (1e-6, 1e-7, 1e-8):
        d = e * scale
        Up, Um = U.copy(), U.copy()
        Up[n, j, i] += d
        Um[n, j, i] -= d
        Jp, Jm = J(Up), J(Um)
        c, fwd, bwd = (Jp - Jm) / (2 * d), (Jp - J0) / d, (J0 - Jm) / d
        cen.append(c)
        spread.append(abs(fwd - bwd) / max(abs(c), floor, 1e-300))
    for k in (0, 1):
        if abs(cen[k] - cen[k + 1]) <= 1e-5 * max(abs(cen[k + 1]), floor, 1e-300):
            return cen[k + 1]
    return cen[int(np.argmin(spread))]


def check_dU0(U, U0b, c, run, cells):
    """dJ/dU0 at the given (n, j, i) against kink-free central differences of run()
    (clean_difference), the entries weighted by the component's physical scale: 1e-5
    relative over the sampled entries (2-norm) and 1e-4 for each entry."""
    sc = scales(U)
    J = lambda V: float((c * run(V)).sum())
    J0 = J(U)
    floor = 1e-3 * max(abs(U0b[n, j, i]) * sc[n] for n, j, i in cells)
    a, f = [], []
    for n, j, i in cells:
        fd0 = clean_difference(J, U, n, j, i, sc[n], J0, floor / sc[n])
        a.append(U0b[n, j, i] * sc[n])
        f.append(fd0 * sc[n])
    a, f = np.array(a), np.array(f)
    assert np.linalg.norm(a - f) <= 1e-5 * np.linalg.norm(f), (a, f)
    assert np.all(np.abs(a - f) <= 1e-4 * np.maximum(np.abs(f), 1e-3 * np.abs(f).max())), (cells, a, f)


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
    grid = oracle.make_grid(NX, 2, lvd["dx"], lvd["dy"], periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0),
                            inlet=lvd["inlet"])
    run = Frozen(oracle, grid, U, dts, chemistry)
    if chemistry:
        # d/d ln A_r
        h = 1e-6
        fd = np.zeros(21)
        for r in range(21):
            m = np.ones(21)
            m[r] = np.exp(h)
            Jp = float((c * run(U, m)).sum())
            m[r] = np.exp(-h)
            Jm = float((c * run(U, m)).sum())
            fd[r] = (Jp - Jm) / (2 * h)
        assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-5, (g, fd)
    else:
        assert np.all(g == 0.0)
    # d/dU0 at sampled cells, for the components present initially (the absent
    # species cannot be perturbed both ways)
    rng = np.random.default_rng(3)
    cells = [(n, int(rng.integers(0, 2)), int(rng.integers(0, NX))) for n in (0, 1, 8, 9, 10, 11) for _ in range(2)]
    check_dU0(U, U0b, c, run, cells)
    run.close()
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
    run = Frozen(oracle, grid, U, dts, True)
    fin = fa.final.cpu().numpy()
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    for dt in dts:
        Ug, dta, st, _ = oracle.strang_step(grid, Ug, dt)
        assert st == 0 and dta == dt
    assert np.max(np.abs(fin - Ug[2:-2, 2:-2].transpose(2, 0, 1)) / scales(U)[:, None, None]) < 1e-8
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
    cells = [(n, int(rng.integers(0, ny)), int(rng.integers(0, nx))) for n in (0, 1, 8, 9, 10, 11)]
    check_dU0(U, U0b, c, run, cells)
    run.close()
    fa.close()


def test_flow_adjoint_chemistry_call_in_conserved_variables(gpu, oracle):
    # a 1 x 1 periodic grid: both faces of the cell see the cell itself, the fluxes
    # cancel exactly and every stage is the identity, so the run is the chemistry calls
    # alone as a map of the conserved state (rho Y_k, rho u, rho v, rho E): this checks
    # the transpose through rho and e (y = u_k/rho, e = E/rho - |m|^2/(2 rho^2))
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U = W.ignition_batch(16, seed=3)[:, 3:4, None].copy()  # (NV, 1, 1): H2/air at 1291 K, igniting
    ns = U.shape[0] - 3
    rho = U[:ns].sum()
    U[ns] = rho * 7.0
    U[ns + 1] = -rho * 4.0
    U[ns + 2] += 0.5 * (49.0 + 16.0) * rho
    lvd = dict(nx=1, ny=1, dx=1e-3, dy=1e-3, periodic=(1, 1))
    lv = hf.make_level(**lvd)
    dts = np.full(12, 1e-6)
    fa = hf.FlowAdjoint(gpu, lv, torch.from_numpy(U).cuda(), len(dts), dts=dts, checkpoint_every=5)
    c = weights(U)
    U0b, g = fa.adjoint(torch.from_numpy(c).cuda())
    U0b = U0b.cpu().numpy()
    grid = oracle.make_grid(1, 1, 1e-3, 1e-3, periodic=(1, 1))
    run = Frozen(oracle, grid, U, dts, True)
    fin = fa.final.cpu().numpy()
    assert np.max(np.abs(fin - run(U)) / scales(U)[:, None, None]) < 1e-10
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
    check_dU0(U, U0b, c, run, [(n, 0, 0) for n in (0, 1, 8, 9, 10, 11)])
    run.close()
    fa.close()
