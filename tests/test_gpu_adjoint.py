"""Discrete adjoint of 0D chemistry runs (hf_chem_objective / hf_chem_adjoint) against
the CPU oracle.

Cells: H2/air at rest, T ~ U[1000, 1500] K, p ~ U[1, 5] atm, phi ~ U[0.5, 2] (the
sensitivity workload), 40 chemistry calls of 1 us each.  The oracle differentiates
the same runs by central differences in ln(multiplier_r) with step 1e-6, replaying
each cell's accepted step sequence (the frozen-step map the adjoint differentiates)
and, separately, re-running the adaptive integrator.  Agreement bar: 1e-5 relative
of the gradient vector of every cell (2-norm), and 1e-4 relative on every component
above 1e-3 of the cell's largest (1e-4 of the largest below): the differences carry
rounding noise of ~1e-6 of the largest component, amplified where ignition is under way.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DT, NCALLS = 1e-6, 40


def cells(n=8, seed=1):
    from hyperflow_gb300 import workloads as W
    return W.ignition_batch(n, seed=seed)


def sens(gpu, objective, k=7):
    import hyperflow_gb300 as hf
    return hf.ChemSensitivity(gpu, DT, NCALLS, objective=objective, checkpoint_every=k)


def grad_err(g, ref):
    """(max over cells of the 2-norm relative error, max over cells of the component
    error measure of the module docstring)."""
    worst_n, worst_c = 0.0, 0.0
    for a, b in zip(g, ref):
        worst_n = max(worst_n, float(np.linalg.norm(a - b) / np.linalg.norm(b)))
        scale = np.max(np.abs(b))
        big = np.abs(b) > 1e-3 * scale
        rel = np.abs(a - b) / np.where(big, np.abs(b), scale)
        worst_c = max(worst_c, float(np.max(rel)))
    return worst_n, worst_c


def test_objective_matches_oracle(gpu, oracle):
    U = cells(16)
    for obj in ("ignition_delay", "peak_pressure", "final_T"):
        J = sens(gpu, obj).objective(torch.from_numpy(U).cuda()).cpu().numpy()
        Jr, bad = oracle.chem_objective(U.T, DT, NCALLS, obj)
        assert bad == -1
        assert np.array_equal(np.isnan(J), np.isnan(Jr))
        ok = ~np.isnan(Jr)
        assert ok.sum() >= 8
        assert np.max(np.abs(J[ok] - Jr[ok]) / np.abs(Jr[ok])) < 1e-8, obj


# final_T is taken mid-ignition (10 calls): at equilibrium T no longer depends on the
# rates and the differences are rounding noise (~1e-6 K); cells whose largest
# sensitivity is below 1 K are left out for the same reason
@pytest.mark.parametrize("objective,ncalls,floor", [("ignition_delay", NCALLS, 0.0), ("final_T", 10, 1.0)])
def test_adjoint_matches_frozen_fd(gpu, oracle, objective, ncalls, floor):
    import hyperflow_gb300 as hf
    U = cells(8)
    s = hf.ChemSensitivity(gpu, DT, ncalls, objective=objective, checkpoint_every=7)
    J, G, _ = s.adjoint(torch.from_numpy(U).cuda())
    J, G = J.cpu().numpy(), G.cpu().numpy().T
    Jr, Gr, bad = oracle.chem_sens_fd(U.T, DT, ncalls, objective, fd_h=1e-6, frozen=True)
    assert bad == -1
    nan = np.isnan(Jr)
    assert np.array_equal(np.isnan(J), nan)
    assert np.all(G[nan] == 0.0)
    ok = ~nan & (np.abs(Gr).max(1) > floor)
    assert ok.sum() >= 4
    en, ec = grad_err(G[ok], Gr[ok])
    assert en < 1e-5 and ec < 1e-4, (en, ec)
    # the adaptive integrator's differences agree with the frozen-step derivative too
    _, Ga, _ = oracle.chem_sens_fd(U.T, DT, ncalls, objective, fd_h=1e-6, frozen=False)
    en, ec = grad_err(G[ok], Ga[ok])
    assert en < 1e-4 and ec < 1e-3, (en, ec)


def test_peak_pressure_gradient(gpu, oracle):
    # the peak is the equilibrium pressure at the end of the window: its sensitivities
    # are tiny, so they are compared on the scale of the objective itself
    U = cells(8)
    J, G, _ = sens(gpu, "peak_pressure").adjoint(torch.from_numpy(U).cuda())
    J, G = J.cpu().numpy(), G.cpu().numpy().T
    Jr, Gr, bad = oracle.chem_sens_fd(U.T, DT, NCALLS, "peak_pressure", fd_h=1e-6, frozen=True)
    assert bad == -1
    assert np.max(np.abs(G - Gr) / np.abs(Jr)[:, None]) < 1e-7


def test_checkpoint_interval_does_not_change_results(gpu):
    U = torch.from_numpy(cells(8)).cuda()
    outs = [sens(gpu, "ignition_delay", k).adjoint(U, initial=True) for k in (1, 7, 40, 1000)]
    for J, G, G0 in outs[1:]:
        assert torch.equal(torch.nan_to_num(J), torch.nan_to_num(outs[0][0]))
        assert torch.equal(G, outs[0][1])
        assert torch.equal(G0, outs[0][2])


def test_initial_composition_gradient(gpu):
    # dJ/dY_k(0) at fixed rho and e (the last species closes the mass) against central
    # differences of the GPU objective: rho Y_k += rho d, rho Y_N2 -= rho d
    U = cells(4)
    s = sens(gpu, "ignition_delay")
    J, _, G0 = s.adjoint(torch.from_numpy(U).cuda(), initial=True)
    G0 = G0.cpu().numpy()
    rho = U[:9].sum(0)
    J = J.cpu().numpy()
    for k in (0, 1, 2):  # H2, O2 (central differences), H2O (absent: forward differences)
        d = 1e-7
        Up, Um = U.copy(), U.copy()
        Up[k] += rho * d
        Up[8] -= rho * d
        Um[k] -= rho * d
        Um[8] += rho * d
        Jp = s.objective(torch.from_numpy(Up).cuda()).cpu().numpy()
        if k < 2:
            Jm = s.objective(torch.from_numpy(Um).cuda()).cpu().numpy()
            fd, tol = (Jp - Jm) / (2 * d), 1e-4
        else:
            fd, tol = (Jp - J) / d, 1e-2
        ok = ~np.isnan(fd)
        assert ok.sum() >= 2
        assert np.max(np.abs(G0[k][ok] - fd[ok]) / np.abs(fd[ok])) < tol, k


def test_autograd_function(gpu):
    import hyperflow_gb300 as hf
    U = torch.from_numpy(cells(8)).cuda()
    s = sens(gpu, "ignition_delay")
    ln_mult = torch.zeros(21, dtype=torch.float64, requires_grad=True)
    J = hf.ChemObjective.apply(ln_mult, U, s)
    w = torch.nan_to_num(J.detach(), nan=0.0)
    (torch.nan_to_num(J, nan=0.0) * 1.0).sum().backward()
    _, G, _ = s.adjoint(U)
    assert torch.allclose(ln_mult.grad, torch.nan_to_num(G).sum(1).cpu(), rtol=1e-14, atol=0)
    assert w.abs().sum() > 0
