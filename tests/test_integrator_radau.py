"""The oracle's stiff integrator (Rodas4, the algorithm the GPU kernels run) against an
independent one on the same ODE: scipy's Radau IIA (order 5) on the oracle's
constant-(rho, e) right-hand side and analytic Jacobian, at rtol 1e-12 / atol 1e-20.
0D stoichiometric H2/air cells (the file's 9 species): two run to near equilibrium and
two end at their ignition point (T0 + 400 K), where T changes fastest.
- Rodas4 at the same tight tolerance agrees to rounding-level errors: the restated
  integrator converges to the ODE's solution.
- Rodas4 at the reference's tolerances (rtol 1e-8, atol 1e-15) stays within the
  reference's own bar for 0D chemistry against a tight integration
  (HyperFlow_V3/tests/validate.py:140-170: T relative 1e-7, Y absolute 1e-8), the
  CVODE BDF integrator it replaces being held to the same bar."""
import os
import sys

import numpy as np
import pytest

scipy_integrate = pytest.importorskip("scipy.integrate")
ROOT = os.path.join(os.path.dirname(__file__), "..")

CASES = [  # T0 (K), p (atm), dt (s)
    (1500.0, 1.0, 2e-4),
    (2000.0, 0.5, 5e-5),
    (1500.0, 1.0, 1.44e-5),  # the ignition point (T0 + 400 K at 1.441e-5 s)
    (1200.0, 5.0, 1.14e-5),  # the ignition point (1.138e-5 s)
]


@pytest.fixture(scope="module")
def O():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    oracle.set_species(9)
    return oracle


def radau(O, q, dt):
    rho = q[:9].sum()
    e = q[11] / rho
    Tg = [1000.0]

    def f(t, y):
        dy, T, _ = O.chem_rhs(rho, e, y, Tg[0])
        Tg[0] = T
        return dy

    def jac(t, y):
        return O.chem_jac(rho, e, y, Tg[0])[0]

    sol = scipy_integrate.solve_ivp(f, (0.0, dt), q[:8] / rho, method="Radau", rtol=1e-12, atol=1e-20, jac=jac)
    assert sol.success
    y = sol.y[:, -1]
    return y, O.chem_rhs(rho, e, y, Tg[0])[1]


@pytest.mark.parametrize("T0,p,dt", CASES)
def test_rodas4_against_radau(O, T0, p, dt):
    X = np.zeros(9)
    X[0], X[1], X[8] = 2.0, 1.0, 3.76
    q = O.primitive(T0, p * 101325.0, X=X / X.sum())
    rho = q[:9].sum()
    yR, TR = radau(O, q, dt)
    for rtol, atol, t_bar, y_bar in ((1e-12, 1e-20, 1e-11, 1e-11), (1e-8, 1e-15, 1e-7, 1e-8)):
        u, st, _ = O.chem_advance(q, dt, rtol=rtol, atol=atol, max_steps=200000)
        assert st == 0
        T = O.properties(u[None])[2][0]
        assert abs(T - TR) / TR < t_bar, (rtol, abs(T - TR) / TR)
        assert np.abs(u[:8] / rho - yR).max() < y_bar, (rtol, np.abs(u[:8] / rho - yR).max())
