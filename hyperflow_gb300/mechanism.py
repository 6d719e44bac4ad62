"""Host-side mechanism data and state construction for setting up workloads.

Reads the generated table ``csrc/mech_h2li.h`` (species, molecular weights,
NASA7 coefficients) and restates ``primitive()`` of HyperFlow_V3/src/BlockAMR.cpp:20-24
(a conserved state from T, p and mole or mass fractions) in numpy.  Used to
build initial conditions; the hot path never calls it.
"""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GAS_CONSTANT = 8314.46261815324
ONE_ATM = 101325.0
SPECIES = ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2", "AR"]


def _table():
    text = open(os.path.join(HERE, "csrc", "mech_h2li.h")).read()

    def arr(name):
        m = re.search(r"constexpr double %s\[[^=]*= \{(.*?)\};" % name, text, re.S)
        return np.array([float(v) for v in re.findall(r"[-+]?\d+\.?\d*(?:e[-+]?\d+)?", m.group(1))])

    mw = arr("MW")
    lo = arr("NASA_LOW").reshape(-1, 7)
    hi = arr("NASA_HIGH").reshape(-1, 7)
    return mw, lo, hi


MW, NASA_LOW, NASA_HIGH = _table()


def _coef(T, ns):
    return np.where(T <= 1000.0, 1, 0), NASA_LOW[:ns], NASA_HIGH[:ns]


def species_e_RT(T, ns):
    """e_k/(R T) per unit mole, shape (ns,) for scalar T."""
    a = NASA_LOW[:ns] if T <= 1000.0 else NASA_HIGH[:ns]
    hRT = a[:, 0] + T * (a[:, 1] / 2 + T * (a[:, 2] / 3 + T * (a[:, 3] / 4 + T * a[:, 4] / 5))) + a[:, 5] / T
    return hRT - 1.0


def mix_e(Y, T):
    """specific internal energy (J/kg) of mass fractions Y at T."""
    ns = len(Y)
    return GAS_CONSTANT * T * float(np.sum(Y / MW[:ns] * species_e_RT(T, ns)))


def composition(spec, ns):
    """'H2:2,O2:1,N2:3.76' -> normalised vector over ns species."""
    v = np.zeros(ns)
    for part in spec.split(","):
        name, val = part.split(":")
        v[SPECIES.index(name.strip().upper() if name.strip().upper() == "AR" else name.strip())] += float(val)
    return v / v.sum()


def primitive(T, p, X=None, Y=None, u=0.0, v=0.0, ns=9):
    """Conserved state (NV,) from temperature, pressure and composition (BlockAMR.cpp:20-24)."""
    W = MW[:ns]
    if Y is None:
        X = np.asarray(X, dtype=np.float64)
        Y = X * W / np.sum(X * W)
    Y = np.asarray(Y, dtype=np.float64)
    rho = p / (GAS_CONSTANT * T * np.sum(Y / W))
    q = np.zeros(ns + 3)
    q[:ns] = rho * Y
    q[ns] = rho * u
    q[ns + 1] = rho * v
    q[ns + 2] = rho * (mix_e(Y, T) + 0.5 * (u * u + v * v))
    return q


def mixture_X(phi=1.0, diluent=0.7, diluent_species="AR", ns=10):
    """H2/O2 at equivalence ratio phi with a mole fraction `diluent` of an inert."""
    x = np.zeros(ns)
    x[0], x[1] = 2.0 * phi, 1.0
    x[:2] *= (1.0 - diluent) / x[:2].sum()
    x[SPECIES.index(diluent_species)] += diluent
    return x
