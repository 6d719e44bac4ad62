"""Seeded synthetic workloads (initial conditions) of the benchmark configurations.

  det1d  : planar detonation, 2000 x 2 cells on 0.1 m (dx = 5e-5 m), H2/O2 with 70% (mole)
           diluent at 1 atm / 298 K, a 20-cell driver at 40 atm / 3000 K; reflecting left,
           transmissive right, reflecting top/bottom (the sun_cj case layout).
  det2d  : cellular detonation, 2048 x 512 cells, dx = 1e-4 m (0.2048 m x 0.0512 m),
           same mixture, a 64-column hot band at 40 atm / 3000 K, density perturbed by a
           seeded U(-1%, +1%) in those columns; periodic in y, reflecting left, transmissive
           right.
  chem   : 2^20 independent cells, T ~ U[800, 2500] K, p ~ logU[0.1, 10] atm,
           phi ~ logU[0.3, 3], diluent ~ U[0, 0.8], dt ~ logU[1e-7, 1e-6] s.
  ignition: 4096 0D cells of H2/air (O2 : N2 = 1 : 3.76, the reference's 9 species),
           T ~ U[1000, 1500] K, p ~ U[1, 5] atm, phi ~ U[0.5, 2], for the sensitivity
           (adjoint) runs.
  sun_cj, teng_case1: the reference's two case configurations
           (HyperFlow_V3/cases/sun_cj/smoke.json, cases/teng_case1/smoke.json) as one
           uniform level at their finest resolution.
  blast2d, entropy_wave: the blast and moving-refinement checks of
           HyperFlow_V3/tests/validate.py as one uniform level at their finest resolution.
The diluent is argon (the inert AR extension species, 10-species mechanism) unless
diluent="N2" is asked for (9 species, the reference mechanism as is).
"""
import numpy as np

from . import mechanism as M


def _ns(diluent):
    return 10 if diluent.upper() == "AR" else 9


def detonation(nx, ny, dx, hot_columns, seed=0, diluent="AR", dilution=0.7, T0=298.0, p0=101325.0, T_hot=3000.0,
               p_hot=40 * 101325.0, perturb=0.01):
    """(NV, ny, nx) initial state: fresh mixture with a hot band in the first columns."""
    ns = _ns(diluent)
    X = M.mixture_X(1.0, dilution, "AR" if ns == 10 else "N2", ns)
    fresh = M.primitive(T0, p0, X=X, ns=ns)
    hot = M.primitive(T_hot, p_hot, X=X, ns=ns)
    U = np.empty((ns + 3, ny, nx))
    U[:] = fresh[:, None, None]
    U[:, :, :hot_columns] = hot[:, None, None]
    if perturb:
        rng = np.random.default_rng(seed)
        f = 1.0 + rng.uniform(-perturb, perturb, size=(ny, hot_columns))
        U[:, :, :hot_columns] *= f[None]
    return U, fresh


def det2d(seed=0, diluent="AR", nx=2048, ny=512, hot_columns=64):
    U, fresh = detonation(nx, ny, 1e-4, hot_columns=min(hot_columns, nx), seed=seed, diluent=diluent)
    level = dict(nx=nx, ny=ny, dx=1e-4, dy=1e-4, periodic=(0, 1), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("transmissive", "reflecting"), inlet=fresh)
    return U, level


def det1d(diluent="AR", nx=2000):
    U, fresh = detonation(nx, 2, 0.1 / nx, hot_columns=20, perturb=0.0, diluent=diluent)
    level = dict(nx=nx, ny=2, dx=0.1 / nx, dy=0.1 / nx, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("transmissive", "reflecting"), inlet=fresh)
    return U, level


def chem_batch(n=1 << 20, seed=0, diluent="AR"):
    """(NV, n) states and (n,) intervals of independent 0D cells."""
    ns = _ns(diluent)
    rng = np.random.default_rng(seed)
    T = rng.uniform(800.0, 2500.0, n)
    p = 101325.0 * np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))
    phi = np.exp(rng.uniform(np.log(0.3), np.log(3.0), n))
    dil = rng.uniform(0.0, 0.8, n)
    dt = np.exp(rng.uniform(np.log(1e-7), np.log(1e-6), n))
    W = M.MW[:ns]
    dsp = M.SPECIES.index("AR" if ns == 10 else "N2")
    X = np.zeros((n, ns))
    X[:, 0] = 2.0 * phi
    X[:, 1] = 1.0
    X[:, :2] *= ((1.0 - dil) / X[:, :2].sum(1))[:, None]
    X[:, dsp] += dil
    if ns == 9:
        # air-like nitrogen when the diluent is nitrogen: keep at least 3.76 N2 per O2 mole
        pass
    return _cells_at_rest(T, p, X, ns), dt


def _cells_at_rest(T, p, X, ns):
    """(NV, n) conserved states at rest from temperatures, pressures and mole fractions."""
    W = M.MW[:ns]
    n = len(T)
    Y = X * W / (X * W).sum(1, keepdims=True)
    rho = p / (M.GAS_CONSTANT * T * (Y / W).sum(1))
    e = np.empty(n)
    lo, hi = M.NASA_LOW[:ns], M.NASA_HIGH[:ns]
    for sel, a in ((T <= 1000.0, lo), (T > 1000.0, hi)):
        t = T[sel][:, None]
        hRT = a[:, 0] + t * (a[:, 1] / 2 + t * (a[:, 2] / 3 + t * (a[:, 3] / 4 + t * a[:, 4] / 5))) + a[:, 5] / t
        e[sel] = M.GAS_CONSTANT * T[sel] * ((Y[sel] / W) * (hRT - 1.0)).sum(1)
    U = np.zeros((ns + 3, n))
    U[:ns] = (rho[:, None] * Y).T
    U[ns + 2] = rho * e
    return U


def ignition_batch(n=4096, seed=0):
    """(NV, n) H2/air 0D cells (9 species): T ~ U[1000,1500] K, p ~ U[1,5] atm, phi ~ U[0.5,2]."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(1000.0, 1500.0, n)
    p = 101325.0 * rng.uniform(1.0, 5.0, n)
    phi = rng.uniform(0.5, 2.0, n)
    X = np.zeros((n, 9))
    X[:, M.SPECIES.index("H2")] = 2.0 * phi
    X[:, M.SPECIES.index("O2")] = 1.0
    X[:, M.SPECIES.index("N2")] = 3.76
    return _cells_at_rest(T, p, X, 9)


def wedge(nx=512, ny=256, mach=7.0, angle_deg=30.0, T0=300.0, p0=0.1 * 101325.0, length=0.032, x_tip=0.004):
    """Oblique detonation over a wedge: stoichiometric H2/air (9 species) at p0 / T0 moving
    at `mach` times its sound speed, rotated by angle_deg toward the bottom wall
    (u0 = V cos a, v0 = -V sin a, the teng_osw convention of BlockAMR.cpp:61-66); the
    bottom is the wedge surface from x = 0 on (x_tip cells of length upstream of the tip
    keep a zero-gradient bottom), inflow at the left and top, transmissive on the right.
    Returns (U (NV, ny, nx), level keys)."""
    ns = 9
    X = np.zeros(ns)
    X[M.SPECIES.index("H2")], X[M.SPECIES.index("O2")], X[M.SPECIES.index("N2")] = 2.0, 1.0, 3.76
    X /= X.sum()
    W = M.MW[:ns]
    a_lo = M.NASA_LOW[:ns]
    cpR = float(np.sum(X * (a_lo[:, 0] + T0 * (a_lo[:, 1] + T0 * (a_lo[:, 2] + T0 * (a_lo[:, 3] + T0 * a_lo[:, 4]))))))
    gam = cpR / (cpR - 1.0)
    a = np.sqrt(gam * M.GAS_CONSTANT * T0 / float(np.sum(X * W)))
    V = mach * a
    th = np.radians(angle_deg)
    q = M.primitive(T0, p0, X=X, u=V * np.cos(th), v=-V * np.sin(th), ns=ns)
    dx = length / nx
    U = np.empty((ns + 3, ny, nx))
    U[:] = q[:, None, None]
    level = dict(nx=nx, ny=ny, dx=dx, dy=dx, xlo=-x_tip, ylo=0.0, periodic=(0, 0),
                 boundary_lo=("inflow", "wedge"), boundary_hi=("transmissive", "inflow"), inlet=q, wedge_start=0.0)
    return U, level


def _air_X(ns=9):
    """H2:2, O2:1, N2:3.76 by mole, normalised."""
    X = np.zeros(ns)
    X[M.SPECIES.index("H2")], X[M.SPECIES.index("O2")], X[M.SPECIES.index("N2")] = 2.0, 1.0, 3.76
    return X / X.sum()


def sun_cj(nx=25000, ny=8):
    """The Sun-CJ smoke case as one level at its finest resolution (base 6250 x 2 cells on
    0.5 m x 1.0 m, two levels of ratio 2: dx = 2e-5 m, dy = 0.125 m).  Stoichiometric H2/air
    at rest at 1 atm / 300 K with a 2 mm hot spot at 90 atm / 3000 K against the reflecting
    left wall: a cell is hot by the fraction clamp((w - (x - dx/2)) / dx, 0, 1) of its
    centre x (HyperFlow_V3/src/BlockAMR.cpp:75,87-90, cases/sun_cj/smoke.json); transmissive
    right, reflecting top and bottom; CFL 0.5 to 1e-7 s.  nx < 25000 keeps the leading
    nx x 2e-5 m of the domain.  By 1e-7 s the disturbance has reached x = 2.44 mm; every
    cell beyond it holds the far-field state (at rest, evolving only by its own chemistry),
    so a cut well past that point leaves the run unchanged.
    Returns (U (NV, ny, nx), level keys, case dict)."""
    dx = 0.5 / 25000
    dy = 1.0 / ny
    X = _air_X()
    fresh = M.primitive(300.0, 101325.0, X=X, ns=9)
    hot = M.primitive(3000.0, 90.0 * 101325.0, X=X, ns=9)
    U = np.empty((12, ny, nx))
    for i in range(nx):
        x = (i + 0.5) * dx
        f = min(max((0.002 - (x - 0.5 * dx)) / dx, 0.0), 1.0)
        U[:, :, i] = (f * hot + (1.0 - f) * fresh)[:, None]
    level = dict(nx=nx, ny=ny, dx=dx, dy=dy, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("transmissive", "reflecting"), inlet=fresh)
    return U, level, dict(cfl=0.5, end_time=1e-7)


def teng_case1(refine=4):
    """The Teng oblique-detonation case 1 smoke configuration as one level: base 144 x 64
    cells on 2.304 mm x 1.024 mm from x = -0.128 mm, refined by `refine` (4 = its two
    levels of ratio 2: dx = dy = 4e-6 m).  Stoichiometric H2/air at 958.1 K / 1.2029 MPa
    moving at 2737.7 m/s turned 19 degrees toward the wedge (u0 = V cos a, v0 = -V sin a,
    HyperFlow_V3/src/BlockAMR.cpp:61-66, cases/teng_case1/smoke.json); inflow left and top,
    wedge bottom from x = 0, transmissive right; CFL 0.6 to 2e-9 s.
    Returns (U (NV, ny, nx), level keys, case dict)."""
    nx, ny = 144 * refine, 64 * refine
    angle = 19.0 * np.arccos(-1.0) / 180.0
    q = M.primitive(958.1, 1202900.0, X=_air_X(), u=2737.7 * np.cos(angle), v=-2737.7 * np.sin(angle), ns=9)
    U = np.empty((12, ny, nx))
    U[:] = q[:, None, None]
    level = dict(nx=nx, ny=ny, dx=0.002304 / nx, dy=0.001024 / ny, xlo=-0.000128, ylo=0.0, periodic=(0, 0),
                 boundary_lo=("inflow", "wedge"), boundary_hi=("transmissive", "inflow"), inlet=q, wedge_start=0.0)
    return U, level, dict(cfl=0.6, end_time=2e-9)


def blast2d(reacting=True):
    """A disc of stoichiometric H2/air at 1500 K / 10 atm in the same mixture at rest at
    300 K / 1 atm, closed by reflecting walls; each cell is the 4 x 4-point average of the
    disc indicator (HyperFlow_V3/src/BlockAMR.cpp:69,97-121).  One level at the finest
    resolution of the reference's checks:
      reacting=False: tests/validate.py:122-129, 0.02 m square, base 24 x 24 with two
                      levels (96 x 96), centre (0.01, 0.01), radius 2 mm, no chemistry,
                      output at 1e-6 and 2e-6 s;
      reacting=True:  tests/validate.py:174-179, 0.01 m square, base 16 x 16 with one
                      level (32 x 32), centre (0.005, 0.005), radius 1.5 mm, chemistry,
                      output at 1e-7 and 2e-7 s.
    CFL 0.6.  Returns (U (NV, n, n), level keys, case dict)."""
    if reacting:
        n, length, centre, radius, times = 32, 0.01, 0.005, 0.0015, [1e-7, 2e-7]
    else:
        n, length, centre, radius, times = 96, 0.02, 0.01, 0.002, [1e-6, 2e-6]
    X = _air_X()
    fresh = M.primitive(300.0, 101325.0, X=X, ns=9)
    hot = M.primitive(1500.0, 10.0 * 101325.0, X=X, ns=9)
    dx = length / n
    quad = 4
    U = np.empty((12, n, n))
    for j in range(n):
        for i in range(n):
            x, y = (i + 0.5) * dx, (j + 0.5) * dx
            acc = np.zeros(12)
            for b in range(quad):
                for a in range(quad):
                    xx = x + dx * ((a + 0.5) / quad - 0.5)
                    yy = y + dx * ((b + 0.5) / quad - 0.5)
                    acc += hot if np.hypot(xx - centre, yy - centre) < radius else fresh
            U[:, j, i] = acc / (quad * quad)
    level = dict(nx=n, ny=n, dx=dx, dy=dx, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("reflecting", "reflecting"), inlet=fresh)
    return U, level, dict(cfl=0.6, end_time=times[-1], output_times=times, chemistry=reacting)


def entropy_wave():
    """A Gaussian temperature dip (T = 300 K / (1 + 0.2 exp(-r^2 / sigma^2)), sigma 0.7 mm,
    centre (3 mm, 4 mm)) at 1 atm in stoichiometric H2/air moving at (300, 200) m/s through
    a periodic 0.01 m square; each cell is the 4 x 4-point average of the state
    (HyperFlow_V3/src/BlockAMR.cpp:97-110).  The moving-refinement check of
    tests/validate.py:104-119 (base 16 x 16 with two levels) on one level of 64 x 64 cells;
    no chemistry, CFL 0.6, output at 2e-6 and 4e-6 s.
    Returns (U (NV, 64, 64), level keys, case dict)."""
    n, length, quad = 64, 0.01, 4
    cx, cy, sigma, amp = 0.003, 0.004, 0.0007, 0.2
    X = _air_X()
    dx = length / n
    U = np.empty((12, n, n))
    for j in range(n):
        for i in range(n):
            x, y = (i + 0.5) * dx, (j + 0.5) * dx
            acc = np.zeros(12)
            for b in range(quad):
                for a in range(quad):
                    xx = x + dx * ((a + 0.5) / quad - 0.5)
                    yy = y + dx * ((b + 0.5) / quad - 0.5)
                    bump = 1.0 + amp * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (sigma * sigma))
                    acc += M.primitive(300.0 / bump, 101325.0, X=X, u=300.0, v=200.0, ns=9)
            U[:, j, i] = acc / (quad * quad)
    level = dict(nx=n, ny=n, dx=dx, dy=dx, periodic=(1, 1), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("transmissive", "reflecting"), inlet=M.primitive(300.0, 101325.0, X=X, ns=9))
    return U, level, dict(cfl=0.6, end_time=4e-6, output_times=[2e-6, 4e-6], chemistry=False)
