"""ctypes wrapper around the CPU oracle (``liboracle.so``).

Test infrastructure only: the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use it to check results.  The GPU package never
imports it.  States are AoS float64 arrays of shape (..., NS+3) in the
reference's component order (rhoY_0..rhoY_{NS-1}, rho*u, rho*v, rho*E).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

BC_REFLECTING, BC_TRANSMISSIVE, BC_INFLOW, BC_WEDGE = 0, 1, 2, 3
MAXV = 13
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("xlo", ctypes.c_double), ("ylo", ctypes.c_double),
                ("periodic", ctypes.c_int * 2), ("bc_lo", ctypes.c_int * 2), ("bc_hi", ctypes.c_int * 2),
                ("inlet", ctypes.c_double * MAXV), ("wedge_start", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("first_order_stages", ctypes.c_long), ("roundoff_repairs", ctypes.c_long),
                ("retries", ctypes.c_long), ("chem_failures", ctypes.c_long)]


def build():
    """Compile liboracle.so with the committed Makefile (g++ only)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.or_set_species.argtypes = [ctypes.c_int]
        L.or_molecular_weight.restype = ctypes.c_double
        L.or_mix_e.restype = ctypes.c_double
        L.or_mix_e.argtypes = [_dp, ctypes.c_double]
        L.or_mix_cv.restype = ctypes.c_double
        L.or_mix_cv.argtypes = [_dp, ctypes.c_double]
        L.or_species_thermo.argtypes = [ctypes.c_double, _dp, _dp, _dp]
        L.or_properties.argtypes = [_dp, ctypes.c_int64, _dp, _dp, _dp, _ip]
        L.or_hllc.argtypes = [_dp, _dp, ctypes.c_int, _dp, _dp, _dp]
        L.or_minmod.argtypes = [_dp, _dp, _dp, ctypes.c_int]
        L.or_net_production.argtypes = [ctypes.c_double, _dp, _dp]
        L.or_progress.argtypes = [ctypes.c_double, _dp, _dp, _dp, _dp, _dp]
        L.or_chem_rhs.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]
        L.or_chem_jac.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, ctypes.c_int]
        L.or_chem_advance.argtypes = [_dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_long, _lp]
        L.or_chem_batch_stats.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, _dp, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int, _lp, _lp]
        L.or_chem_flops.argtypes = [ctypes.c_double, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_int, _dp]
        L.or_flux_flops.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp]
        L.or_chem_batch.restype = ctypes.c_int64
        L.or_chem_batch.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, _dp, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, _lp]
        L.or_rodas4_circle.argtypes = [_dp, ctypes.c_double, ctypes.c_int]
        L.or_set_rate_mult.argtypes = [_dp]
        L.or_set_flux_threads.argtypes = [ctypes.c_int]
        L.or_run_record.restype = ctypes.c_void_p
        L.or_run_record.argtypes = [ctypes.POINTER(Grid), _dp, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int]
        L.or_run_replay.argtypes = [ctypes.c_void_p, ctypes.POINTER(Grid), _dp, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int]
        L.or_run_free.argtypes = [ctypes.c_void_p]
        L.or_chem_objective.restype = ctypes.c_int64
        L.or_chem_objective.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, ctypes.c_int, _dp]
        L.or_chem_sens_fd.restype = ctypes.c_int64
        L.or_chem_sens_fd.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, _dp, _dp]
        L.or_fill_ghosts.argtypes = [ctypes.POINTER(Grid), _dp]
        L.or_euler_stage.argtypes = [ctypes.POINTER(Grid), _dp, _dp, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.or_repair_roundoff.argtypes = [ctypes.POINTER(Grid), _dp, _lp]
        L.or_validate.argtypes = [ctypes.POINTER(Grid), _dp]
        L.or_flow.argtypes = [ctypes.POINTER(Grid), _dp, ctypes.c_double, ctypes.POINTER(Stats)]
        L.or_react.argtypes = [ctypes.POINTER(Grid), _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.or_cfl_dt.restype = ctypes.c_double
        L.or_cfl_dt.argtypes = [ctypes.POINTER(Grid), _dp, ctypes.c_double]
        L.or_strang_step.argtypes = [ctypes.POINTER(Grid), _dp, _dp, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, ctypes.POINTER(Stats)]
        L.or_interp_cell.restype = ctypes.c_double
        L.or_interp_cell.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def set_species(ns):
    if lib().or_set_species(ns) != 0:
        raise ValueError("species count must be 9 or 10")


def nspecies():
    return lib().or_nspecies()


def molecular_weights():
    return np.array([lib().or_molecular_weight(k) for k in range(nspecies())])


def species_thermo(T):
    ns = nspecies()
    cp, h, s = np.zeros(ns), np.zeros(ns), np.zeros(ns)
    lib().or_species_thermo(float(T), _p(cp), _p(h), _p(s))
    return cp, h, s


def mix_e(Y, T):
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    return lib().or_mix_e(_p(Y), float(T))


def mix_cv(Y, T):
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    return lib().or_mix_cv(_p(Y), float(T))


def properties(q):
    """Batched physics.cpp:4-15; returns (p, a, T, status) with status 1 = inadmissible."""
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, nspecies() + 3)
    n = len(q)
    p, a, T = np.zeros(n), np.zeros(n), np.zeros(n)
    st = np.zeros(n, dtype=np.int32)
    lib().or_properties(_p(q), n, _p(p), _p(a), _p(T), st.ctypes.data_as(_ip))
    return p, a, T, st


def hllc(l, r, n, pl, pr):
    l = np.ascontiguousarray(l, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    pl = np.ascontiguousarray(pl, dtype=np.float64)
    pr = np.ascontiguousarray(pr, dtype=np.float64)
    out = np.zeros(nspecies() + 3)
    lib().or_hllc(_p(l), _p(r), int(n), _p(pl), _p(pr), _p(out))
    return out


def minmod(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros_like(a)
    lib().or_minmod(_p(a), _p(b), _p(out), a.size)
    return out


def net_production(T, C):
    C = np.ascontiguousarray(C, dtype=np.float64)
    w = np.zeros(nspecies())
    lib().or_net_production(float(T), _p(C), _p(w))
    return w


def progress(T, C):
    C = np.ascontiguousarray(C, dtype=np.float64)
    kf, kr, qf, qr = (np.zeros(21) for _ in range(4))
    lib().or_progress(float(T), _p(C), _p(kf), _p(kr), _p(qf), _p(qr))
    return kf, kr, qf, qr


def chem_rhs(rho, e, y, T_guess=1000.0):
    y = np.ascontiguousarray(y, dtype=np.float64)
    T = np.array([T_guess])
    dy = np.zeros(nspecies() - 1)
    st = lib().or_chem_rhs(float(rho), float(e), _p(y), _p(T), _p(dy))
    return dy, float(T[0]), st


def chem_jac(rho, e, y, T_guess=1000.0, fd=False):
    y = np.ascontiguousarray(y, dtype=np.float64)
    T = np.array([T_guess])
    n = nspecies() - 1
    J = np.zeros(n * n)
    st = lib().or_chem_jac(float(rho), float(e), _p(y), _p(T), _p(J), int(fd))
    return J.reshape(n, n), st


def chem_advance(u, dt, rtol=1e-8, atol=1e-15, max_steps=5000):
    """One cell through chemistry.cpp:55-76; returns (new state, status, attempts)."""
    u = np.array(u, dtype=np.float64)
    steps = ctypes.c_long(0)
    st = lib().or_chem_advance(_p(u), float(dt), float(rtol), float(atol), int(max_steps), ctypes.byref(steps))
    return u, st, steps.value


def chem_batch(U, dt, rtol=1e-8, atol=1e-15, threads=0, dt_cell=None):
    """chemistry_batch.cpp:21-50 over AoS cells; returns (U_new, first_failed or -1, attempts)."""
    U = np.ascontiguousarray(np.array(U, dtype=np.float64).reshape(-1, nspecies() + 3))
    steps = np.zeros(len(U), dtype=np.int64)
    dtc = None if dt_cell is None else np.ascontiguousarray(dt_cell, dtype=np.float64)
    bad = lib().or_chem_batch(_p(U), len(U), float(dt), None if dtc is None else _p(dtc), float(rtol),
                              float(atol), int(threads), steps.ctypes.data_as(_lp))
    return U, int(bad), steps


OBJECTIVES = {"ignition_delay": 0, "peak_pressure": 1, "final_T": 2}


def chem_batch_stats(U, dt, rtol=1e-8, atol=1e-15, threads=0, dt_cell=None):
    """Accepted and rejected Rodas4 steps per cell of a (count, NV) AoS batch advanced
    over dt (or dt_cell per cell); -1 accepted marks a failed cell.  U is unchanged."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    n = U.shape[0]
    acc, rej = np.zeros(n, np.int64), np.zeros(n, np.int64)
    dtc = None if dt_cell is None else np.ascontiguousarray(dt_cell, dtype=np.float64)
    lib().or_chem_batch_stats(_p(U), n, float(dt), _p(dtc) if dtc is not None else None, float(rtol), float(atol),
                              int(threads), acc.ctypes.data_as(_lp), rej.ctypes.data_as(_lp))
    return acc, rej


def chem_flops(u, newton=3):
    """FP64 flops and transcendental calls of one chemistry right-hand side and one
    analytic Jacobian at the AoS state u, the UV inversion fixed at `newton` iterations
    from the state's own temperature: (rhs_flops, rhs_trans, jac_flops, jac_trans)."""
    u = np.asarray(u, dtype=np.float64)
    ns = nspecies()
    rho = float(u[:ns].sum())
    e = float(u[ns + 2] / rho - 0.5 * ((u[ns] / rho) ** 2 + (u[ns + 1] / rho) ** 2))
    T = float(properties(u[None, :])[2][0])
    y = np.ascontiguousarray(u[:ns - 1] / rho)
    out = np.zeros(4)
    lib().or_chem_flops(rho, e, _p(y), T, int(newton), _p(out))
    return tuple(out)


def flux_flops(stencil, direction=0, newton=3):
    """FP64 flops of the flux path at a 4-cell stencil (4 x NV AoS states along
    `direction`), every UV inversion fixed at `newton` iterations from 1000 K:
    {"face": one face (MUSCL, 2 EOS, HLLC), "cell": one cell's update and validation,
    "combine": one cell's Heun combine, "face_transcendental": calls per face}."""
    st = np.ascontiguousarray(np.asarray(stencil, dtype=np.float64).reshape(4, -1))
    out = np.zeros(4)
    lib().or_flux_flops(_p(st), int(direction), int(newton), _p(out))
    return {"face": out[0], "cell": out[1], "combine": out[2], "face_transcendental": out[3]}


def set_flux_threads(threads=1):
    """Threads of the flux, update and validation loops (1: the reference's serial
    loops; 0: all host threads).  Results do not depend on it."""
    lib().or_set_flux_threads(int(threads))


def set_rate_mult(mult=None):
    """Rate multipliers (NR) for every later oracle call; None resets them."""
    if mult is None:
        lib().or_set_rate_mult(None)
    else:
        m = np.ascontiguousarray(mult, dtype=np.float64)
        lib().or_set_rate_mult(_p(m))


def chem_objective(U, dt, nsub, objective, dT=400.0, rtol=1e-8, atol=1e-15, mult=None, threads=0):
    """Objective of AoS 0D cells over nsub adaptive chemistry calls of dt each;
    mult: rate multipliers (NR) or None.  Returns (J, first_failed or -1)."""
    U = np.ascontiguousarray(np.array(U, dtype=np.float64).reshape(-1, nspecies() + 3))
    J = np.zeros(len(U))
    m = None if mult is None else np.ascontiguousarray(mult, dtype=np.float64)
    bad = lib().or_chem_objective(_p(U), len(U), float(dt), int(nsub), OBJECTIVES[objective], float(dT),
                                  float(rtol), float(atol), None if m is None else _p(m), int(threads), _p(J))
    return J, int(bad)


def chem_sens_fd(U, dt, nsub, objective, dT=400.0, rtol=1e-8, atol=1e-15, fd_h=1e-6, frozen=True, threads=0):
    """Central differences dJ/d(ln multiplier_r) (count, NR); frozen replays the
    unperturbed accepted step sequence.  Returns (J, grad, first_failed or -1)."""
    U = np.ascontiguousarray(np.array(U, dtype=np.float64).reshape(-1, nspecies() + 3))
    J = np.zeros(len(U))
    G = np.zeros((len(U), 21))
    bad = lib().or_chem_sens_fd(_p(U), len(U), float(dt), int(nsub), OBJECTIVES[objective], float(dT), float(rtol),
                                float(atol), float(fd_h), int(bool(frozen)), int(threads), _p(J), _p(G))
    return J, G, int(bad)


class FrozenRun:
    """Strang steps with given step sizes on a one-level grid whose chemistry calls
    record their accepted step sizes; replay() re-runs them with those steps frozen
    (the map a discrete adjoint of the run differentiates).  U: ghosted AoS array."""

    def __init__(self, g, U, dts, rtol=1e-8, atol=1e-15, threads=0):
        self.g, self.rtol, self.atol, self.threads = g, rtol, atol, threads
        self.U = np.ascontiguousarray(U, dtype=np.float64).copy()
        d = np.ascontiguousarray(dts, dtype=np.float64)
        self.h = lib().or_run_record(ctypes.byref(g), _p(self.U), len(d), _p(d), float(rtol), float(atol),
                                     int(threads))
        if not self.h:
            raise RuntimeError("oracle run failed")

    def replay(self, U):
        V = np.ascontiguousarray(U, dtype=np.float64).copy()
        if lib().or_run_replay(self.h, ctypes.byref(self.g), _p(V), float(self.rtol), float(self.atol),
                               int(self.threads)):
            raise RuntimeError("oracle replay failed")
        return V

    def close(self):
        if self.h:
            lib().or_run_free(self.h)
            self.h = None


def rodas4_circle(y, tend, nsteps):
    y = np.array(y, dtype=np.float64)
    lib().or_rodas4_circle(_p(y), float(tend), int(nsteps))
    return y


def make_grid(nx, ny, dx, dy, xlo=0.0, ylo=0.0, periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0),
              inlet=None, wedge_start=0.0):
    g = Grid()
    g.nx, g.ny, g.dx, g.dy, g.xlo, g.ylo = nx, ny, dx, dy, xlo, ylo
    g.periodic[0], g.periodic[1] = periodic
    g.bc_lo[0], g.bc_lo[1] = bc_lo
    g.bc_hi[0], g.bc_hi[1] = bc_hi
    if inlet is not None:
        for n, v in enumerate(inlet):
            g.inlet[n] = float(v)
    g.wedge_start = wedge_start
    return g


def ghosted(interior):
    """(ny, nx, nv) interior -> (ny+4, nx+4, nv) ghosted array (ghosts NaN)."""
    ny, nx, nv = interior.shape
    U = np.full((ny + 4, nx + 4, nv), np.nan)
    U[2:-2, 2:-2] = interior
    return U


def fill_ghosts(g, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    lib().or_fill_ghosts(ctypes.byref(g), _p(U))
    return U


def euler_stage(g, Ug, h, first_order=False):
    Ug = np.ascontiguousarray(Ug, dtype=np.float64)
    out = Ug.copy()
    nv = Ug.shape[-1]
    fx = np.zeros((g.ny, g.nx + 1, nv))
    fy = np.zeros((g.ny + 1, g.nx, nv))
    st = lib().or_euler_stage(ctypes.byref(g), _p(Ug), _p(out), float(h), int(first_order), _p(fx), _p(fy))
    return out, fx, fy, st


def repair_roundoff(g, U):
    """repairRoundoff (BlockAMR.cpp:299-334) of a one-level ghosted state (every cell a
    leaf): (repaired copy, status 0 ok / 1 material or insufficient donor, zeroed count)."""
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    n = ctypes.c_long(0)
    st = lib().or_repair_roundoff(ctypes.byref(g), _p(U), ctypes.byref(n))
    return U, st, n.value


def flow(g, U, h):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    s = Stats()
    st = lib().or_flow(ctypes.byref(g), _p(U), float(h), ctypes.byref(s))
    return U, st, s


def cfl_dt(g, U, cfl):
    U = np.ascontiguousarray(U, dtype=np.float64)
    return lib().or_cfl_dt(ctypes.byref(g), _p(U), float(cfl))


def strang_step(g, U, dt, chemistry=True, rtol=1e-8, atol=1e-15, threads=0):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    d = np.array([dt], dtype=np.float64)
    s = Stats()
    st = lib().or_strang_step(ctypes.byref(g), _p(U), _p(d), int(chemistry), float(rtol), float(atol),
                              int(threads), ctypes.byref(s))
    return U, float(d[0]), st, s


def interp_cell(q, xm, xp, ym, yp):
    args = [np.ascontiguousarray(v, dtype=np.float64) for v in (q, xm, xp, ym, yp)]
    out = np.zeros((4, len(args[0])))
    theta = lib().or_interp_cell(*[_p(a) for a in args], _p(out))
    return out, theta


SPECIES = ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2", "AR"]
GAS_CONSTANT = 8314.46261815324


def composition(spec, kind="X"):
    """'H2:2,O2:1,N2:3.76' -> normalised vector over the active species."""
    ns = nspecies()
    v = np.zeros(ns)
    for part in spec.split(","):
        name, val = part.split(":")
        v[SPECIES.index(name.strip())] = float(val)
    return v / v.sum()


def primitive(T, p, X=None, Y=None, u=0.0, v=0.0):
    """BlockAMR.cpp:20-24 (state from T, p and mole or mass fractions), restated."""
    W = molecular_weights()
    if Y is None:
        X = np.asarray(X, dtype=np.float64)
        Y = X * W / np.sum(X * W)
    Y = np.asarray(Y, dtype=np.float64)
    rho = p / (GAS_CONSTANT * T * np.sum(Y / W))
    e = mix_e(Y, T)
    q = np.zeros(len(W) + 3)
    q[:len(W)] = rho * Y
    q[len(W)] = rho * u
    q[len(W) + 1] = rho * v
    q[len(W) + 2] = rho * (e + 0.5 * (u * u + v * v))
    return q


# ---------------------------------------------------------------- block-AMR operations
class TagCriteria(ctypes.Structure):
    _fields_ = [("pressure_tag", ctypes.c_double), ("temperature_tag", ctypes.c_double),
                ("fuel_rate_tag", ctypes.c_double), ("density_tag", ctypes.c_double),
                ("chemistry", ctypes.c_int), ("box_only", ctypes.c_int), ("has_box", ctypes.c_int),
                ("box", ctypes.c_double * 4), ("velocity", ctypes.c_double * 2)]


def _amr_sigs():
    L = lib()
    if getattr(L, "_amr", False):
        return L
    L.or_totals.argtypes = [_dp, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _dp]
    L.or_average_down.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp]
    L.or_reflux.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_int), _dp, ctypes.POINTER(ctypes.c_int64), _dp,
                            ctypes.POINTER(ctypes.c_int64), ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.or_tag.restype = ctypes.c_int
    L.or_tag.argtypes = [ctypes.POINTER(Grid), _dp, ctypes.c_double, ctypes.POINTER(TagCriteria),
                         ctypes.POINTER(ctypes.c_ubyte)]
    L._amr = True
    return L


def totals(cells, vol, mask=None, absolute=False):
    """BlockAMR.cpp:347-355 over AoS cells (n, NV); mask: (n,) bytes or None."""
    cells = np.ascontiguousarray(cells, dtype=np.float64)
    out = np.zeros(cells.shape[-1])
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    _amr_sigs().or_totals(_p(cells), len(cells), None if m is None else m.ctypes.data, float(vol), int(absolute),
                          _p(out))
    return out


def average_down(fine):
    """(nyf, nxf, NV) -> (nyf/2, nxf/2, NV)."""
    fine = np.ascontiguousarray(fine, dtype=np.float64)
    nyf, nxf, nv = fine.shape
    out = np.zeros((nyf // 2, nxf // 2, nv))
    _amr_sigs().or_average_down(_p(fine), nxf, nyf, _p(out))
    return out


def reflux(Uc, fxc, fyc, boxes, fxf_list, fyf_list, h, dxc, dyc, periodic=(0, 0)):
    """Uc (nyc, nxc, NV) after reflux; boxes: [(filo, fjlo, fihi, fjhi)], fine face fluxes per box."""
    Uc = np.ascontiguousarray(Uc, dtype=np.float64).copy()
    nyc, nxc, nv = Uc.shape
    fx = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel() for a in fxf_list])
    fy = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel() for a in fyf_list])
    xo = np.cumsum([0] + [a.size for a in fxf_list[:-1]]).astype(np.int64)
    yo = np.cumsum([0] + [a.size for a in fyf_list[:-1]]).astype(np.int64)
    b = np.ascontiguousarray(np.array(boxes, dtype=np.int32).ravel())
    fxc = np.ascontiguousarray(fxc, dtype=np.float64)
    fyc = np.ascontiguousarray(fyc, dtype=np.float64)
    _amr_sigs().or_reflux(_p(Uc), nxc, nyc, int(periodic[0]), int(periodic[1]), _p(fxc), _p(fyc), len(boxes),
                          b.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(fx),
                          xo.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _p(fy),
                          yo.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), float(h), float(dxc), float(dyc))
    return Uc


def tag(g, Ug, t, crit):
    """BlockAMR::ErrorEst on a ghosted level; returns ((ny, nx) uint8 tags, status)."""
    Ug = np.ascontiguousarray(Ug, dtype=np.float64)
    tags = np.zeros((g.ny, g.nx), dtype=np.uint8)
    st = _amr_sigs().or_tag(ctypes.byref(g), _p(Ug), float(t), ctypes.byref(crit),
                            tags.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    return tags, st
