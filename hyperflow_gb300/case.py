"""The reference's case configuration (the JSON object of HyperFlow V3's input files and
of its test scripts' configs) turned into what this package runs: the initial state of
a level, that level's keys for make_level, and the run options of run_case /
run_amr_case (HyperFlow_V3/src/main.cpp:15-35, src/BlockAMR.cpp:29-121, the ErrorEst keys
of :170-200 and the run loop's keys of :400-420).

The reference builds its finer levels by evaluating the initial condition at their
resolution; load(config, refine=r) evaluates it on the base grid refined 2^r times, so
that a case can also run on one level at its finest resolution.
"""
import numpy as np

from . import mechanism as M

AIR = "H2:2,O2:1,N2:3.76"
EX_FRESH = "H2:0.02852103,O2:0.226362,N2:0.745117"
EX_HOT = ("H:0.000247,O:0.001617,H2O:0.225404,OH:0.014915,O2:0.013336,H2:0.002429,H2O2:0.000002601600,"
          "HO2:0.00001857550,N2:0.742031")
PROBLEMS = ("uniform", "entropy_wave", "blast2d", "sod_x", "sod_y", "teng_osw", "sun_cj", "example6", "example7")


def primitive(T, p, comp, mole, u=0.0, v=0.0):
    """The conserved state of T, p and a composition string by mole (mole=True) or mass
    fractions, normalised (BlockAMR.cpp:20-24)."""
    f = M.composition(comp, 9)
    return M.primitive(T, p, X=f, u=u, v=v, ns=9) if mole else M.primitive(T, p, Y=f, u=u, v=v, ns=9)


def states(c):
    """(fresh, hot) states of the case (BlockAMR.cpp:61-77); raises on an unknown problem."""
    problem = c["problem"]
    if problem not in PROBLEMS:
        raise ValueError("unknown problem %r" % problem)
    u0, v0 = c.get("u0", 0.0), c.get("v0", 0.0)
    if problem == "teng_osw":
        speed, angle = c["inflow_speed"], c["wedge_angle_deg"]
        if not (speed > 0 and 0 < angle < 90):
            raise ValueError("invalid wedge inflow speed or angle")
        rad = angle * np.arccos(-1.0) / 180.0
        u0, v0 = speed * np.cos(rad), -speed * np.sin(rad)
    fresh = primitive(c.get("T0", 300.0), c.get("P0", 101325.0), AIR, True, u0, v0)
    hot = primitive(c.get("hot_T", 1500.0), c.get("hot_P", 10.0 * 101325.0), AIR, True)
    if problem in ("example6", "example7"):
        fresh = primitive(298.0, 101325.0, EX_FRESH, False)
        hot = primitive(2941.677242, 1481999.362037, EX_HOT, False, 800.0 if problem == "example6" else 2000.0)
    elif problem == "sun_cj":
        hot = primitive(3000.0, 90.0 * 101325.0, AIR, True)
    return fresh, hot


def initial(c, x, y, dx, dy, fresh, hot, length):
    """BlockAMR::initial (BlockAMR.cpp:84-121) of the cell centred at (x, y)."""
    problem = c["problem"]
    if problem in ("uniform", "teng_osw"):
        return fresh
    if problem == "sun_cj":
        f = min(max((c.get("hotspot_width", 0.002) - (x - 0.5 * dx)) / dx, 0.0), 1.0)
        return f * hot + (1 - f) * fresh
    if problem == "example6":
        f = min(max((0.4 - (x - 0.5 * dx)) / dx, 0.0), 1.0)
        return f * hot + (1 - f) * fresh
    if problem in ("sod_x", "sod_y"):
        axis = problem == "sod_x"
        centre, width = (x, dx) if axis else (y, dy)
        front = c.get("interface", 0.5 * length[0 if axis else 1])
        f = min(max((front - centre + 0.5 * width) / width, 0.0), 1.0)
        return f * hot + (1 - f) * fresh
    quad = c.get("initial_subsamples", 4)
    if quad < 1 or quad > 32:
        raise ValueError("invalid initial quadrature")
    centre = c.get("center", [0.3 * length[0], 0.5 * length[1]])
    if len(centre) != 2:
        raise ValueError("center must have two coordinates")
    acc = np.zeros_like(fresh)
    for b in range(quad):
        for a in range(quad):
            xx = x + dx * ((a + 0.5) / quad - 0.5)
            yy = y + dy * ((b + 0.5) / quad - 0.5)
            if problem == "entropy_wave":
                sigma = c.get("sigma", 0.08 * length[0])
                r2 = (xx - centre[0]) * (xx - centre[0]) + (yy - centre[1]) * (yy - centre[1])
                bump = 1 + c.get("amplitude", 0.2) * np.exp(-r2 / (sigma * sigma))
                acc += primitive(c.get("T0", 300.0) / bump, c.get("P0", 101325.0), AIR, True, c.get("u0", 0.0),
                                 c.get("v0", 0.0))
            else:
                if problem == "example7":
                    lower = min(yy, length[1] - yy)
                    front = max(0.5, 0.25 + lower)
                    inside = xx < front - 32 * np.finfo(np.float64).eps * length[0]
                else:
                    inside = np.hypot(xx - centre[0], yy - centre[1]) < c.get("radius", 0.1 * length[1])
                acc += hot if inside else fresh
    return acc / (quad * quad)


def load(c, refine=0):
    """(U0 (12, ny, nx) initial state, level keys, run options) of a case configuration
    on its base grid refined 2^refine times."""
    nc, length = c["base_cells"], c["length"]
    origin, periodic = c.get("origin", [0.0, 0.0]), c.get("periodic", [0, 0])
    if len(nc) != 2 or len(length) != 2 or len(origin) != 2 or len(periodic) != 2:
        raise ValueError("base_cells, length, origin and periodic take two values")
    if not (c["end_time"] > 0 and 0 < c.get("cfl", 0.6) <= 0.8):
        raise ValueError("invalid CFL or final time")
    fresh, hot = states(c)
    nx, ny = nc[0] << refine, nc[1] << refine
    dx, dy = length[0] / nc[0] / (1 << refine), length[1] / nc[1] / (1 << refine)
    U = np.empty((12, ny, nx))
    for j in range(ny):
        for i in range(nx):
            U[:, j, i] = initial(c, origin[0] + (i + 0.5) * dx, origin[1] + (j + 0.5) * dy, dx, dy, fresh, hot,
                                 length)
    level = dict(nx=nx, ny=ny, dx=dx, dy=dy, xlo=origin[0], ylo=origin[1], periodic=tuple(int(p) for p in periodic),
                 boundary_lo=tuple(c.get("boundary_lo", ["reflecting", "reflecting"])),
                 boundary_hi=tuple(c.get("boundary_hi", ["transmissive", "reflecting"])), inlet=fresh,
                 wedge_start=c.get("wedge_start", 0.0))
    box = c.get("tag_box") or None
    tags = dict(pressure_tag=c.get("pressure_tag", 0.08), temperature_tag=c.get("temperature_tag", 0.08),
                fuel_rate_tag=c.get("fuel_rate_tag", 50.0), box=tuple(box) if box else None,
                box_only=c.get("tag_mode", "physics") == "box", velocity=tuple(c.get("tag_velocity", [0.0, 0.0])))
    run = dict(cfl=c.get("cfl", 0.6), end_time=c["end_time"], output_times=list(c.get("output_times", [c["end_time"]])),
               chemistry=bool(c.get("chemistry", True)), max_level=c.get("max_level", 2),
               tag_buffer=c.get("tag_buffer", 2),
               regrid_interval=c.get("regrid_interval", 8) if c.get("adaptive", True) else 0, tags=tags,
               block=block_size(nc, c.get("blocking_factor", 4), c.get("max_grid_size", 32)))
    return U, level, run


def block_size(base_cells, blocking_factor=4, max_grid_size=32):
    """The block of the block-AMR stepper closest to the reference's refinement
    granularity: the smallest even size of at least max(8, blocking_factor) cells and at
    most max_grid_size that tiles the refined levels (base cells divisible by half a
    block), or None.  (Larger blocks refine coarser regions: on the reference's inert
    blast check, blocks of 16 leave the finest level empty at the start.)"""
    lo = max(8, int(blocking_factor) + (int(blocking_factor) & 1))
    for b in range(lo, int(max_grid_size) + 1, 2):
        if base_cells[0] % (b // 2) == 0 and base_cells[1] % (b // 2) == 0:
            return b
    return None


def levels(c, max_level=None):
    """The initial state of levels 0..max_level (default: the case's max_level), each the
    initial condition evaluated at that level's resolution (MakeNewLevelFromScratch,
    BlockAMR.cpp:124-131): the U_levels of the block-AMR stepper."""
    top = c.get("max_level", 2) if max_level is None else max_level
    return [load(c, refine=lev)[0] for lev in range(top + 1)]
