"""The reference's output files, written from device state.

Formats of HyperFlow_V3/src/BlockAMR.cpp:
  state_N.csv   :374-391  t,level,i,j,x,y,dx,dy,rho,u,v,p,p_atm,T,rhoE,Y_<species>
  boxes_N.csv   :379-382  level,x_left,x_right,y_bottom,y_top,dx,dy
  history.csv   :80-81, 361-366  step,t,dt,finest_level,leaf_cells,stored_cells,dx_min,
                          dy_min,mass,momentum_x,momentum_y,total_energy,regrids,retries
  summary.json  :426-438
Numbers are printed like the reference's setprecision(17) streams (%.17g), so the
reference's comparison scripts (tests/validate.py, tests/check_cases.py) read them.
Pressure and temperature come from hf_properties on the GPU; sums from hf_totals.
"""
import json
import os

import numpy as np
import torch

from . import solver as S

SPECIES = ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2", "AR"]


def _g(v):
    return format(float(v), ".17g")


def state_rows(ctx, U, level, time, lev=0):
    """Rows of state_N.csv for a uniform level: U (NV, ny, nx) CUDA tensor."""
    nv, ny, nx = U.shape
    ns = nv - 3
    q = U.reshape(nv, -1).contiguous()
    p, _, T, st = S.properties(ctx, q)
    if int(st.max().item()) != 0:
        raise S.DomainError(1, "state_rows: inadmissible cell")
    Q = q.cpu().numpy()
    p, T = p.cpu().numpy(), T.cpu().numpy()
    rho = Q[:ns].sum(0)
    jj, ii = np.divmod(np.arange(nx * ny), nx)
    x = level.xlo + (ii + 0.5) * level.dx
    y = level.ylo + (jj + 0.5) * level.dy
    cols = [np.full(nx * ny, time), np.full(nx * ny, lev), ii, jj, x, y, np.full(nx * ny, level.dx),
            np.full(nx * ny, level.dy), rho, Q[ns] / rho, Q[ns + 1] / rho, p, p / 101325.0, T, Q[ns + 2]]
    cols += [Q[k] / rho for k in range(ns)]
    return np.column_stack(cols)


def write_state(path, ctx, U, level, time, lev=0):
    ns = U.shape[0] - 3
    header = "t,level,i,j,x,y,dx,dy,rho,u,v,p,p_atm,T,rhoE" + "".join(",Y_" + SPECIES[k] for k in range(ns))
    rows = state_rows(ctx, U, level, time, lev)
    with open(path, "w") as f:
        f.write(header + "\n")
        for r in rows:
            f.write(",".join(str(int(v)) if k in (1, 2, 3) else _g(v) for k, v in enumerate(r)) + "\n")


def write_boxes(path, level, boxes=None, lev=0):
    """boxes: [(ilo, jlo, ihi, jhi)] of the level (default: the whole domain)."""
    boxes = boxes or [(0, 0, level.nx - 1, level.ny - 1)]
    with open(path, "w") as f:
        f.write("level,x_left,x_right,y_bottom,y_top,dx,dy\n")
        for (i0, j0, i1, j1) in boxes:
            f.write(",".join([str(lev), _g(level.xlo + i0 * level.dx), _g(level.xlo + (i1 + 1) * level.dx),
                              _g(level.ylo + j0 * level.dy), _g(level.ylo + (j1 + 1) * level.dy), _g(level.dx),
                              _g(level.dy)]) + "\n")


class History:
    """history.csv rows (BlockAMR::log) for a uniform one-level run."""

    HEADER = ("step,t,dt,finest_level,leaf_cells,stored_cells,dx_min,dy_min,mass,momentum_x,momentum_y,"
              "total_energy,regrids,retries\n")

    def __init__(self, path):
        self.f = open(path, "w")
        self.f.write(self.HEADER)
        self.f.flush()

    def log(self, ctx, U, level, step, time, dt, retries=0):
        ns = U.shape[0] - 3
        ps = S.PatchSet(U.shape[0], [(0, 0, level.nx - 1, level.ny - 1)], device=U.device)
        ps.interior(0).copy_(U)
        sums = S.totals(ctx, ps, level.dx * level.dy)
        cells = level.nx * level.ny
        row = [str(step), _g(time), _g(dt), "0", str(cells), str(cells), _g(level.dx), _g(level.dy),
               _g(sum(sums[:ns])), _g(sums[ns]), _g(sums[ns + 1]), _g(sums[ns + 2]), "0", str(retries)]
        self.f.write(",".join(row) + "\n")
        self.f.flush()
        return sums

    def close(self):
        self.f.close()


def write_summary(path, **fields):
    """summary.json with the reference's keys (BlockAMR.cpp:427-437); missing keys are omitted."""
    with open(path, "w") as f:
        json.dump(fields, f, indent=2)
        f.write("\n")


def run_case(ctx, level, U0, end_time, out_dir, cfl=0.5, chemistry=True, max_steps=10 ** 7, **stepper_kw):
    """A uniform-level run to end_time writing the reference's files (a one-level
    BlockAMR::run, BlockAMR.cpp:400-439): state_0/1.csv, boxes_0/1.csv, history.csv,
    summary.json.  Returns the summary dict."""
    os.makedirs(out_dir, exist_ok=True)
    st = S.Stepper(ctx, level, U0, chemistry=chemistry, **stepper_kw)
    write_state(os.path.join(out_dir, "state_0.csv"), ctx, st.state(), level, 0.0)
    write_boxes(os.path.join(out_dir, "boxes_0.csv"), level)
    hist = History(os.path.join(out_dir, "history.csv"))
    initial = hist.log(ctx, st.state(), level, 0, 0.0, 0.0)
    steps, t, dts = 0, 0.0, []
    c0 = ctx.counters()
    while t < end_time:
        if steps >= max_steps:
            raise RuntimeError("maximum step count reached")
        # the CFL step, shortened to land on end_time (BlockAMR.cpp:412)
        dt_cfl = st.cfl_dt(cfl)
        dt = st.step(dt=min(end_time - t, dt_cfl), cfl=cfl)
        t = end_time if dt >= end_time - t else t + dt
        steps += 1
        dts.append(dt)
        hist.log(ctx, st.state(), level, steps, t, dt, ctx.counters()["retries"] - c0["retries"])
    final_state = st.state()
    write_state(os.path.join(out_dir, "state_1.csv"), ctx, final_state, level, t)
    write_boxes(os.path.join(out_dir, "boxes_1.csv"), level)
    ps = S.PatchSet(final_state.shape[0], [(0, 0, level.nx - 1, level.ny - 1)], device=final_state.device)
    ps.interior(0).copy_(final_state)
    final = S.totals(ctx, ps, level.dx * level.dy)
    c1 = ctx.counters()
    hist.close()
    summary = dict(completed=True, final_time=t, cfl=cfl, steps=steps, retries=c1["retries"] - c0["retries"],
                   finest_level=0, leaf_cells=level.nx * level.ny, max_leaf_cells=level.nx * level.ny,
                   full_finest_cells=level.nx * level.ny, dx_min=level.dx, dy_min=level.dy, regrids=0,
                   max_remap_relative_defect=0.0, reflux_stage_interfaces=0,
                   positivity_first_order_stages=c1["first_order_stages"] - c0["first_order_stages"],
                   roundoff_redistributions=c1["roundoff_repairs"] - c0["roundoff_repairs"],
                   chemistry_cell_calls=c1["chem_cell_calls"] - c0["chem_cell_calls"],
                   min_dt=min(dts) if dts else 0.0, max_dt=max(dts) if dts else 0.0,
                   initial_conserved_integrals=initial, final_conserved_integrals=final, time_subcycling=False,
                   refinement_ratio=[2, 2])
    write_summary(os.path.join(out_dir, "summary.json"), **summary)
    st.close()
    return summary
