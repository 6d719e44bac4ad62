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


# ------------------------------------------------------------------ multi-level runs
def leaf_masks(acts, shapes, block):
    """Per level l, the (ny_l, nx_l) bool map of its leaf cells (BlockAMR::mask,
    BlockAMR.cpp:165-168): cells of an active block of level l (level 0: act None = all)
    that lie under no active block of level l+1 (a block footprint of block/2 cells)."""
    masks = []
    for l, (act, (ny, nx)) in enumerate(zip(acts, shapes)):
        if act is None:
            m = np.ones((ny, nx), bool)
        else:
            m = np.kron(act, np.ones((block, block), np.uint8)).astype(bool)[:ny, :nx]
        if l + 1 < len(acts) and acts[l + 1] is not None:
            h = block // 2
            m &= ~np.kron(acts[l + 1], np.ones((h, h), np.uint8)).astype(bool)[:ny, :nx]
        masks.append(m)
    return masks


def amr_state_rows(Qs, masks, base, time, props):
    """state_N.csv rows of the leaf cells of every level, coarse to fine, each level in
    row-major cell order (BlockAMR::snapshot, BlockAMR.cpp:374-391).  Qs[l]: (NV, ny_l,
    nx_l) numpy state of level l; props(q (NV, n)) -> (p, T) numpy arrays."""
    out = []
    for l, (Q, m) in enumerate(zip(Qs, masks)):
        jj, ii = np.nonzero(m)
        if len(ii) == 0:
            continue
        nv = Q.shape[0]
        ns = nv - 3
        q = np.ascontiguousarray(Q[:, jj, ii])
        p, T = props(q)
        dx, dy = base.dx / (1 << l), base.dy / (1 << l)
        rho = q[:ns].sum(0)
        n = len(ii)
        cols = [np.full(n, time), np.full(n, l), ii, jj, base.xlo + (ii + 0.5) * dx, base.ylo + (jj + 0.5) * dy,
                np.full(n, dx), np.full(n, dy), rho, q[ns] / rho, q[ns + 1] / rho, p, p / 101325.0, T, q[ns + 2]]
        cols += [q[k] / rho for k in range(ns)]
        out.append(np.column_stack(cols))
    return np.concatenate(out)


def write_rows(path, rows, ns):
    header = "t,level,i,j,x,y,dx,dy,rho,u,v,p,p_atm,T,rhoE" + "".join(",Y_" + SPECIES[k] for k in range(ns))
    with open(path, "w") as f:
        f.write(header + "\n")
        for r in rows:
            f.write(",".join(str(int(v)) if k in (1, 2, 3) else _g(v) for k, v in enumerate(r)) + "\n")


def amr_boxes(acts, shapes, block):
    """[(level, ilo, jlo, ihi, jhi)]: level 0's domain, then every active block."""
    out = []
    for l, (act, (ny, nx)) in enumerate(zip(acts, shapes)):
        if act is None:
            out.append((l, 0, 0, nx - 1, ny - 1))
            continue
        for bj, bi in zip(*np.nonzero(act)):
            out.append((l, bi * block, bj * block, min((bi + 1) * block, nx) - 1, min((bj + 1) * block, ny) - 1))
    return out


def write_amr_boxes(path, boxes, base):
    """boxes_N.csv (BlockAMR.cpp:379-382) from amr_boxes()."""
    with open(path, "w") as f:
        f.write("level,x_left,x_right,y_bottom,y_top,dx,dy\n")
        for (l, i0, j0, i1, j1) in boxes:
            dx, dy = base.dx / (1 << l), base.dy / (1 << l)
            f.write(",".join([str(l), _g(base.xlo + i0 * dx), _g(base.xlo + (i1 + 1) * dx), _g(base.ylo + j0 * dy),
                              _g(base.ylo + (j1 + 1) * dy), _g(dx), _g(dy)]) + "\n")


def run_amr_case(ctx, level, U0, end_time, out_dir, cfl=0.5, output_times=None, max_level=1, block=32,
                 tag_buffer=2, regrid_interval=8, chemistry=True, chem="batched", tags=None, max_steps=10 ** 7,
                 stepper=None, props=None, U_levels=None):
    """BlockAMR::run (BlockAMR.cpp:400-439) on the block-AMR stepper, writing the
    reference's files: state_N.csv and boxes_N.csv at t = 0 and at every output time
    (leaf cells of every level), history.csv after every step, summary.json.  The step is
    the CFL step of all levels shortened to land on the next output time; a regrid
    follows every regrid_interval-th step unless it reached the end time (:420).
    U_levels: the initial state of levels 1, 2, ... (case.levels), taken by the initial
    hierarchy's new blocks as the reference's MakeNewLevelFromScratch does; without it
    they interpolate level 0.  stepper / props: an object with AmrStepper's methods built
    with regrid_interval 0, and props(q (NV, n) numpy) -> (p, T) numpy, in place of the GPU
    stepper and the GPU EOS (the host logic is the same for any hierarchy).  Returns the
    summary dict."""
    os.makedirs(out_dir, exist_ok=True)
    targets = list(output_times or [end_time])
    prev = 0.0
    for target in targets:
        if not (prev < target <= end_time):
            raise ValueError("invalid output times")
        prev = target
    if abs(targets[-1] - end_time) > 1e-14 * end_time:
        raise ValueError("last output must equal final time")
    am = stepper or S.AmrStepper(ctx, level, U0, max_level=max_level, block=block, tag_buffer=tag_buffer,
                                 regrid_interval=0, chemistry=chemistry, chem=chem, rtol=1e-8, atol=1e-15, tags=tags,
                                 U_levels=U_levels)
    ns = U0.shape[0] - 3

    def gpu_props(q):
        p, _, T, st = S.properties(ctx, torch.from_numpy(q).to(U0.device))
        if int(st.max().item()) != 0:
            raise S.DomainError(1, "snapshot: inadmissible cell")
        return p.cpu().numpy(), T.cpu().numpy()

    props = props or gpu_props

    def hierarchy():
        finest = am.info(0)["finest"]
        Qs, acts, shapes = [], [], []
        for lev in range(finest + 1):
            U, act = am.level(lev)
            Qs.append(U.cpu().numpy())
            acts.append(None if lev == 0 else act)
            shapes.append(tuple(U.shape[1:]))
        return finest, Qs, acts, shapes

    def snapshot(frame, time):
        finest, Qs, acts, shapes = hierarchy()
        rows = amr_state_rows(Qs, leaf_masks(acts, shapes, block), level, time, props)
        write_rows(os.path.join(out_dir, "state_%d.csv" % frame), rows, ns)
        write_amr_boxes(os.path.join(out_dir, "boxes_%d.csv" % frame), amr_boxes(acts, shapes, block), level)

    def counts():
        finest, _, acts, shapes = hierarchy()
        leaf = sum(am.info(lev)["leaf_cells"] for lev in range(finest + 1))
        stored = level.nx * level.ny + sum(int(a.sum()) * block * block for a in acts[1:])
        return finest, leaf, stored

    hist = open(os.path.join(out_dir, "history.csv"), "w")
    hist.write(History.HEADER)
    c0 = ctx.counters()
    steps, t, regrids, dts, frame, max_leaf = 0, 0.0, 0, [], 0, 0

    def log(dt):
        nonlocal max_leaf
        finest, leaf, stored = counts()
        max_leaf = max(max_leaf, leaf)
        sums = am.totals()
        row = [str(steps), _g(t), _g(dt), str(finest), str(leaf), str(stored), _g(level.dx / (1 << finest)),
               _g(level.dy / (1 << finest)), _g(sum(sums[:ns])), _g(sums[ns]), _g(sums[ns + 1]), _g(sums[ns + 2]),
               str(regrids), str(ctx.counters()["retries"] - c0["retries"])]
        hist.write(",".join(row) + "\n")
        hist.flush()
        return sums

    initial = am.totals()
    snapshot(0, 0.0)
    log(0.0)
    for target in targets:
        while t < target:
            if steps >= max_steps:
                raise RuntimeError("maximum step count reached")
            dt = am.step(dt=min(target - t, am.cfl_dt(cfl)), cfl=cfl)
            t = target if dt >= target - t else t + dt
            steps += 1
            dts.append(dt)
            if max_level > 0 and regrid_interval > 0 and steps % regrid_interval == 0 and t < end_time:
                am.regrid()
                regrids += 1
            log(dt)
        frame += 1
        snapshot(frame, t)
    hist.close()
    final = am.totals()
    finest, leaf, _ = counts()
    c1 = ctx.counters()
    summary = dict(completed=True, final_time=t, cfl=cfl, steps=steps, retries=c1["retries"] - c0["retries"],
                   finest_level=finest, leaf_cells=leaf, max_leaf_cells=max_leaf,
                   full_finest_cells=(level.nx << finest) * (level.ny << finest), dx_min=level.dx / (1 << finest),
                   dy_min=level.dy / (1 << finest), regrids=regrids,
                   positivity_first_order_stages=c1["first_order_stages"] - c0["first_order_stages"],
                   roundoff_redistributions=c1["roundoff_repairs"] - c0["roundoff_repairs"],
                   chemistry_cell_calls=c1["chem_cell_calls"] - c0["chem_cell_calls"],
                   min_dt=min(dts) if dts else 0.0, max_dt=max(dts) if dts else 0.0,
                   initial_conserved_integrals=list(initial), final_conserved_integrals=list(final),
                   time_subcycling=False, refinement_ratio=[2, 2])
    write_summary(os.path.join(out_dir, "summary.json"), **summary)
    am.close()
    return summary
