#!/usr/bin/env python3
"""Benchmark: cell-steps/s of the Strang-split reacting-Euler step on the 2D H2/O2/Ar
detonation (2048 x 512 cells, FP64), one GPU per rank.

One "step" is one full Strang step of the whole grid: flow(dt/2) (two Euler stages
and the Heun combine), react(dt), flow(dt/2), with the CFL dt.  The headline value
is a device-resident run of CUDA-graph steps: plain flux kernels (ghost fill, face,
update; faster than the fused TMA-tile kernel on this FP64-bound path, --flux fused
selects it) and the batched work-queue chemistry.  The plain drop-in chemistry (one
thread per cell) is timed the same way beside it, so batched_over_plain compares the
chemistry forms alone.  `e2e` runs the same steps through the public stepper API with
the state in pinned HOST memory, copied in and out every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank runs an independent replica (one grid per GPU; the
step of one grid is not sharded): value = all ranks' cell-steps over the slowest
rank's time.  --impl reference times the CPU restatement of the reference (the
reference itself needs Cantera, SUNDIALS and AMReX, absent here) on this host's cores:
the same W warm-up and K timed steps as the GPU arm, on a 2048 x 32 periodic strip of
the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s, 2D H2 detonation FP64: batched vs plain GPU; adjoint/forward time"
NX, NY = 2048, 512
STRIP_ROWS = 32  # rows of the periodic strip the CPU legs time
# From one ncu capture of the probe launch below at the full size (2048 x 512, the state
# after the 3 warm-up and 8 timed steps; `bench.py --probe-only --warmup 11`, the second
# k_chem_batched launch of the probe, 1,090,021 step attempts, k_chem_batched<10, 4, 0>):
# * FP64 flops per integrator step attempt (DFMA x 2 + DADD + DMUL thread instructions
#   over the launch's attempts; the screened cells' kinetics pass is included), the
#   executed-flop figure beside the algorithmic one;
# * DRAM bytes of that launch (dram__bytes_read.sum + dram__bytes_write.sum): mostly the
#   lanes' stack frames written back from L2.
EXECUTED_FLOPS_PER_ATTEMPT = 2.063e4
PROBE_TRAFFIC = 5011249000
# algorithmic HBM bytes of one cell-step (NS = 10): 4 Euler stages reading U (and U_old in
# the Heun stages) and writing U, plus chemistry reading and writing U
BYTES_PER_CELL_STEP = 1248


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=8)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cfl", type=float, default=0.5)
    p.add_argument("--flux", default="auto", choices=["auto", "fused", "plain"],
                   help="flux form of the headline run (auto: the tuner's choice)")
    p.add_argument("--no-tune", action="store_true", help="keep the library's default launch settings")
    p.add_argument("--probe-only", action="store_true",
                   help="only the roofline probe's two chemistry launches (for an ncu capture of the second)")
    p.add_argument("--curve-steps", type=int, default=500,
                   help="steps of the per-step cost curve of the headline form (0 disables it)")
    p.add_argument("--curve-every", type=int, default=25)
    p.add_argument("--chem-cells", type=int, default=1 << 20,
                   help="cells of the chemistry-only batch (0 = skip)")
    p.add_argument("--adj-cells", type=int, default=4096,
                   help="0D H2/air cells of the adjoint measurement (0 disables it)")
    p.add_argument("--adj-calls", type=int, default=2000, help="chemistry calls (of 1e-7 s) per adjoint run")
    p.add_argument("--adj-objectives", default="ignition_delay",
                   help="comma-separated: ignition_delay, peak_pressure, final_T")
    p.add_argument("--adj1d-cells", type=int, default=1000,
                   help="cells of the 1D detonation whose run is differentiated (0 disables it)")
    p.add_argument("--adj1d-steps", type=int, default=1000, help="CFL Strang steps of that run")
    p.add_argument("--det1d-steps", type=int, default=2000,
                   help="device-resident steps of the 1D detonation, 2000 x 2 cells (0 disables it)")
    p.add_argument("--det1d-cpu-steps", type=int, default=50, help="oracle steps of its CPU line")
    p.add_argument("--amr-steps", type=int, default=2000,
                   help="coarse steps of the 3-level block-AMR wedge (0 disables it)")
    p.add_argument("--nx", type=int, default=NX)
    p.add_argument("--ny", type=int, default=NY)
    return p.parse_args(argv)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(dist, x, device):
    """The largest x over the ranks of the process group (x itself without one)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, units_per_rank, steps, slowest_ms):
    """Whole-job throughput of `world` independent replicas: all ranks' units over the
    slowest rank's time (units per second)."""
    return world * units_per_rank * steps / (slowest_ms * 1e-3)


def workload_config(args):
    """The workload both arms time (the GPU arm on the whole grid, the CPU arm on a strip
    of it)."""
    return {"workload": "2D H2/O2/Ar detonation %dx%d, 64-column hot band at 40 atm/3000 K, +-1%% density "
                        "perturbation, periodic y, CFL %.2f" % (args.nx, args.ny, args.cfl),
            "cells": args.nx * args.ny, "species": 10, "mechanism": "H2_Li + inert AR extension",
            "chem_tolerances": "rtol 1e-8 atol 1e-15", "steps_timed": "steps %d..%d of the run" % (
                args.warmup + 1, args.warmup + args.steps)}


class Clocks:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ CPU (oracle) legs
def _oracle(ns):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    oracle.set_species(ns)
    return oracle


def flux_roofline(ff, nv, cells, flux_ms_per_step, fp64_peak, hbm_gbs):
    """The flux path's roofline over a step (4 Euler stages, 2 Heun combines): the
    oracle's counted FP64 flops per cell-step (ff = oracle.flux_flops of a face stencil:
    2 faces per cell-stage, one cell update and validation per stage, a combine in each
    Heun stage) and the algorithmic HBM bytes per cell-step (stage 1 reads U and writes
    U1, stage 2 reads U1 and U_old and writes U: 5 state transfers per flow half-step)
    over the measured flux time per step; the bound is the larger fraction."""
    flops = 4 * (2 * ff["face"] + ff["cell"]) + 2 * ff["combine"]
    nbytes = 2 * (2 + 3) * nv * 8
    sec = flux_ms_per_step * 1e-3
    gf = flops * cells / sec / 1e9
    gb = nbytes * cells / sec / 1e9
    return {"kernels": "k_face_plain (x, y) + k_update_plain, k_fill, k_cfl of a step",
            "bound": "fp64" if gf / fp64_peak >= gb / hbm_gbs else "hbm", "ms_per_step": flux_ms_per_step,
            "fp64": {"flops_per_cell_step": flops, "achieved": gf, "peak": fp64_peak, "unit": "GFLOP/s",
                     "frac": gf / fp64_peak, "per_face": ff["face"], "per_cell_update": ff["cell"],
                     "per_combine": ff["combine"],
                     "source": "the oracle's flux functions on a counting scalar, 3 UV Newton iterations per "
                               "EOS solve from 1000 K, at a subsonic face of the fresh gas (HLLC star state)"},
            "hbm": {"bytes_per_cell_step": nbytes, "achieved": gb, "peak": hbm_gbs, "unit": "GB/s",
                    "frac": gb / hbm_gbs}}


def cpu_window(steps, warm, rows=STRIP_ROWS, nx=NX, threads=0, serial_steps=0, cfl=0.5):
    """The oracle's Strang steps on a periodic strip (nx x rows) of the 2D detonation: warm
    untimed steps, then `steps` timed ones, every loop on all host threads (OpenMP flux,
    update and validation loops, OpenMP dynamic,8 chemistry; the same results as serial
    loops).  serial_steps > 0 also times that many steps of the same window with the
    reference's threading (serial flux loop, OpenMP chemistry), from the same start."""
    oracle = _oracle(10)
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=0, diluent="AR", nx=nx, ny=rows)
    g = oracle.make_grid(nx, rows, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    oracle.set_flux_threads(0)

    def step(Ug):
        dt = oracle.cfl_dt(g, Ug, cfl)
        Ug, _, st, _ = oracle.strang_step(g, Ug, dt, threads=threads)
        if st:
            raise RuntimeError("oracle step failed")
        return Ug

    try:
        for _ in range(warm):
            Ug = step(Ug)
        start = Ug.copy()
        per = []
        for _ in range(steps):
            t0 = time.perf_counter()
            Ug = step(Ug)
            per.append(1e3 * (time.perf_counter() - t0))
        serial = None
        if serial_steps:
            oracle.set_flux_threads(1)
            Us, sper = start, []
            for _ in range(serial_steps):
                t0 = time.perf_counter()
                Us = step(Us)
                sper.append(1e3 * (time.perf_counter() - t0))
            serial = {"value": nx * rows * serial_steps / (1e-3 * sum(sper)),
                      "ms_per_step": sum(sper) / serial_steps,
                      "sample": "steps %d..%d of the same %dx%d strip, serial flux loop (the reference's threading), "
                                "OpenMP dynamic,8 chemistry" % (warm + 1, warm + serial_steps, nx, rows)}
    finally:
        oracle.set_flux_threads(1)
    el = 1e-3 * sum(per)
    return {"value": nx * rows * steps / el, "unit": "cell-steps/s", "cores": threads or os.cpu_count(),
            "kind": "port", "ms_per_step": 1e3 * el / steps, "per_step_ms": [round(v, 2) for v in per],
            "cells_per_step": nx * rows,
            "sample": "steps %d..%d (after %d warm-up steps) of a %dx%d periodic strip of the 2D detonation, every "
                      "loop on all host threads; the per-cell rate stands for the %s-cell grid" % (
                          warm + 1, warm + steps, warm, nx, rows, "full"),
            "reference_threading": serial}


def tight_errors(states, ref_states):
    """T relative and Y_k absolute errors (max over cells) of AoS states against the
    tight oracle's; Y_k = rho Y_k / rho of the reference."""
    import numpy as np
    oracle = _oracle(10)
    Tg, Tr = oracle.properties(states)[2], oracle.properties(ref_states)[2]
    rho = ref_states[:, :10].sum(1)
    return {"T_rel_max": float(np.max(np.abs(Tg - Tr) / Tr)),
            "Y_abs_max": float(np.max(np.abs(states[:, :10] - ref_states[:, :10]) / rho[:, None]))}


def tight_oracle_strip(U0, lvd, dts, nx, rows):
    """The oracle's Strang steps of a strip at rtol 1e-12 / atol 1e-20 with the given
    step sizes (AoS interior states)."""
    oracle = _oracle(10)
    oracle.set_flux_threads(0)
    g = oracle.make_grid(nx, rows, lvd["dx"], lvd["dy"], periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0),
                         inlet=lvd["inlet"])
    Ug = oracle.ghosted(U0.transpose(1, 2, 0))
    try:
        for dt in dts:
            Ug, dta, st, _ = oracle.strang_step(g, Ug, dt, rtol=1e-12, atol=1e-20)
            if st or dta != dt:
                raise RuntimeError("tight oracle step failed")
    finally:
        oracle.set_flux_threads(1)
    return Ug[2:-2, 2:-2].reshape(-1, U0.shape[0])


def algorithmic_flops(X_aos, dt, ns=10, sample_tight=256, order=None):
    """The FP64 work the oracle's integrator needs for one chemistry call of these cells at
    the reference's tolerances (rtol 1e-8, atol 1e-15): its accepted Rodas4 steps, each
    6 right-hand sides + 1 analytic Jacobian (both counted by the oracle's counting
    scalar, UV inversion fixed at 3 Newton iterations) + 1 LU factorisation ((2/3) n^3)
    + 6 triangular solves (2 n^2 each), n = NS - 1 unknowns.  Transcendental calls (exp,
    log, pow) are counted apart.  The same count at the tight tolerances (rtol 1e-12,
    atol 1e-20) on the `sample_tight` costliest cells (by `order`, else the first)."""
    import numpy as np
    oracle = _oracle(ns)
    fr, tr, fj, tj = oracle.chem_flops(X_aos[0])
    n = ns - 1
    per_step = 6 * fr + fj + 2.0 * n ** 3 / 3.0 + 6 * 2.0 * n * n
    trans_step = 6 * tr + tj
    t0 = time.perf_counter()
    acc, rej = oracle.chem_batch_stats(X_aos, dt)
    secs = time.perf_counter() - t0
    ok = acc >= 0
    out = {"per_accepted_step": {"flops": per_step, "transcendental_calls": trans_step, "rhs_flops": fr,
                                 "jacobian_flops": fj, "lu_flops": 2.0 * n ** 3 / 3.0, "solve_flops": 2.0 * n * n},
           "cells": int(len(acc)), "accepted_steps": int(acc[ok].sum()), "oracle_rejected": int(rej[ok].sum()),
           "failed_cells": int((~ok).sum()), "flops": float(acc[ok].sum()) * per_step,
           "transcendental_calls": float(acc[ok].sum()) * trans_step, "oracle_seconds": secs}
    if sample_tight:
        idx = order[:sample_tight] if order is not None else np.arange(min(sample_tight, len(acc)))
        a_ref = acc[idx]
        a_tight, _ = oracle.chem_batch_stats(X_aos[idx], dt, rtol=1e-12, atol=1e-20)
        good = (a_ref > 0) & (a_tight > 0)
        out["tight_sample"] = {"cells": int(len(idx)), "accepted_steps_ref_tol": int(a_ref[good].sum()),
                               "accepted_steps_tight": int(a_tight[good].sum()),
                               "tight_over_ref": float(a_tight[good].sum() / max(a_ref[good].sum(), 1))}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cb = cpu_window(args.steps, args.warmup, nx=args.nx, rows=min(STRIP_ROWS, args.ny), cfl=args.cfl)
    line = {"metric": METRIC, "value": cb["value"], "unit": "cell-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(args),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "per_step_ms": cb["per_step_ms"], "cells_per_step": cb["cells_per_step"],
            "note": "the reference (Cantera/SUNDIALS/AMReX) cannot be built here; this arm times the CPU restatement "
                    "of its path on a strip of the workload: ms_per_step is the strip's measured time per step, "
                    "value its cell-steps/s"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def chem_input(hf, ctx, level, U, dt, nv):
    """The input of the chemistry call of the Strang step from state U over dt: flow(dt/2)
    on the GPU (ghost fill, two plain Euler stages, Heun combine).  (NV, n) tensor."""
    pa = hf.PatchArray(nv, level.nx, level.ny)
    pa.interior().copy_(U)
    hf.fill(ctx, level, pa)
    t1 = pa.like()
    hf.euler_stage(ctx, level, pa, t1, 0.5 * dt, form=0)
    hf.fill(ctx, level, t1)
    x = pa.like()
    hf.euler_stage(ctx, level, t1, x, 0.5 * dt, u_old=pa, form=0)
    return x.interior().contiguous().reshape(nv, -1).clone()


def chem_probe(hf, ctx, level, U, dt, nv):
    """Two batched chemistry launches on the chemistry input of the step from U: the first
    builds the per-cell history, the second is timed (the chemistry class of the context's
    CUDA-event timing: ordering kernels + the queue kernel).  Returns (X (NV, n) before the
    calls, launch ms, GPU attempts, cost order)."""
    import torch
    X = chem_input(hf, ctx, level, U, dt, nv)
    cb = hf.ChemistryBatch(ctx, "batched")
    cb.advance(X.clone(), dt)
    c0 = ctx.counters()
    ctx.set_timing(True)
    cb.advance(X.clone(), dt)
    ms, _ = ctx.timing()["chem"]
    ctx.set_timing(False)
    attempts = ctx.counters()["chem_steps"] - c0["chem_steps"]
    order = torch.argsort(cb.history[1].to(torch.int64), descending=True, stable=True).cpu().numpy()
    return X, ms, attempts, order


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import hyperflow_gb300 as hf
    from hyperflow_gb300 import workloads as W
    U0, lvd = W.det2d(seed=rank, diluent="AR", nx=args.nx, ny=args.ny)
    ctx = hf.Context("H2_Li+AR", device=local)
    level = hf.make_level(**lvd)
    cells = args.nx * args.ny
    nv = U0.shape[0]

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def slowest(x):
        return max_over_ranks(dist, x, "cuda")

    tuning = None
    flux = "plain" if args.flux == "auto" else args.flux
    if not args.no_tune and not args.probe_only:
        # launch settings measured on this workload before the timed region: the chemistry
        # input of the step after the warm-up steps, and one Euler stage of that state
        from hyperflow_gb300 import tune
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=flux, chem="batched")
        for _ in range(args.warmup):
            st.step(cfl=args.cfl)
        Ut, dtt = st.state(), st.cfl_dt(args.cfl)
        st.close()
        Xt = chem_input(hf, ctx, level, Ut, dtt, nv)
        tuning = {"chemistry": tune.tune_chemistry(ctx, Xt, dtt), "flux": tune.tune_flux(ctx, level, Ut, dtt),
                  "sample": "the chemistry call and one Euler stage of the step after %d warm-up steps" % args.warmup}
        del Xt, Ut
        if args.flux == "auto":
            flux = tuning["flux"]["best"]
        # the cooperative threshold over whole graph steps at the chosen register budget
        m = tuning["chemistry"]["best"][0]
        tuning["stepper"] = tune.tune_stepper(ctx, level, torch.from_numpy(U0).cuda(), args.cfl, flux=flux,
                                              warm=args.warmup, steps=4,
                                              candidates=[(m, 16), (m, 3), (m, 5), (m, 7)])
        tuning["stepper"]["sample"] = "4 graph steps after %d warm-up steps per candidate" % args.warmup
    args.flux = flux

    if args.probe_only:
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem="batched")
        for _ in range(args.warmup):
            st.step(cfl=args.cfl)
        U, dt = st.state(), st.cfl_dt(args.cfl)
        st.close()
        _, ms, att, _ = chem_probe(hf, ctx, level, U, dt, nv)
        print(json.dumps({"probe": "k_chem_batched, second launch", "ms": ms, "attempts": att}), flush=True)
        return

    def timed(chem, steps, warmup, clocks=None):
        """A device-resident run of `steps` graph steps after `warmup` single steps."""
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem=chem)
        for _ in range(warmup):
            st.step(cfl=args.cfl)
        c0 = ctx.counters()
        ctx.set_timing(True)
        barrier()
        if clocks:
            clocks.start()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        # graph steps back to back, no host round trip; every step reads and writes 4
        # state buffers of 109 MB (inputs larger than the 129 MB L2), no flush
        st.run(steps, cfl=args.cfl)
        ev1.record()
        barrier()
        ms = ev0.elapsed_time(ev1)
        ck = clocks.stop() if clocks else None
        tm = ctx.timing()
        ctx.set_timing(False)
        c1 = ctx.counters()
        return st, slowest(ms), ck, tm, {k: c1[k] - c0[k] for k in c1}

    clocks = Clocks(local)
    st, ms, ck, tm, cnt = timed("batched", args.steps, args.warmup, clocks=clocks)
    value = replica_value(world, cells, args.steps, ms)
    U_probe, dt_probe = st.state(), st.cfl_dt(args.cfl)
    st.close()
    plain = None
    if not args.no_plain:
        pst, pms, _, ptm, pcnt = timed("plain", args.steps, args.warmup)
        pst.close()
        plain = {"value": replica_value(world, cells, args.steps, pms), "ms_per_step": pms / args.steps,
                 "steps": args.steps, "chem_ms_per_step": ptm["chem"][0] / args.steps,
                 "flux_ms_per_step": ptm["flux"][0] / args.steps,
                 "form": "%s flux + one thread per cell chemistry, device-resident graph steps" % args.flux}

    e2e = None
    step_loop = None
    if not args.no_e2e:
        # the same window through Stepper.step(): one graph launch and one status read per
        # step, first without and then with the state copied from and to pinned host memory
        host = torch.from_numpy(U0.copy()).pin_memory()
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem="batched")
        for _ in range(args.warmup):
            st.step(cfl=args.cfl)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            st.step(cfl=args.cfl)
        e1.record()
        barrier()
        step_loop = {"ms_per_step": slowest(e0.elapsed_time(e1)) / args.steps,
                     "note": "the headline window through Stepper.step(), state resident"}
        st.close()
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem="batched")
        for _ in range(args.warmup):
            st.set_host(host)
            st.step(cfl=args.cfl)
            st.get_host(host)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st.set_host(host)
            st.step(cfl=args.cfl)
            st.get_host(host)
        barrier()
        el = slowest(time.perf_counter() - t0)
        st.close()
        nbytes = nv * cells * 8
        e2e = {"value": replica_value(world, cells, args.steps, el * 1e3), "unit": "cell-steps/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}

    curve = None
    if args.curve_steps > 0:
        # per-step cost of the headline form over the run, in chunks of curve_every steps
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem="batched")
        pts, done, total = [], 0, 0.0
        ctx.set_timing(True)
        while done < args.curve_steps:
            n = min(args.curve_every, args.curve_steps - done)
            t0 = ctx.timing()["chem"][0]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            k = st.run(n, cfl=args.cfl)
            e1.record()
            torch.cuda.synchronize()
            done += k
            total += e0.elapsed_time(e1)
            pts.append([done, round(e0.elapsed_time(e1) / k, 2), round((ctx.timing()["chem"][0] - t0) / k, 2)])
        ctx.set_timing(False)
        curve = {"steps": done, "every": args.curve_every, "columns": ["step", "ms_per_step", "chem_ms_per_step"],
                 "points": pts, "mean_ms_per_step": total / done, "value_over_run": cells * done / (1e-3 * total),
                 "final_time": st.time}
        st.close()

    # roofline probe: one full-size batched chemistry launch and the oracle's algorithmic
    # FP64 work for the same input
    probe = None
    if rank == 0:
        X, pms_, patt, order = chem_probe(hf, ctx, level, U_probe, dt_probe, nv)
        probe = {"workload": "chemistry call of the Strang step after the timed steps (input = flow(dt/2) of the "
                             "state, dt = its CFL step %.4e s), %d cells; second of two launches on it" % (
                                 dt_probe, cells),
                 "launch_ms": pms_, "gpu_attempts": patt}
        if not args.no_cpu:
            Xa = np.ascontiguousarray(X.cpu().numpy().T)
            probe["algorithmic"] = algorithmic_flops(Xa, dt_probe, order=order)
        del X

    chem_batch = None
    chem_sample = None
    if args.chem_cells > 0:
        # chemistry-only batch of independent 0D cells with very uneven stiffness
        # (T ~ U[800,2500] K, p ~ logU[0.1,10] atm, phi ~ logU[0.3,3], Ar ~ U[0,0.8],
        # dt ~ logU[1e-7,1e-6] s): one all-or-nothing advance per form, same inputs
        Uc, dtc_np = W.chem_batch(args.chem_cells, seed=11, diluent="AR")
        dtc = torch.from_numpy(dtc_np).cuda()
        chem_batch = {"cells": args.chem_cells}
        for form in ("batched", "plain"):
            field = torch.from_numpy(Uc).cuda()
            cb = hf.ChemistryBatch(ctx, form)
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            cb.advance(field, 0.0, dt_cell=dtc)
            e1.record()
            barrier()
            cms = slowest(e0.elapsed_time(e1))
            chem_batch[form] = {"ms": cms, "cells_per_s": replica_value(world, args.chem_cells, 1, cms)}
            if form == "batched":  # a sample for the error against the tight oracle
                chem_sample = (field[:, :512].cpu().numpy().T.copy(), Uc[:, :512].T.copy(), dtc_np[:512].copy())
            del field
        chem_batch["batched_over_plain"] = chem_batch["plain"]["ms"] / chem_batch["batched"]["ms"]

    adjoint = None
    if args.adj_cells > 0:
        # discrete adjoint of 0D ignition runs: d(ignition delay, peak pressure)/d ln A_r for
        # the 21 reactions, 2000 chemistry calls of 1e-7 s, checkpoints every 50 calls;
        # forward = the same runs without the adjoint (hf_chem_objective)
        ctx9 = hf.Context("H2_Li", device=local)
        Ua = torch.from_numpy(W.ignition_batch(args.adj_cells, seed=5 + rank)).cuda()
        adjoint = {"workload": "%d 0D H2/air cells at rest, T ~ U[1000,1500] K, p ~ U[1,5] atm, phi ~ U[0.5,2]; "
                               "%d chemistry calls of 1e-7 s; checkpoint every 50 calls" % (args.adj_cells,
                                                                                              args.adj_calls),
                   "parameters": "ln A_r, 21 reactions"}
        for obj in args.adj_objectives.split(","):
            sa = hf.ChemSensitivity(ctx9, 1e-7, args.adj_calls, objective=obj, checkpoint_every=50)
            sa.objective(Ua)  # warm-up (module load, scratch)
            barrier()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            Jf = sa.objective(Ua)
            e1.record()
            Ja, Ga, _ = sa.adjoint(Ua)
            e2.record()
            barrier()
            fms, ams = slowest(e0.elapsed_time(e1)), slowest(e1.elapsed_time(e2))
            ok = ~torch.isnan(Jf)
            adjoint[obj] = {"forward_ms": fms, "adjoint_ms": ams, "adjoint_over_forward": ams / fms,
                            "cells_with_objective": int(ok.sum().item()),
                            "objective_median": float(Jf[ok].median().item()) if ok.any() else None,
                            "adjoint_objective_equals_forward": bool(torch.equal(Jf[ok], Ja[ok]))}
        adjoint["adjoint_over_forward"] = max(v["adjoint_over_forward"] for v in adjoint.values()
                                              if isinstance(v, dict))
        del ctx9

    if args.adj1d_cells > 0:
        # discrete adjoint of the 1D planar detonation (H2/O2/Ar, nx x 2 cells on 0.1 m,
        # 20-cell driver): d(induction length)/d ln A_r and d/dU0 over adj1d_steps CFL
        # steps with checkpoints every 50; forward = recording the run (plain forms)
        U1, lv1 = W.det1d(diluent="AR", nx=args.adj1d_cells)
        level1 = hf.make_level(**lv1)
        barrier()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        t0 = time.perf_counter()
        e0.record()
        fa = hf.FlowAdjoint(ctx, level1, torch.from_numpy(U1).cuda(), args.adj1d_steps, cfl=args.cfl,
                            checkpoint_every=50)
        e1.record()
        t1 = time.perf_counter()
        Uf = fa.final.clone().requires_grad_(True)
        Jl = hf.induction_length(Uf, lv1["dx"])
        (seed,) = torch.autograd.grad(Jl, Uf)
        t2 = time.perf_counter()
        e2.record()  # the seed's torch ops are not part of either phase
        ea = torch.cuda.Event(enable_timing=True)
        _, gl = fa.adjoint(seed.contiguous())
        ea.record()
        barrier()
        t3 = time.perf_counter()
        fwd = slowest(e0.elapsed_time(e1))
        adj = slowest(e2.elapsed_time(ea))
        fa.close()
        if adjoint is None:
            adjoint = {}
        adjoint["flow_1d"] = {
            "workload": "1D H2/O2/Ar detonation %dx2 cells on 0.1 m, 20-cell driver at 40 atm/3000 K, %d CFL %.2f "
                        "Strang steps, checkpoint every 50" % (args.adj1d_cells, args.adj1d_steps, args.cfl),
            "objective": "induction length (shock-to-reaction-front distance), %.4e m" % float(Jl.item()),
            "forward_ms": fwd, "adjoint_ms": adj, "adjoint_over_forward": adj / fwd,
            "host_wall_s": {"forward": t1 - t0, "adjoint": t3 - t2},
            "dJ_dlnA_largest": [int(k) for k in np.argsort(-np.abs(gl))[:3]]}
        adjoint["adjoint_over_forward"] = max(v["adjoint_over_forward"] for v in adjoint.values()
                                              if isinstance(v, dict) and "adjoint_over_forward" in v)

    det1d = None
    if args.det1d_steps > 0:
        # the 1D planar detonation (2000 x 2 cells on 0.1 m, 20-cell driver at 40 atm /
        # 3000 K, Ar diluent): device-resident graph steps of the headline forms from t = 0;
        # few stiff cells, so single cells' chemistry sets the step time
        U1, l1 = W.det1d(diluent="AR", nx=2000)
        tuning1 = None
        if not args.no_tune:
            # a few thousand cells: the stiff cells' serial chains set the step, and the
            # cooperative phase pays here (tuned on this workload, then restored)
            from hyperflow_gb300 import tune
            restore = tune.get_chem_tuning(ctx)
            tuning1 = tune.tune_stepper(ctx, hf.make_level(**l1), torch.from_numpy(U1).cuda(), args.cfl,
                                        flux=args.flux, warm=20, steps=20)
            tuning1["sample"] = "20 graph steps after 20 from t = 0 per candidate"
        s1 = hf.Stepper(ctx, hf.make_level(**l1), torch.from_numpy(U1).cuda(), flux=args.flux, chem="batched")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        done1 = s1.run(args.det1d_steps, cfl=args.cfl)
        e1.record()
        torch.cuda.synchronize()
        ms1 = e0.elapsed_time(e1)
        det1d = {"workload": "1D H2/O2/Ar detonation 2000x2 cells on 0.1 m, 20-cell driver at 40 atm/3000 K, "
                             "reflecting left/top/bottom, transmissive right, CFL %.2f; %d device-resident steps "
                             "from t = 0" % (args.cfl, done1),
                 "value": 4000 * done1 / (ms1 * 1e-3), "unit": "cell-steps/s", "ms_per_step": ms1 / max(done1, 1),
                 "final_time": s1.time, "tuning": tuning1}
        s1.close()
        if tuning1 is not None:
            tune.set_chem_tuning(ctx, *restore)
        if not args.no_cpu and args.det1d_cpu_steps > 0:
            oracle = _oracle(10)
            g1 = oracle.make_grid(2000, 2, l1["dx"], l1["dy"], periodic=(0, 0), bc_lo=(0, 0), bc_hi=(1, 0),
                                  inlet=l1["inlet"])
            Ug1 = oracle.ghosted(U1.transpose(1, 2, 0))
            oracle.set_flux_threads(0)
            t0 = time.perf_counter()
            for _ in range(args.det1d_cpu_steps):
                Ug1, _, st1, _ = oracle.strang_step(g1, Ug1, oracle.cfl_dt(g1, Ug1, args.cfl))
            el1 = time.perf_counter() - t0
            oracle.set_flux_threads(1)
            det1d["cpu_baseline"] = {"value": 4000 * args.det1d_cpu_steps / el1, "unit": "cell-steps/s",
                                     "cores": os.cpu_count(), "kind": "port",
                                     "sample": "steps 1..%d of the same run, every loop on all host threads" %
                                               args.det1d_cpu_steps}

    amr = None
    if args.amr_steps > 0:
        # the 3-level block-AMR oblique detonation (base 512 x 256, ratio 2, 32 x 32 blocks,
        # density-gradient tags, regrid every 4 steps): leaf cell-steps/s over amr_steps
        # coarse steps from the uniform free stream, graph-captured steps
        ctx9a = hf.Context("H2_Li", device=local)
        Uw, lw = W.wedge(nx=512, ny=256)
        amr = {"workload": "oblique detonation over a 30 deg wedge, Mach 7 stoichiometric H2/air at 0.1 atm / 300 K, "
                           "base 512x256, max_level 2, 32x32 blocks, density tag 0.05, regrid every 4 steps; %d "
                           "coarse steps from the uniform free stream" % args.amr_steps}
        am = None
        try:
            am = hf.AmrStepper(ctx9a, hf.make_level(**lw), torch.from_numpy(Uw).cuda(), max_level=2, block=32,
                               tag_buffer=2, regrid_interval=4, tags=dict(density_tag=0.05))
            leaf0 = sum(am.info(l)["leaf_cells"] for l in range(3))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            leaf_steps = 0
            for _ in range(args.amr_steps):
                leaf_steps += sum(am.info(l)["leaf_cells"] for l in range(3))
                am.step(cfl=args.cfl)
            e1.record()
            torch.cuda.synchronize()
            ams = e0.elapsed_time(e1)
            amr.update({"value": leaf_steps / (ams * 1e-3), "unit": "leaf cell-steps/s",
                        "ms_per_step": ams / args.amr_steps, "final_time": am.time,
                        "leaf_cells": [am.info(l)["leaf_cells"] for l in range(3)], "leaf_cells_at_start": leaf0,
                        "graph_steps": am.stats()["graph_steps"]})
        except hf.HyperFlowError as e:  # reported, not fatal to the headline line
            amr["error"] = str(e)
        if am is not None:
            am.close()
        ctx9a.close()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    pk = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    chem_ms, chem_n = tm["chem"]
    launch_ms = probe["launch_ms"]
    bytes_per_launch = 2 * nv * 8 * cells  # read and write every cell state once
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    fp64_peak = ctx.fp64_peak()
    fp64 = {"peak": fp64_peak, "unit": "GFLOP/s",
            "peak_source": "measured in this run (hf_fp64_peak: independent DFMA chains on every SM)",
            "executed": {"achieved": EXECUTED_FLOPS_PER_ATTEMPT * probe["gpu_attempts"] / (launch_ms * 1e-3) / 1e9,
                         "flops_per_attempt": EXECUTED_FLOPS_PER_ATTEMPT,
                         "note": "ncu FP64 instruction count per integrator step attempt (one capture of this "
                                 "probe launch at full size) x the launch's attempts"}}
    if "algorithmic" in probe:
        alg = probe["algorithmic"]
        fp64["achieved"] = alg["flops"] / (launch_ms * 1e-3) / 1e9
        fp64["frac"] = fp64["achieved"] / fp64_peak
        fp64["executed"]["frac"] = fp64["executed"]["achieved"] / fp64_peak
        fp64["algorithmic_flops_per_launch"] = alg["flops"]
    roof = {"kernel": "k_chem_batched", "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": PROBE_TRAFFIC,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one capture of this probe "
                              "launch at full size (bench.py --probe-only --warmup 11, its second k_chem_batched launch)",
            "algorithmic_bytes_per_launch": bytes_per_launch, "launch_ms": launch_ms,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in pk else "fallback 6.8 TB/s",
            "fp64": fp64,
            "whole_step": {"bytes_per_cell_step": BYTES_PER_CELL_STEP,
                           "achieved": BYTES_PER_CELL_STEP * value / 1e9, "frac": BYTES_PER_CELL_STEP * value / 1e9 / hbm,
                           "unit": "GB/s"},
            "note": "the chemistry kernel is FP64-pipe bound, not HBM bound: the HBM fraction is reported per the "
                    "contract, the fp64 object (algorithmic FP64 work of the launch's input over its time) is the "
                    "binding roof"}
    # the flux path's roofline: a subsonic face stencil of the fresh gas (x direction)
    mid = max(0, min(args.nx // 2, args.nx - 4))
    ff = _oracle(nv - 3).flux_flops(U0[:, 0, mid:mid + 4].T, 0, 3)
    roof["flux"] = flux_roofline(ff, nv, cells, tm["flux"][0] / args.steps, fp64_peak, hbm)
    accuracy = None
    if not args.no_cpu:
        # error of the GPU results against the tight FP64 oracle (rtol 1e-12,
        # atol 1e-20): 2 graph steps of a 2048 x 4 strip of the same detonation (the
        # oracle replays the GPU's step sizes), and 512 cells of the uneven chemistry batch
        rows = 4
        Us, ls = W.det2d(seed=0, diluent="AR", nx=args.nx, ny=rows)
        ss = hf.Stepper(ctx, hf.make_level(**ls), torch.from_numpy(Us).cuda(), flux=args.flux, chem="batched")
        dts = [ss.step(cfl=args.cfl) for _ in range(2)]
        got = ss.state().cpu().numpy().transpose(1, 2, 0).reshape(-1, nv)
        ss.close()
        t0 = time.perf_counter()
        ref = tight_oracle_strip(Us, ls, dts, args.nx, rows)
        accuracy = {"oracle": "CPU restatement, Rodas4 at rtol 1e-12 / atol 1e-20", "target": "T rel <= 1e-6",
                    "strip": dict(tight_errors(got, ref), cells=args.nx * rows, steps=2,
                                  oracle_seconds=time.perf_counter() - t0)}
        if chem_sample is not None:
            # per cell with a step limit the tight tolerance needs (the 5000-step limit
            # of the reference's integrator is for its own rtol 1e-8)
            oracle = _oracle(10)
            gotc, U0c, dtc_s = chem_sample
            refc = np.empty_like(U0c)
            ok = True
            for k in range(len(U0c)):
                refc[k], stc, _ = oracle.chem_advance(U0c[k], dtc_s[k], rtol=1e-12, atol=1e-20, max_steps=10 ** 6)
                ok = ok and stc == 0
            if ok:
                accuracy["chem_batch"] = dict(tight_errors(gotc, refc), cells=len(U0c))

    cpu = None
    if not args.no_cpu:
        # the same window as the GPU arm on a 2048 x 32 strip, all host threads on every
        # loop, and the reference's threading (serial flux loop) on its first steps
        cb = cpu_window(args.steps, args.warmup, nx=args.nx, rows=min(STRIP_ROWS, args.ny),
                        serial_steps=min(args.steps, 4), cfl=args.cfl)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "ms_per_step", "cells_per_step",
                                  "reference_threading")}
    config = workload_config(args)
    config.update({"form": "%s flux + batched chemistry" % args.flux,
                   "l2": "device-resident graph steps, each reading and writing 4 state buffers of 109 MB (inputs "
                         "larger than L2), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"})
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
        "clocks": ck, "e2e": e2e, "gpu_launches": cnt["kernel_launches"],
        "breakdown_ms_per_step": {"flux": tm["flux"][0] / args.steps, "chem": chem_ms / args.steps,
                                  "other": tm["other"][0] / args.steps},
        "chem_attempts_per_cell_step": cnt["chem_steps"] / max(cnt["chem_cell_calls"], 1),
        "plain": plain, "batched_over_plain": (value / plain["value"]) if plain else None,
        "step_loop": step_loop, "curve": curve, "chem_batch_uneven": chem_batch, "tuning": tuning,
        "roofline": roof, "roofline_probe": probe, "cpu_baseline": cpu, "accuracy": accuracy, "adjoint": adjoint,
        "det1d": det1d, "amr": amr,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
