#!/usr/bin/env python3
"""Benchmark: cell-steps/s of the Strang-split reacting-Euler step on the 2D H2/O2/Ar
detonation (2048 x 512 cells, FP64), one GPU per rank.

One "step" is one full Strang step of the whole grid: flow(dt/2) (two Euler stages
and the Heun combine), react(dt), flow(dt/2), with the CFL dt.  The headline value
is the device-resident run of CUDA-graph steps: plain flux kernels (ghost fill, face,
update; faster than the fused TMA-tile kernel on this FP64-bound path, --flux fused
selects it) and the batched work-queue chemistry; the plain drop-in form (face/update
kernels + one-thread-per-cell chemistry, host-driven steps) is timed beside it.  `e2e`
runs the same steps through the public stepper API with the state in pinned HOST
memory, copied in and out every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun) every rank runs an independent replica (one grid per GPU; the
step of one grid is not sharded): value = all ranks' cell-steps
over the slowest rank's time.  --impl reference times the CPU restatement of the
reference (the reference itself needs Cantera, SUNDIALS and AMReX, absent here) on
this host's cores over a bounded sample of the same workload.
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
# ncu counts of k_chem_batched on the 512 x 128 case (profiles/k_chem_batched_det2d_512x128.md):
# FP64 flops per integrator step attempt (DFMA x 2 + DADD + DMUL thread instructions of
# the fourth chemistry launch over its 1.322e6 attempts), and the DRAM bytes of that
# launch.  Those bytes are 13.6 MB of state plus ~42 MB of spill write-back; the spill
# part follows the persistent grid's local-memory footprint, not the cell count, so the
# capture is reported as measured and the full-size traffic is left null.
FLOPS_PER_ATTEMPT = 1.79e4
TRAFFIC_CAPTURE = {"workload": "2D H2/O2/Ar detonation 512x128, fourth chemistry launch", "cells": 65536,
                   "attempts": 1.322e6, "dram_read_bytes": 11.8e6, "dram_write_bytes": 43.7e6,
                   "algorithmic_bytes": 2 * 13 * 8 * 65536}
NX, NY = 2048, 512


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=8)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--plain-steps", type=int, default=None, help="steps timed for the plain form (default: steps)")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cfl", type=float, default=0.5)
    p.add_argument("--flux", default="plain", choices=["fused", "plain"], help="flux form of the headline run")
    p.add_argument("--chem", default="persistent", choices=["persistent", "plain"],
                   help="chemistry form of the headline run")
    p.add_argument("--chem-cells", type=int, default=1 << 18,
                   help="cells of the extra chemistry-only batch (0 = skip)")
    p.add_argument("--adj-cells", type=int, default=4096,
                   help="0D H2/air cells of the adjoint measurement (0 disables it)")
    p.add_argument("--adj-calls", type=int, default=2000, help="chemistry calls (of 1e-7 s) per adjoint run")
    p.add_argument("--adj-objectives", default="ignition_delay",
                   help="comma-separated: ignition_delay, peak_pressure, final_T")
    p.add_argument("--adj1d-cells", type=int, default=1000,
                   help="cells of the 1D detonation whose run is differentiated (0 disables it)")
    p.add_argument("--adj1d-steps", type=int, default=1000, help="CFL Strang steps of that run")
    p.add_argument("--det1d-steps", type=int, default=100,
                   help="timed steps of the 1D detonation sample, 2000 x 2 cells (0 disables it)")
    p.add_argument("--amr-steps", type=int, default=8,
                   help="timed steps of the 3-level block-AMR wedge sample (0 disables it)")
    p.add_argument("--nx", type=int, default=NX)
    p.add_argument("--ny", type=int, default=NY)
    return p.parse_args()


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


# ------------------------------------------------------------------ CPU (oracle) leg
def cpu_sample(steps=2, warm=1, rows=4, threads=0, nx=NX, flux_threads=0):
    """Oracle Strang steps on a periodic strip (nx x rows) of the same workload.
    flux_threads 1: the reference's serial flux loop; 0: OpenMP over all host threads
    (same results).  Chemistry always uses OpenMP dynamic,8 over `threads` threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from hyperflow_gb300 import workloads as W
    oracle.build()
    oracle.set_species(10)
    oracle.set_flux_threads(flux_threads)
    U, lvd = W.det2d(seed=0, diluent="AR", nx=nx, ny=rows)
    g = oracle.make_grid(nx, rows, 1e-4, 1e-4, periodic=(0, 1), bc_lo=(0, 0), bc_hi=(1, 0), inlet=lvd["inlet"])
    Ug = oracle.ghosted(U.transpose(1, 2, 0))
    for _ in range(warm):
        dt = oracle.cfl_dt(g, Ug, 0.5)
        Ug, _, st, _ = oracle.strang_step(g, Ug, dt, threads=threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        dt = oracle.cfl_dt(g, Ug, 0.5)
        Ug, _, st, _ = oracle.strang_step(g, Ug, dt, threads=threads)
        if st:
            raise RuntimeError("oracle step failed")
    el = time.perf_counter() - t0
    oracle.set_flux_threads(1)
    cores = threads or os.cpu_count()
    flux = "serial flux loop (the reference's threading)" if flux_threads == 1 else "OpenMP flux loops"
    return {"value": nx * rows * steps / el, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": "%d Strang steps (after %d warm-up) of a %dx%d periodic strip of the 2D detonation; "
                      "%s, OpenMP dynamic,8 chemistry" % (steps, warm, nx, rows, flux),
            "seconds": el}


def tight_errors(states, ref_states):
    """T relative and Y_k absolute errors (max over cells) of AoS states against the
    tight oracle's; Y_k = rho Y_k / rho of the reference."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.set_species(10)
    Tg, Tr = oracle.properties(states)[2], oracle.properties(ref_states)[2]
    rho = ref_states[:, :10].sum(1)
    return {"T_rel_max": float(np.max(np.abs(Tg - Tr) / Tr)),
            "Y_abs_max": float(np.max(np.abs(states[:, :10] - ref_states[:, :10]) / rho[:, None]))}


def tight_oracle_strip(U0, lvd, dts, nx, rows):
    """The oracle's Strang steps of a strip at rtol 1e-12 / atol 1e-20 with the given
    step sizes (AoS interior states)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    oracle.set_species(10)
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


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # a bounded sample: K/4 timed oracle steps after one warm-up step on a 4-row strip,
    # every loop on all host threads (flux loops included: a stronger baseline than
    # the reference's serial flux loop, same results)
    cb = cpu_sample(steps=max(1, args.steps // 4), warm=1, rows=4, nx=args.nx, flux_threads=0)
    line = {"metric": METRIC, "value": cb["value"], "unit": "cell-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * args.nx * args.ny / cb["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "2D H2/O2/Ar detonation %dx%d, 64-column hot band, periodic y" % (args.nx, args.ny),
                       "cells": args.nx * args.ny},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (Cantera/SUNDIALS/AMReX) cannot be built here; this arm times the CPU "
                    "restatement of its path"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
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
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def slowest(x):
        return max_over_ranks(dist, x, "cuda")

    def timed(flux, chem, steps, warmup, timing=False, clocks=None, resident=False):
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=flux, chem=chem)
        for _ in range(warmup):
            st.step(cfl=args.cfl)
        c0 = ctx.counters()
        if timing:
            ctx.set_timing(True)
        barrier()
        if clocks:
            clocks.start()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        if resident:
            # device-resident run: graph steps back to back, no host round trip; every
            # step reads and writes 4 state buffers of 109 MB (> 129 MB L2), no flush
            st.run(steps, cfl=args.cfl)
        else:
            for _ in range(steps):
                st.step(cfl=args.cfl)
                flush.zero_()
        ev1.record()
        barrier()
        ms = ev0.elapsed_time(ev1)
        ck = clocks.stop() if clocks else None
        tm = ctx.timing() if timing else None
        if timing:
            ctx.set_timing(False)
        c1 = ctx.counters()
        st.close()
        return slowest(ms), ck, tm, {k: c1[k] - c0[k] for k in c1}

    clocks = Clocks(local)
    ms, ck, tm, cnt = timed(args.flux, args.chem, args.steps, args.warmup, timing=True, clocks=clocks,
                            resident=args.chem == "persistent")
    value = replica_value(world, cells, args.steps, ms)
    plain = None
    if not args.no_plain:
        ps = args.plain_steps or args.steps
        pms, _, ptm, pcnt = timed("plain", "plain", ps, args.warmup, timing=True)
        plain = {"value": replica_value(world, cells, ps, pms), "ms_per_step": pms / ps, "steps": ps,
                 "chem_ms_per_step": ptm["chem"][0] / ps, "flux_ms_per_step": ptm["flux"][0] / ps}

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
        # bounded sample of the 1D planar detonation (2000 x 2 cells on 0.1 m, 20-cell
        # driver at 40 atm / 3000 K, Ar diluent): the same graph-captured steps as the
        # headline run; few stiff cells, so one cell's chemistry sets the step time
        U1, l1 = W.det1d(diluent="AR", nx=2000)
        s1 = hf.Stepper(ctx, hf.make_level(**l1), torch.from_numpy(U1).cuda(), flux=args.flux, chem=args.chem)
        for _ in range(args.warmup):
            s1.step(cfl=args.cfl)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        done1 = s1.run(args.det1d_steps, cfl=args.cfl)
        e1.record()
        torch.cuda.synchronize()
        ms1 = e0.elapsed_time(e1)
        det1d = {"workload": "1D H2/O2/Ar detonation 2000x2 cells on 0.1 m, 20-cell driver at 40 atm/3000 K, "
                             "reflecting left/top/bottom, transmissive right, CFL %.2f; %d device-resident steps after "
                             "%d warm-up steps" % (args.cfl, done1, args.warmup),
                 "value": 4000 * done1 / (ms1 * 1e-3), "unit": "cell-steps/s", "ms_per_step": ms1 / max(done1, 1)}
        s1.close()

    amr = None
    if args.amr_steps > 0:
        # bounded sample of the 3-level block-AMR oblique detonation (base 512 x 256,
        # ratio 2, 32 x 32 blocks, density-gradient tags, regrid every 4 steps): leaf
        # cell-steps/s over the timed steps; host-driven steps (one status read per
        # stage), CUDA events around them
        from hyperflow_gb300 import workloads as W2
        ctx9a = hf.Context("H2_Li", device=local)
        Uw, lw = W2.wedge(nx=512, ny=256)
        amr = {"workload": "oblique detonation over a 30 deg wedge, Mach 7 stoichiometric H2/air at 0.1 atm / 300 K, "
                           "base 512x256, max_level 2, 32x32 blocks, density tag 0.05, regrid every 4 steps; "
                           "%d timed steps after %d warm-up steps from the uniform free stream" % (
                               args.amr_steps, args.warmup)}
        am = None
        try:
            am = hf.AmrStepper(ctx9a, hf.make_level(**lw), torch.from_numpy(Uw).cuda(), max_level=2, block=32,
                               tag_buffer=2, regrid_interval=4, tags=dict(density_tag=0.05))
            for _ in range(args.warmup):
                am.step(cfl=args.cfl)
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
                        "ms_per_step": ams / args.amr_steps,
                        "leaf_cells": [am.info(l)["leaf_cells"] for l in range(3)], "leaf_cells_at_start": leaf0})
        except hf.HyperFlowError as e:  # reported, not fatal to the headline line
            amr["error"] = str(e)
        if am is not None:
            am.close()
        ctx9a.close()

    e2e = None
    if not args.no_e2e:
        st = hf.Stepper(ctx, level, torch.from_numpy(U0).cuda(), flux=args.flux, chem=args.chem)
        host = torch.from_numpy(U0.copy()).pin_memory()
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
        e2e = {"value": replica_value(world, cells, args.steps, el * 1e3), "unit": "cell-steps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    pk = peaks()
    chem_ms, chem_n = tm["chem"]
    bytes_per_launch = 2 * nv * 8 * cells  # read and write every cell state once
    achieved = bytes_per_launch / (chem_ms / max(chem_n, 1) * 1e-3) / 1e9
    hbm = pk.get("hbm_gbs", 6800.0)
    # FP64 roof: flops per integrator step attempt counted by ncu on this kernel
    # (DFMA x2 + DADD + DMUL thread instructions / attempts of the launch, 512 x 128
    # case), times the attempts counted live in the timed steps, over the live time
    fp64_peak = ctx.fp64_peak()
    fp64_achieved = FLOPS_PER_ATTEMPT * cnt["chem_steps"] / (chem_ms * 1e-3) / 1e9
    roof = {"kernel": "k_chem_batched", "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": None, "traffic_capture": TRAFFIC_CAPTURE,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in pk else "fallback 6.8 TB/s",
            "fp64": {"achieved": fp64_achieved, "peak": fp64_peak, "unit": "GFLOP/s", "frac": fp64_achieved / fp64_peak,
                     "peak_source": "measured in this run (hf_fp64_peak: independent DFMA chains on every SM)",
                     "flops_per_attempt": FLOPS_PER_ATTEMPT},
            "note": "the chemistry kernel is FP64-pipe bound, not HBM bound: the HBM fraction is reported per "
                    "the contract, the fp64 object is the binding roof; traffic_capture = ncu dram bytes of one launch "
                    "of the small case (spill write-back dominates it, so it does not scale to the full launch by cells)"}
    accuracy = None
    if not args.no_cpu and rank == 0:
        # error of the GPU results against the tight FP64 oracle (rtol 1e-12,
        # atol 1e-20): 2 graph steps of a 2048 x 4 strip of the same detonation (the
        # oracle replays the GPU's step sizes), and 512 cells of the uneven chemistry batch
        rows = 4
        Us, ls = W.det2d(seed=0, diluent="AR", nx=args.nx, ny=rows)
        ss = hf.Stepper(ctx, hf.make_level(**ls), torch.from_numpy(Us).cuda(), flux=args.flux, chem=args.chem)
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
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.set_species(10)
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
        # all host threads on every loop (the baseline), and the reference's threading
        # (serial flux loop) beside it
        cb = cpu_sample(steps=4, warm=1, rows=32, nx=args.nx, flux_threads=0)
        ca = cpu_sample(steps=2, warm=1, rows=32, nx=args.nx, flux_threads=1)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        cpu["reference_threading"] = {k: ca[k] for k in ("value", "sample")}
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "2D H2/O2/Ar detonation %dx%d, 64-column hot band at 40 atm/3000 K, +-1%% density "
                               "perturbation, periodic y, CFL %.2f" % (args.nx, args.ny, args.cfl),
                   "cells": cells, "species": 10, "mechanism": "H2_Li + inert AR extension",
                   "chem_tolerances": "rtol 1e-8 atol 1e-15", "form": "%s flux + batched chemistry" % args.flux,
                   "l2": "headline: device-resident run, each step reads and writes 4 state buffers of 109 MB "
                         "(inputs larger than L2), no flush; plain form: 256 MB buffer written between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": ck, "e2e": e2e, "gpu_launches": cnt["kernel_launches"],
        "breakdown_ms_per_step": {"flux": tm["flux"][0] / args.steps, "chem": tm["chem"][0] / args.steps,
                                  "other": tm["other"][0] / args.steps},
        "chem_attempts_per_cell_step": cnt["chem_steps"] / max(cnt["chem_cell_calls"], 1),
        "plain": plain, "batched_over_plain": (value / plain["value"]) if plain else None,
        "chem_batch_uneven": chem_batch,
        "roofline": roof, "cpu_baseline": cpu, "accuracy": accuracy, "adjoint": adjoint, "det1d": det1d,
        "amr": amr,
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
