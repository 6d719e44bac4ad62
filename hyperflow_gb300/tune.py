"""Autotuner of the step's launch settings, by measurement on the caller's workload.

* Chemistry (hf_set_chem_tuning): the blocks of 64 lanes per SM the batched queue kernel
  is built for (its per-lane register budget) and the cooperative threshold (cells that
  took at least 2^b - 1 step attempts in the previous call are integrated by groups of 8
  lanes, 4 cells per warp; 16, the default: never, and the kernel without that phase).
  Each candidate runs the batched chemistry three times on the same sample call (the
  chemistry input of a Strang step of the workload): the first two build the per-cell
  history (cost order, warm-started step sizes) as consecutive steps do, the third is
  timed with CUDA events.  A candidate replaces the default only when it is more than
  MARGIN faster on the sample: one call stands for the steps that follow, and a
  cooperative setting whose queue stays empty on the sample can still engage, and cost,
  in later steps.
* Stepper chemistry (tune_stepper): the same settings timed over a few whole graph
  steps of the caller's stepper from one start state, each candidate from a fresh
  stepper (its history builds up over the steps as it does in a run, so a cooperative
  setting shows whether its queue engages and pays).  Small, tail-bound problems (a 1D
  detonation of a few thousand cells) gain from the cooperative phase; large ones lose
  throughput to it.
* Flux form: one Euler stage of the workload's state with the plain per-face kernels and
  with the fused TMA-tile kernel (32 x 7 cells per CTA), each timed after a warm-up; the
  faster form is returned for the caller's stepper.

Settings change launch shapes only: results agree to rounding across candidates and are
reproducible for a fixed setting.
"""
import ctypes

import torch

from . import _lib as L
from . import solver as S

CHEM_DEFAULT = (4, 16)
CHEM_CANDIDATES = [CHEM_DEFAULT, (5, 16), (6, 16), (8, 16), (4, 3), (4, 5), (4, 7)]
MARGIN = 0.03
STEP_CANDIDATES = [CHEM_DEFAULT, (4, 3), (4, 5), (4, 7)]


def pick(sweep, key, default=CHEM_DEFAULT, margin=MARGIN):
    """The sweep entry to apply: the fastest by `key` when it is more than `margin` faster
    than the `default` setting's entry, else the default's (the fastest when the sweep
    has no default entry)."""
    best = min(sweep, key=lambda r: r[key])
    base = [r for r in sweep if (r["blocks_per_sm"], r["coop_min_bucket"]) == tuple(default)]
    if base and best[key] >= (1.0 - margin) * base[0][key]:
        return base[0]
    return best


def get_chem_tuning(ctx):
    m, c = ctypes.c_int32(0), ctypes.c_int32(0)
    ctx.lib.hf_get_chem_tuning(ctypes.byref(m), ctypes.byref(c))
    return int(m.value), int(c.value)


def set_chem_tuning(ctx, blocks_per_sm=0, coop_min_bucket=0):
    ctx.check(ctx.lib.hf_set_chem_tuning(int(blocks_per_sm), int(coop_min_bucket)), "set_chem_tuning")


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def tune_chemistry(ctx, X, dt, candidates=CHEM_CANDIDATES, apply=True):
    """X: (NV, n) float64 CUDA tensor, the input of one chemistry call over dt (not
    modified).  Returns {"best": (blocks_per_sm, coop_min_bucket), "sweep": [...]} and, with
    apply, leaves the best setting in force."""
    before = get_chem_tuning(ctx)
    sweep = []
    try:
        for minb, coop in candidates:
            set_chem_tuning(ctx, minb, coop)
            cb = S.ChemistryBatch(ctx, "batched")
            for _ in range(2):
                cb.advance(X.clone(), dt)
            field = X.clone()
            c0 = ctx.counters()
            torch.cuda.synchronize()
            e0, e1 = _events()
            e0.record()
            cb.advance(field, dt)
            e1.record()
            torch.cuda.synchronize()
            c1 = ctx.counters()
            sweep.append({"blocks_per_sm": minb, "coop_min_bucket": coop, "ms": e0.elapsed_time(e1),
                          "coop_cells": c1["chem_coop_cells"] - c0["chem_coop_cells"],
                          "attempts": c1["chem_steps"] - c0["chem_steps"]})
            del field
    finally:
        set_chem_tuning(ctx, *before)
    best = pick(sweep, "ms")
    if apply:
        set_chem_tuning(ctx, best["blocks_per_sm"], best["coop_min_bucket"])
    return {"best": (best["blocks_per_sm"], best["coop_min_bucket"]), "sweep": sweep}


def tune_flux(ctx, level, U, dt, repeats=3):
    """U: (NV, ny, nx) state of a one-patch level; dt: a step of it (stages of dt/2 are
    timed).  Returns {"best": "plain"|"fused", "ms": {form: ms per stage}}."""
    nv, ny, nx = U.shape
    pa = S.PatchArray(nv, nx, ny)
    pa.interior().copy_(U)
    S.fill(ctx, level, pa)
    out = pa.like()
    ms = {}
    for name, form in (("plain", L.HF_FLUX_PLAIN), ("fused", L.HF_FLUX_FUSED)):
        S.euler_stage(ctx, level, pa, out, 0.5 * dt, form=form)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        for _ in range(repeats):
            S.euler_stage(ctx, level, pa, out, 0.5 * dt, form=form)
        e1.record()
        torch.cuda.synchronize()
        ms[name] = e0.elapsed_time(e1) / repeats
    return {"best": min(ms, key=ms.get), "ms": ms}


def tune_stepper(ctx, level, U, cfl, flux="plain", warm=2, steps=6, candidates=STEP_CANDIDATES, apply=True):
    """U: (NV, ny, nx) state; the batched chemistry settings timed over `steps` graph steps
    (after `warm` steps) of a fresh stepper per candidate.  Returns {"best": (...),
    "sweep": [{"blocks_per_sm", "coop_min_bucket", "ms_per_step", "coop_cells"}]} and, with
    apply, leaves the best setting in force (the default unless one beats it by MARGIN)."""
    before = get_chem_tuning(ctx)
    sweep = []
    try:
        for minb, coop in candidates:
            set_chem_tuning(ctx, minb, coop)
            st = S.Stepper(ctx, level, U, flux=flux, chem="batched")
            try:
                for _ in range(warm):
                    st.step(cfl=cfl)
                c0 = ctx.counters()
                torch.cuda.synchronize()
                e0, e1 = _events()
                e0.record()
                st.run(steps, cfl=cfl)
                e1.record()
                torch.cuda.synchronize()
                c1 = ctx.counters()
            finally:
                st.close()
            sweep.append({"blocks_per_sm": minb, "coop_min_bucket": coop, "ms_per_step": e0.elapsed_time(e1) / steps,
                          "coop_cells": c1["chem_coop_cells"] - c0["chem_coop_cells"]})
    finally:
        set_chem_tuning(ctx, *before)
    best = pick(sweep, "ms_per_step")
    if apply:
        set_chem_tuning(ctx, best["blocks_per_sm"], best["coop_min_bucket"])
    return {"best": (best["blocks_per_sm"], best["coop_min_bucket"]), "sweep": sweep}
