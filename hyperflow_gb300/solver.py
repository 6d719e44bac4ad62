"""Python mirror of the reference's per-block interface over the C ABI.

Names follow HyperFlow V3: ``properties``/``admissible``/``hllc``
(src/physics.cpp:4-48), ``ChemistryBatch.advance`` (src/chemistry_batch.cpp:21-50),
``fill`` / ``FlowBoundary`` (src/BlockAMR.cpp:137-146, src/FlowBoundary.hpp),
``ConservativeInterp.interp`` (src/ConservativeInterp.cpp), and a ``Stepper``
running the loop body of ``BlockAMR::run`` (src/BlockAMR.cpp:409-419).  Errors
raise like the reference: ``DomainError`` where it throws std::domain_error,
``RuntimeError`` for a failed chemistry cell ("chemistry cell k: ...").

Device data are torch float64 CUDA tensors used as plain memory: states are
structure-of-arrays, shape (NV, ...), NV = NS + 3, component order
rhoY_0..rhoY_{NS-1}, rho*u, rho*v, rho*E (src/solver.hpp:17-25).
"""
import ctypes

import numpy as np
import torch

from . import _lib as L

SPECIES = ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2", "AR"]
BC = {"reflecting": L.HF_BC_REFLECTING, "transmissive": L.HF_BC_TRANSMISSIVE, "inflow": L.HF_BC_INFLOW,
      "wedge": L.HF_BC_WEDGE}


class HyperFlowError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (L.STATUS_NAMES.get(status, status), message))
        self.status = status


class DomainError(HyperFlowError):
    """std::domain_error of the reference (inadmissible state)."""


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _need_cuda64(t, name):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64):
        raise TypeError("%s must be a float64 CUDA tensor" % name)


def _need_state(ctx, t, name):
    """A float64 CUDA state whose leading dimension is the context's NV = NS + 3."""
    _need_cuda64(t, name)
    if t.dim() < 2 or t.shape[0] != ctx.nv:
        raise ValueError("%s must have %d components (the mechanism's %d species + 3), got shape %s"
                         % (name, ctx.nv, ctx.ns, tuple(t.shape)))


class Context:
    """hf_init/hf_destroy: one mechanism on one device (src/BlockAMR.cpp:29-30)."""

    def __init__(self, mechanism="H2_Li", device=None):
        self.lib = L.load()
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        h = ctypes.c_void_p()
        st = self.lib.hf_init(mechanism.encode() if mechanism else None, int(device), ctypes.byref(h))
        if st != L.HF_OK:
            raise HyperFlowError(st, "hf_init(%r) failed" % mechanism)
        self.h = h
        self.ns = self.lib.hf_nspecies(h)
        self.nv = self.ns + 3

    def close(self):
        if getattr(self, "h", None):
            self.lib.hf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what=""):
        if st == L.HF_OK:
            return
        msg = (self.lib.hf_last_error(self.h) or b"").decode()
        cls = DomainError if st in (L.HF_ERR_INADMISSIBLE, L.HF_ERR_NEGATIVE, L.HF_ERR_FACE,
                                    L.HF_ERR_COMBINE) else HyperFlowError
        raise cls(st, (what + ": " if what else "") + msg)

    def counters(self):
        c = L.Counters()
        self.lib.hf_get_counters(self.h, ctypes.byref(c))
        return {f: getattr(c, f) for f, _ in L.Counters._fields_}

    def set_timing(self, enable=True):
        """Per-kernel-class CUDA-event timing (resets the sums)."""
        self.lib.hf_set_timing(self.h, int(bool(enable)))

    def timing(self):
        """{"flux"|"chem"|"other": (ms, launches)} since set_timing(True)."""
        ms = (ctypes.c_double * 3)()
        n = (ctypes.c_int64 * 3)()
        self.lib.hf_get_timing(self.h, ms, n)
        return {k: (ms[i], n[i]) for i, k in enumerate(("flux", "chem", "other"))}

    def fp64_peak(self):
        """Measured FP64 FMA throughput of the device in GFLOP/s (hf_fp64_peak)."""
        g = ctypes.c_double(0.0)
        self.check(self.lib.hf_fp64_peak(self.h, ctypes.byref(g), _stream()), "fp64_peak")
        return g.value

    def set_rate_scale(self, scale=None):
        if scale is None:
            self.check(self.lib.hf_set_rate_scale(self.h, None))
        else:
            arr = (ctypes.c_double * 21)(*[float(s) for s in scale])
            self.check(self.lib.hf_set_rate_scale(self.h, arr))


# ------------------------------------------------------------------ physics.cpp
def properties(ctx, q):
    """Batched properties(): q (NV, count) -> (p, a, T, status); status 1 = inadmissible."""
    _need_cuda64(q, "q")
    q = q.contiguous()
    n = q.shape[1]
    p, a, T = (torch.empty(n, dtype=torch.float64, device=q.device) for _ in range(3))
    st = torch.empty(n, dtype=torch.int32, device=q.device)
    r = ctx.lib.hf_properties(ctx.h, _ptr(q), n, n, _ptr(p), _ptr(a), _ptr(T), _ptr(st), _stream())
    if r not in (L.HF_OK, L.HF_ERR_INADMISSIBLE):
        ctx.check(r, "properties")
    return p, a, T, st


def admissible(ctx, q):
    """admissible() (physics.cpp:45-48) for each column of q."""
    return properties(ctx, q)[3] == 0


def hllc(ctx, left, right, props_l, props_r, direction):
    """hllc() (physics.cpp:17-38): left/right (NV, n), props (3, n) = (p, a, T); direction 0=x, 1=y."""
    for t, nm in ((left, "left"), (right, "right"), (props_l, "props_l"), (props_r, "props_r")):
        _need_cuda64(t, nm)
    n = left.shape[1]
    left, right = left.contiguous(), right.contiguous()
    props_l, props_r = props_l.contiguous(), props_r.contiguous()
    out = torch.empty_like(left)
    ctx.check(ctx.lib.hf_hllc(ctx.h, _ptr(left), _ptr(right), _ptr(props_l), _ptr(props_r), n, n, int(direction),
                              _ptr(out), _stream()), "hllc")
    return out


# ------------------------------------------------------------------ grids
def make_level(nx, ny, dx, dy, xlo=0.0, ylo=0.0, periodic=(0, 0), boundary_lo=("reflecting", "reflecting"),
               boundary_hi=("transmissive", "reflecting"), inlet=None, wedge_start=0.0):
    """hf_level from the reference's case keys (BlockAMR.cpp:38-59 defaults)."""
    lv = L.Level()
    lv.nx, lv.ny, lv.dx, lv.dy, lv.xlo, lv.ylo = int(nx), int(ny), float(dx), float(dy), float(xlo), float(ylo)
    for d in range(2):
        lv.periodic[d] = int(periodic[d])
        lo, hi = boundary_lo[d], boundary_hi[d]
        lv.bc_lo[d] = BC[lo] if isinstance(lo, str) else int(lo)
        lv.bc_hi[d] = BC[hi] if isinstance(hi, str) else int(hi)
    if inlet is not None:
        for n, v in enumerate(inlet):
            lv.inlet[n] = float(v)
    lv.wedge_start = float(wedge_start)
    return lv


class PatchArray:
    """One patch with ng ghost layers: a (NV, ny+2ng, pitch) float64 CUDA tensor."""

    def __init__(self, nv, nx, ny, ng=2, ilo=0, jlo=0, device="cuda", pitch=None):
        self.nv, self.nx, self.ny, self.ng = nv, nx, ny, ng
        self.pitch = pitch or ((nx + 2 * ng + 1) // 2 * 2)
        self.rows = ny + 2 * ng
        self.data = torch.zeros(nv, self.rows, self.pitch, dtype=torch.float64, device=device)
        p = L.Patch()
        p.ilo, p.jlo, p.nx, p.ny, p.ng = ilo, jlo, nx, ny, ng
        p.pitch, p.comp_stride, p.offset = self.pitch, self.rows * self.pitch, 0
        self.patch = p

    def interior(self):
        g = self.ng
        return self.data[:, g:g + self.ny, g:g + self.nx]

    def ghosted(self):
        """(NV, ny+2ng, nx+2ng) view including ghosts."""
        return self.data[:, :, :self.nx + 2 * self.ng]

    def like(self):
        o = PatchArray(self.nv, self.nx, self.ny, self.ng, self.patch.ilo, self.patch.jlo, self.data.device,
                       self.pitch)
        return o


def fill(ctx, level, patch_array):
    """Ghost fill of a one-patch level (BlockAMR::fill + FlowBoundary)."""
    ctx.check(ctx.lib.hf_fill_ghosts(ctx.h, ctypes.byref(level), ctypes.byref(patch_array.patch), 1,
                                     _ptr(patch_array.data), _stream()), "fill")


def euler_stage(ctx, level, u_in, u_out, h, first_order=False, u_old=None, form=L.HF_FLUX_PLAIN, faces=False):
    """One Euler stage (BlockAMR.cpp:210-243) of a one-patch level; Heun combine with u_old.

    Returns (fx, fy) face fluxes when faces=True (plain form only)."""
    fx = fy = None
    if faces:
        nv, nx, ny = u_in.nv, u_in.nx, u_in.ny
        fx = torch.empty(nv, ny, nx + 1, dtype=torch.float64, device=u_in.data.device)
        fy = torch.empty(nv, ny + 1, nx, dtype=torch.float64, device=u_in.data.device)
    bad = ctypes.c_int64(-1)
    st = ctx.lib.hf_flux_update(ctx.h, ctypes.byref(level), ctypes.byref(u_in.patch), 1, _ptr(u_in.data),
                                _ptr(u_old.data) if u_old is not None else None, _ptr(u_out.data), _ptr(fx),
                                _ptr(fy), float(h), int(first_order), int(form), ctypes.byref(bad), _stream())
    ctx.check(st, "euler stage (bad cell %d)" % bad.value)
    return fx, fy


def flux_adjoint(ctx, level, u_in, ubar_out, h, first_order=False):
    """Adjoint of one Euler stage (hf_flux_adjoint): u_in holds the forward stage's input
    with its ghosts filled, ubar_out the cotangent of the stage output (same layout);
    returns a PatchArray holding J^T ubar_out on the interior cells."""
    out = u_in.like()
    ctx.check(ctx.lib.hf_flux_adjoint(ctx.h, ctypes.byref(level), ctypes.byref(u_in.patch), _ptr(u_in.data),
                                      _ptr(ubar_out.data), float(h), int(first_order), _ptr(out.data), _stream()),
              "flux_adjoint")
    return out


def cfl_dt(ctx, level, patch_array, cfl):
    """stableDt (BlockAMR.cpp:335-346)."""
    dt = ctypes.c_double(0.0)
    ctx.check(ctx.lib.hf_cfl_dt(ctx.h, ctypes.byref(level), ctypes.byref(patch_array.patch), 1,
                                _ptr(patch_array.data), float(cfl), ctypes.byref(dt), _stream()), "cfl_dt")
    return dt.value


def validate(ctx, level, patch_array):
    bad = ctypes.c_int64(-1)
    ctx.check(ctx.lib.hf_validate(ctx.h, ctypes.byref(level), ctypes.byref(patch_array.patch), 1,
                                  _ptr(patch_array.data), ctypes.byref(bad), _stream()), "validate")


class ConservativeInterp:
    """ConservativeInterp::interp (src/ConservativeInterp.cpp:18-51), ratio 2."""

    def __init__(self, ctx):
        self.ctx = ctx

    def interp(self, coarse, fine, region):
        """Fill fine cells of region (filo, fjlo, fihi, fjhi; fine level index) from coarse."""
        r = (ctypes.c_int32 * 4)(*[int(v) for v in region])
        self.ctx.check(self.ctx.lib.hf_interp_coarse_to_fine(self.ctx.h, ctypes.byref(coarse.patch),
                                                             _ptr(coarse.data), ctypes.byref(fine.patch),
                                                             _ptr(fine.data), r, _stream()), "interp")


# ------------------------------------------------------------------ chemistry
class ChemistryBatch:
    """ChemistryBatch (src/chemistry_batch.hpp): all-or-nothing advance of a batch of cells.

    form: "plain" (one thread per cell), "persistent" (device work queue; the same
    per-cell step sequence as plain), or "batched" (persistent queue plus frozen-cell
    screening, warm-started step sizes and a cost-ordered queue, using per-cell
    history kept by this object between calls)."""

    FORMS = {"plain": L.HF_CHEM_PLAIN, "persistent": L.HF_CHEM_PERSISTENT, "batched": -1}

    def __init__(self, ctx, form="batched", rtol=1e-8, atol=1e-15):
        self.ctx = ctx
        if form not in self.FORMS:
            raise ValueError("unknown chemistry form %r" % form)
        self.form = form
        self.rtol, self.atol = rtol, atol
        self.history = None

    def advance(self, field, dt, count=None, dt_cell=None, cell_index=None, comp_stride=None):
        """field: (NV, n) float64 CUDA tensor (SoA), advanced in place over dt.

        Raises RuntimeError("chemistry cell k: ...") on failure; field is unchanged then."""
        if cell_index is None:
            _need_state(self.ctx, field, "field")
        else:
            _need_cuda64(field, "field")
        if cell_index is None:
            if not field.is_contiguous():
                raise ValueError("field must be contiguous (NV, n)")
            n = field.shape[1] if count is None else int(count)
            if n > field.shape[1]:
                raise ValueError("invalid chemistry batch extent")
            cs = field.shape[1]
        else:
            n = cell_index.numel() if count is None else int(count)
            cs = int(comp_stride)
        if dt_cell is not None:
            _need_cuda64(dt_cell, "dt_cell")
        first = ctypes.c_int64(-1)
        if self.form == "batched":
            if self.history is None or self.history[0].numel() != n:
                self.history = (torch.zeros(n, dtype=torch.float64, device=field.device),
                                torch.zeros(n, dtype=torch.int32, device=field.device))
            hist = L.ChemHistory(self.history[0].data_ptr(), self.history[1].data_ptr())
            st = self.ctx.lib.hf_chem_advance_batched(self.ctx.h, _ptr(field), cs, _ptr(cell_index), n, float(dt),
                                                      _ptr(dt_cell), float(self.rtol), float(self.atol),
                                                      ctypes.byref(hist), ctypes.byref(first), _stream())
        else:
            st = self.ctx.lib.hf_chem_advance(self.ctx.h, _ptr(field), cs, _ptr(cell_index), n, float(dt),
                                              _ptr(dt_cell), float(self.rtol), float(self.atol),
                                              self.FORMS[self.form], ctypes.byref(first), _stream())
        if st in (L.HF_ERR_CHEM_FAIL, L.HF_ERR_MAXSTEPS):
            e = RuntimeError("chemistry cell %d: %s" % (first.value,
                                                        (self.ctx.lib.hf_last_error(self.ctx.h) or b"").decode()))
            e.first_failed = first.value
            e.status = st
            raise e
        self.ctx.check(st, "chemistry")
        return field


# ------------------------------------------------------------------ sensitivities
OBJECTIVES = {"ignition_delay": L.HF_OBJ_IGNITION_DELAY, "peak_pressure": L.HF_OBJ_PEAK_PRESSURE,
              "final_T": L.HF_OBJ_FINAL_T}


class ChemSensitivity:
    """0D constant-(rho, e) runs of `ncalls` chemistry calls of `dt` each and the
    discrete adjoint of their objective (hf_chem_objective / hf_chem_adjoint; an
    extension, the reference has no sensitivity code).

    objective: "ignition_delay" (time T first reaches T_0 + ignition_dT, linear in t
    between call boundaries; NaN if never), "peak_pressure" (max over boundaries) or
    "final_T".  Gradients are d J / d ln(multiplier_r) for the 21 reactions of H2_Li,
    the derivative of the run with its accepted step sequence frozen."""

    def __init__(self, ctx, dt, ncalls, objective="ignition_delay", ignition_dT=400.0, checkpoint_every=50,
                 rtol=1e-8, atol=1e-15):
        if objective not in OBJECTIVES:
            raise ValueError("unknown objective %r" % objective)
        self.ctx = ctx
        self.dt, self.ncalls = float(dt), int(ncalls)
        self.opts = L.AdjointOpts(OBJECTIVES[objective], int(checkpoint_every), float(ignition_dT), float(rtol),
                                  float(atol))

    def _fail(self, st, first):
        if st in (L.HF_ERR_CHEM_FAIL, L.HF_ERR_MAXSTEPS):
            e = RuntimeError("chemistry cell %d: %s" % (first.value,
                                                        (self.ctx.lib.hf_last_error(self.ctx.h) or b"").decode()))
            e.first_failed = first.value
            e.status = st
            raise e
        self.ctx.check(st, "chem_sensitivity")

    def objective(self, U0):
        """U0: (NV, n) float64 CUDA tensor (not modified) -> objective (n,)."""
        _need_cuda64(U0, "U0")
        U0 = U0.contiguous()
        n = U0.shape[1]
        J = torch.empty(n, dtype=torch.float64, device=U0.device)
        first = ctypes.c_int64(-1)
        st = self.ctx.lib.hf_chem_objective(self.ctx.h, _ptr(U0), n, n, self.dt, self.ncalls, ctypes.byref(self.opts),
                                            _ptr(J), ctypes.byref(first), _stream())
        self._fail(st, first)
        return J

    def adjoint(self, U0, initial=False):
        """-> (J (n,), dJ/d ln multiplier (21, n), dJ/dY0 (NS-1, n) or None)."""
        _need_cuda64(U0, "U0")
        U0 = U0.contiguous()
        n = U0.shape[1]
        J = torch.empty(n, dtype=torch.float64, device=U0.device)
        G = torch.empty(21, n, dtype=torch.float64, device=U0.device)
        G0 = torch.empty(U0.shape[0] - 4, n, dtype=torch.float64, device=U0.device) if initial else None
        first = ctypes.c_int64(-1)
        st = self.ctx.lib.hf_chem_adjoint(self.ctx.h, _ptr(U0), n, n, self.dt, self.ncalls, ctypes.byref(self.opts),
                                          _ptr(J), _ptr(G), _ptr(G0), ctypes.byref(first), _stream())
        self._fail(st, first)
        return J, G, G0


class ChemObjective(torch.autograd.Function):
    """J(ln multipliers) of a ChemSensitivity run, differentiable in the 21 log rate
    multipliers through the discrete adjoint:

        J = ChemObjective.apply(ln_mult, U0, sens);  J.sum().backward()

    ln_mult: (21,) float64 tensor.  Cells whose objective is NaN (no ignition)
    contribute nothing to the gradient.  The context's rate multipliers are reset to 1
    after each call."""

    @staticmethod
    def forward(fctx, ln_mult, U0, sens):
        sens.ctx.set_rate_scale(torch.exp(ln_mult.detach().double()).cpu().tolist())
        try:
            J = sens.objective(U0)
        finally:
            sens.ctx.set_rate_scale(None)
        fctx.sens = sens
        fctx.save_for_backward(ln_mult, U0)
        return J

    @staticmethod
    def backward(fctx, gJ):
        ln_mult, U0 = fctx.saved_tensors
        sens = fctx.sens
        sens.ctx.set_rate_scale(torch.exp(ln_mult.detach().double()).cpu().tolist())
        try:
            _, G, _ = sens.adjoint(U0)
        finally:
            sens.ctx.set_rate_scale(None)
        g = (torch.nan_to_num(G, nan=0.0) * torch.nan_to_num(gJ, nan=0.0)[None, :]).sum(1)
        return g.to(ln_mult.device, ln_mult.dtype), None, None


class FlowAdjoint:
    """A recorded run of Strang steps on a one-patch level and its discrete adjoint
    (hf_flow_record / hf_flow_adjoint; an extension, the reference has no sensitivity
    code).  The run uses the plain forms with the given step sizes (or CFL steps,
    recorded); `final` is its final state and `dts` its step sizes.

        fa = FlowAdjoint(ctx, level, U0, nsteps=1000, checkpoint_every=50)
        U0_bar, dJ_dlnA = fa.adjoint(seed)   # seed = dJ/dU_final, (NV, ny, nx) CUDA
    """

    def __init__(self, ctx, level, U0, nsteps, dts=None, cfl=0.5, checkpoint_every=50, chemistry=True, rtol=1e-8,
                 atol=1e-15):
        _need_state(ctx, U0, "U0")
        self.ctx = ctx
        U0 = U0.contiguous()
        self.shape = tuple(U0.shape)
        self.final = torch.empty_like(U0)
        self.dts = np.zeros(int(nsteps))
        d = None if dts is None else np.ascontiguousarray(dts, dtype=np.float64)
        h = ctypes.c_void_p()
        torch.cuda.synchronize()
        st = ctx.lib.hf_flow_record(ctx.h, ctypes.byref(level), _ptr(U0), int(nsteps),
                                    None if d is None else d.ctypes.data, float(cfl), int(checkpoint_every),
                                    int(bool(chemistry)), float(rtol), float(atol), _ptr(self.final),
                                    self.dts.ctypes.data, ctypes.byref(h), _stream())
        ctx.check(st, "flow_record")
        self.h = h

    def adjoint(self, seed):
        """seed: dJ/dU_final, (NV, ny, nx) float64 CUDA -> (dJ/dU0 tensor, dJ/d ln A (21,) numpy)."""
        _need_cuda64(seed, "seed")
        seed = seed.contiguous()
        U0b = torch.empty(self.shape, dtype=torch.float64, device=seed.device)
        g = np.zeros(21)
        self.ctx.check(self.ctx.lib.hf_flow_adjoint(self.h, _ptr(seed), _ptr(U0b), g.ctypes.data, _stream()),
                       "flow_adjoint")
        return U0b, g

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.hf_flow_tape_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def induction_length(U, dx, product=2, sharp=4):
    """Induction length of a right-running planar detonation from a state (NV, ny, nx)
    (torch or numpy, differentiable in torch): the distance between the shock and the
    reaction front, each located as the centroid of a sharpened jump,
        x_s = sum x_f w_f / sum w_f,  w_f = (rho_i - rho_{i+1})^sharp   (density drop
              at the leading shock),
        x_r = sum x_f v_f / sum v_f,  v_f = (Y_i - Y_{i+1})^sharp with Y the product
              (H2O, species index `product`) mass fraction,
    over the faces x_f = (i + 1) dx between cells i and i+1, rows averaged.  A
    build-defined objective: the reference defines no induction length."""
    xp = torch if isinstance(U, torch.Tensor) else np
    ns = U.shape[0] - 3
    rho = U[:ns].sum(0).mean(0)
    Y = (U[product] / U[:ns].sum(0)).mean(0)
    nx = rho.shape[0]
    xf = (xp.arange(1, nx, dtype=rho.dtype) if xp is np else torch.arange(1, nx, dtype=rho.dtype, device=rho.device))
    xf = xf * dx
    w = (rho[:-1] - rho[1:]) ** sharp
    v = (Y[:-1] - Y[1:]) ** sharp
    return (xf * w).sum() / w.sum() - (xf * v).sum() / v.sum()


# ------------------------------------------------------------------ stepper
class Stepper:
    """Strang-split reacting-Euler stepper on a uniform one-patch level.

    flux: "fused" or "plain"; chem: "batched" (work queue with per-cell history) or
    "plain" (one thread per cell).

    step(): flow(dt/2); react(dt); flow(dt/2) with rollback and dt halving
    (BlockAMR.cpp:409-419).  U0: (NV, ny, nx) float64 CUDA tensor."""

    def __init__(self, ctx, level, U0, chemistry=True, rtol=1e-8, atol=1e-15, flux="fused", chem="batched"):
        _need_state(ctx, U0, "U0")
        self.ctx = ctx
        self.level = level
        self.nv, self.ny, self.nx = U0.shape
        U0 = U0.contiguous()
        h = ctypes.c_void_p()
        ff = {"plain": L.HF_FLUX_PLAIN, "fused": L.HF_FLUX_FUSED}[flux]
        cf = {"plain": L.HF_CHEM_PLAIN, "batched": L.HF_CHEM_PERSISTENT, "persistent": L.HF_CHEM_PERSISTENT}[chem]
        torch.cuda.synchronize()
        ctx.check(ctx.lib.hf_stepper_create(ctx.h, ctypes.byref(level), _ptr(U0), int(bool(chemistry)), float(rtol),
                                            float(atol), ff, cf, ctypes.byref(h)), "stepper_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.hf_stepper_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt=0.0, cfl=0.5):
        d = ctypes.c_double(float(dt))
        self.ctx.check(self.ctx.lib.hf_stepper_step(self.h, float(cfl), ctypes.byref(d), _stream()), "step")
        return d.value

    def run(self, nsteps, cfl=0.5):
        """nsteps CFL steps with no host round trip between graph steps (hf_stepper_run);
        returns the steps completed.  Same results as nsteps calls of step()."""
        done = ctypes.c_int32(0)
        self.ctx.check(self.ctx.lib.hf_stepper_run(self.h, int(nsteps), float(cfl), ctypes.byref(done), _stream()),
                       "stepper_run")
        return done.value

    def state(self):
        out = torch.empty(self.nv, self.ny, self.nx, dtype=torch.float64, device="cuda")
        self.ctx.check(self.ctx.lib.hf_stepper_get(self.h, _ptr(out), _stream()), "stepper_get")
        return out

    def set_host(self, U):
        """Copy valid cells in from host memory (torch CPU tensor, (NV, ny, nx))."""
        self.ctx.check(self.ctx.lib.hf_stepper_set_host(self.h, ctypes.c_void_p(U.data_ptr()), _stream()), "set_host")

    def get_host(self, U):
        self.ctx.check(self.ctx.lib.hf_stepper_get_host(self.h, ctypes.c_void_p(U.data_ptr()), _stream()), "get_host")
        return U

    @property
    def time(self):
        return self.ctx.lib.hf_stepper_time(self.h)

    def cfl_dt(self, cfl=0.5):
        """stableDt of the current state (BlockAMR.cpp:335-346)."""
        d = ctypes.c_double(0.0)
        self.ctx.check(self.ctx.lib.hf_stepper_cfl_dt(self.h, float(cfl), ctypes.byref(d), _stream()), "cfl_dt")
        return d.value

    def set_graph(self, enable=True):
        """Use (default) or bypass the CUDA-graph path of step()."""
        self.ctx.lib.hf_stepper_set_graph(self.h, int(bool(enable)))

    def stats(self):
        """{"graph_steps": n, "host_steps": m}."""
        g, h = ctypes.c_int64(0), ctypes.c_int64(0)
        self.ctx.lib.hf_stepper_stats(self.h, ctypes.byref(g), ctypes.byref(h))
        return {"graph_steps": g.value, "host_steps": h.value}

    def graph_info(self):
        """{"last_flags": status flags of the last graph step, "capture_error": CUDA error
        of a failed capture (zeros: no fallback), "phase_flags": the last single graph
        step's flags at its start, after the first flow, after the chemistry, after the
        second flow}."""
        f, e, ph = ctypes.c_uint32(0), ctypes.c_int32(0), (ctypes.c_uint32 * 4)()
        self.ctx.lib.hf_stepper_graph_info(self.h, ctypes.byref(f), ctypes.byref(e), ph)
        return {"last_flags": f.value, "capture_error": e.value, "phase_flags": list(ph)}


# ------------------------------------------------------------------ block-AMR level operations
class PatchSet:
    """The patches (boxes) of one level in one float64 CUDA buffer, each with ng ghost
    layers; boxes are (ilo, jlo, ihi, jhi) inclusive, in the level's index space."""

    def __init__(self, nv, boxes, ng=2, device="cuda"):
        self.nv, self.ng, self.boxes = nv, ng, [tuple(int(v) for v in b) for b in boxes]
        arr = (L.Patch * len(self.boxes))()
        off = 0
        for k, (i0, j0, i1, j1) in enumerate(self.boxes):
            p = arr[k]
            p.ilo, p.jlo, p.nx, p.ny, p.ng = i0, j0, i1 - i0 + 1, j1 - j0 + 1, ng
            p.pitch = (p.nx + 2 * ng + 1) // 2 * 2
            p.comp_stride = p.pitch * (p.ny + 2 * ng)
            p.offset = off
            off += nv * p.comp_stride
        self.patches = arr
        self.data = torch.zeros(off, dtype=torch.float64, device=device)

    def __len__(self):
        return len(self.boxes)

    def view(self, k):
        """(NV, ny+2ng, pitch) view of patch k."""
        p = self.patches[k]
        return self.data[p.offset:p.offset + self.nv * p.comp_stride].view(self.nv, p.ny + 2 * self.ng, p.pitch)

    def interior(self, k):
        p, g = self.patches[k], self.ng
        return self.view(k)[:, g:g + p.ny, g:g + p.nx]

    def cells(self):
        return sum(p.nx * p.ny for p in self.patches)


def totals(ctx, pset, cell_volume, leaf_mask=None, absolute=False):
    """BlockAMR::totals over the valid cells (leaf_mask: uint8 CUDA tensor packing the
    patches' cells in order, or None)."""
    out = (ctypes.c_double * pset.nv)()
    ctx.check(ctx.lib.hf_totals(ctx.h, pset.patches, len(pset), _ptr(pset.data), _ptr(leaf_mask), float(cell_volume),
                                int(bool(absolute)), out, _stream()), "totals")
    return [out[n] for n in range(pset.nv)]


def repair_roundoff(ctx, parts):
    """BlockAMR::repairRoundoff (BlockAMR.cpp:299-334) in place over the leaf cells of one
    or more levels.  parts: [(level, PatchSet or PatchArray, leaf mask or None), ...],
    coarsest level first; a leaf mask is a uint8 CUDA tensor over the patches' cells packed
    in order, row-major (None: every cell is a leaf).  Returns the number of values set to
    zero; raises DomainError (HF_ERR_NEGATIVE) when a value is materially negative or a
    donor holds too little mass."""
    n = len(parts)
    levels = (L.Level * n)()
    pp = (ctypes.POINTER(L.Patch) * n)()
    npatch = (ctypes.c_int * n)()
    U = (ctypes.c_void_p * n)()
    leaf = (ctypes.c_void_p * n)()
    keep = []
    for k, (lv, ps, mask) in enumerate(parts):
        levels[k] = lv
        if isinstance(ps, PatchArray):
            arr = (L.Patch * 1)(ps.patch)
            keep.append(arr)
            pp[k] = ctypes.cast(arr, ctypes.POINTER(L.Patch))
            npatch[k] = 1
        else:
            pp[k] = ctypes.cast(ps.patches, ctypes.POINTER(L.Patch))
            npatch[k] = len(ps)
        U[k] = _ptr(ps.data)
        leaf[k] = _ptr(mask)
    rep = ctypes.c_int64(0)
    ctx.check(ctx.lib.hf_repair_roundoff(ctx.h, n, levels, pp, npatch, U, leaf, ctypes.byref(rep), _stream()),
              "repair_roundoff")
    return rep.value


def average_down(ctx, fine, coarse):
    """Every coarse cell under a fine patch becomes the mean of its four children."""
    ctx.check(ctx.lib.hf_average_down(ctx.h, fine.patches, len(fine), _ptr(fine.data), coarse.patches, len(coarse),
                                      _ptr(coarse.data), _stream()), "average_down")


def reflux(ctx, coarse_level, coarse, fxc, fyc, fine, fxf, fyf, h):
    """FluxRegister reflux of the coarse cells next to the fine patches (face fluxes
    packed per patch as hf_flux_update writes them)."""
    ctx.check(ctx.lib.hf_reflux(ctx.h, ctypes.byref(coarse_level), coarse.patches, len(coarse), _ptr(coarse.data),
                                _ptr(fxc), _ptr(fyc), fine.patches, len(fine), _ptr(fxf), _ptr(fyf), float(h),
                                _stream()), "reflux")


def tag_criteria(pressure_tag=0.08, temperature_tag=0.08, fuel_rate_tag=50.0, density_tag=0.0, chemistry=True,
                 box=None, box_only=False, velocity=(0.0, 0.0)):
    """hf_tag_criteria from the reference's case keys (BlockAMR.cpp:170-200 defaults)."""
    c = L.TagCriteria()
    c.pressure_tag, c.temperature_tag, c.fuel_rate_tag, c.density_tag = (pressure_tag, temperature_tag,
                                                                         fuel_rate_tag, density_tag)
    c.chemistry, c.box_only, c.has_box = int(bool(chemistry)), int(bool(box_only)), int(box is not None)
    if box is not None:
        for k in range(4):
            c.box[k] = float(box[k])
    c.velocity[0], c.velocity[1] = float(velocity[0]), float(velocity[1])
    return c


def tag_cells(ctx, level, pset, time, pressure_tag=0.08, temperature_tag=0.08, fuel_rate_tag=50.0, density_tag=0.0,
              chemistry=True, box=None, box_only=False, velocity=(0.0, 0.0)):
    """ErrorEst (BlockAMR.cpp:170-200) tags of the valid cells (ghost layers filled)."""
    c = tag_criteria(pressure_tag, temperature_tag, fuel_rate_tag, density_tag, chemistry, box, box_only, velocity)
    tags = torch.zeros(pset.cells(), dtype=torch.uint8, device=pset.data.device)
    ctx.check(ctx.lib.hf_tag_cells(ctx.h, ctypes.byref(level), pset.patches, len(pset), _ptr(pset.data),
                                   float(time), ctypes.byref(c), _ptr(tags), _stream()), "tag_cells")
    return tags


# ------------------------------------------------------------------ multi-level block AMR
class AmrStepper:
    """BlockAMR::run on levels 0..max_level (hf_amr_*): dense level arrays with active
    blocks of `block` cells, no time subcycling, regrid every `regrid_interval` steps.

    level: the base level (make_level); U0: (NV, ny, nx) float64 CUDA tensor; tags: keyword
    arguments of tag_criteria (ErrorEst keys, density_tag extension); U_levels: the initial
    state of levels 1, 2, ... ((NV, ny_l, nx_l) CUDA tensors or None), which the initial
    hierarchy takes for its new blocks instead of interpolating (hf_amr_create_levels)."""

    def __init__(self, ctx, level, U0, max_level=1, block=32, tag_buffer=2, regrid_interval=0, chemistry=True,
                 chem="batched", rtol=1e-8, atol=1e-15, tags=None, U_levels=None):
        _need_state(ctx, U0, "U0")
        self.ctx = ctx
        o = L.AmrOpts()
        o.max_level, o.block, o.tag_buffer, o.regrid_interval = int(max_level), int(block), int(tag_buffer), int(
            regrid_interval)
        o.chemistry = int(bool(chemistry))
        o.chem_form = {"plain": L.HF_CHEM_PLAIN, "batched": L.HF_CHEM_PERSISTENT}[chem]
        o.rtol, o.atol = float(rtol), float(atol)
        o.tags = tag_criteria(chemistry=chemistry, **(tags or {}))
        self.opts = o
        self.nv = U0.shape[0]
        h = ctypes.c_void_p()
        torch.cuda.synchronize()
        if U_levels:
            keep = [U0.contiguous()] + [None if u is None else u.contiguous() for u in U_levels]
            for lev, u in enumerate(keep[1:], 1):
                if u is not None:
                    _need_state(ctx, u, "U_levels")
                    if tuple(u.shape[1:]) != (level.ny << lev, level.nx << lev):
                        raise ValueError("U_levels[%d] must cover level %d" % (lev - 1, lev))
            ptrs = (ctypes.c_void_p * len(keep))(*[None if u is None else u.data_ptr() for u in keep])
            ctx.check(ctx.lib.hf_amr_create_levels(ctx.h, ctypes.byref(level), ptrs, len(keep), ctypes.byref(o),
                                                   ctypes.byref(h), _stream()), "amr_create_levels")
            torch.cuda.synchronize()
        else:
            ctx.check(ctx.lib.hf_amr_create(ctx.h, ctypes.byref(level), _ptr(U0.contiguous()), ctypes.byref(o),
                                            ctypes.byref(h), _stream()), "amr_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.hf_amr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt=0.0, cfl=0.5):
        d = ctypes.c_double(float(dt))
        self.ctx.check(self.ctx.lib.hf_amr_step(self.h, float(cfl), ctypes.byref(d), _stream()), "amr_step")
        return d.value

    def regrid(self):
        self.ctx.check(self.ctx.lib.hf_amr_regrid(self.h, _stream()), "amr_regrid")

    def info(self, lev):
        v = [ctypes.c_int32() for _ in range(5)]
        leaf = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.hf_amr_info(self.h, int(lev), *[ctypes.byref(x) for x in v], ctypes.byref(leaf)),
                       "amr_info")
        return {"nx": v[0].value, "ny": v[1].value, "nbx": v[2].value, "nby": v[3].value, "finest": v[4].value,
                "leaf_cells": leaf.value}

    def level(self, lev):
        """(state (NV, ny_l, nx_l) CUDA tensor, block activity (nby, nbx) numpy uint8)."""
        i = self.info(lev)
        U = torch.empty(self.nv, i["ny"], i["nx"], dtype=torch.float64, device="cuda")
        act = np.zeros((i["nby"], i["nbx"]), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.hf_amr_get_level(self.h, int(lev), _ptr(U), act.ctypes.data, _stream()),
                       "amr_get_level")
        return U, act

    def totals(self):
        out = np.zeros(self.nv)
        self.ctx.check(self.ctx.lib.hf_amr_totals(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                  _stream()), "amr_totals")
        return out

    def cfl_dt(self, cfl=0.5):
        """stableDt over the active cells of every level (BlockAMR.cpp:335-346), the step
        hf_amr_step takes when given dt <= 0 on its host-driven path."""
        d = ctypes.c_double(0.0)
        self.ctx.check(self.ctx.lib.hf_amr_cfl_dt(self.h, float(cfl), ctypes.byref(d), _stream()), "amr_cfl_dt")
        return d.value

    @property
    def time(self):
        return self.ctx.lib.hf_amr_time(self.h)

    def set_graph(self, enable=True):
        """Graph-captured steps (default) or the host-driven path only."""
        self.ctx.lib.hf_amr_set_graph(self.h, int(bool(enable)))

    def stats(self):
        """{"graph_steps": n, "host_steps": m}."""
        g, h = ctypes.c_int64(0), ctypes.c_int64(0)
        self.ctx.lib.hf_amr_stats(self.h, ctypes.byref(g), ctypes.byref(h))
        return {"graph_steps": g.value, "host_steps": h.value}
