"""CPU oracle of the block-AMR composite Strang step.  TEST INFRASTRUCTURE ONLY: tests
import it; the GPU package never does.

A restatement, with the oracle's per-cell functions, of the multi-level stepper's
algorithm at refinement ratio 2 without time subcycling (HyperFlow_V3/src/BlockAMR.cpp:
euler :202-264, flow :266-270, react :271-285, regrid :367-373 with ErrorEst :170-200),
on levels 0..max_level of a domain with the reference's boundary conditions.
- Level l is a dense ghosted array over the whole domain refined 2^l times; level 0 is
  always fully active, level l >= 1 is active in aligned blocks of `block` cells.
- Ghosts: every level by the physical/periodic fill of its whole array, then, in each
  active block's 2-cell frame part that lies in an inactive block of the same level
  (across a periodic edge: the inactive periodic image; outside a non-periodic edge:
  none, the physical ghosts stay), ConservativeInterp from level l-1
  (src/ConservativeInterp.cpp:18-51, oracle.interp_cell).
- Euler stage: level 0 as one box, level l >= 1 block by block (a block face is a wall
  face only where it lies on a reflecting or wedge domain edge), then from the finest
  level down: reflux of level l-1 from level l's face fluxes (FluxRegister, :245-256)
  and average_down (:256), then repairRoundoff over the leaf cells of every level
  (:299-334: species below zero by at most 64 ulp of their peak zeroed, the deficit
  taken from the cell holding the most mass), average_down again if a value was
  repaired, and validation of every level; a stage that fails the repair or the
  validation is redone first order on every level (:258-263).
- flow(h): two stages, Heun combination, average_down, validation.
- step(dt): flow(dt/2), react(dt), flow(dt/2); a failed attempt is rolled back and
  retried with half the step (:411-419).
- react(dt): the leaf cells of every level through the oracle's ChemistryBatch, then
  average_down.
- regrid (every regrid_interval steps, and max_level times to build the initial
  hierarchy from the base level alone), level by level from 0: ErrorEst tags of level
  l's active cells; a level-(l+1) block is active when a tagged cell lies in its level-l
  footprint grown by tag_buffer cells and the footprint grown by 2 cells lies in active
  level-l cells (proper nesting); both wrap across periodic edges and are cut at the
  others.  Blocks that become active are filled by ConservativeInterp from level l;
  blocks that stay keep their data.  As regridChecked (:367-373) the hierarchy is
  averaged down before and after the remap and validated after it, and the leaf totals
  must survive the remap to 1e-8 of the total of the magnitudes.  The block
  rule is the GPU stepper's deterministic choice in place of AMReX's clustering.
States are AoS arrays (..., NS+3); levels are dense ghosted arrays (ny+4, nx+4, NV).
"""
import numpy as np

import oracle

BC = {"reflecting": 0, "transmissive": 1, "inflow": 2, "wedge": 3}


def criteria(pressure_tag=0.08, temperature_tag=0.08, fuel_rate_tag=50.0, density_tag=0.0, chemistry=True,
             box=None, box_only=False, velocity=(0.0, 0.0)):
    """ErrorEst criteria from the reference's case keys (BlockAMR.cpp:170-200 defaults)."""
    c = oracle.TagCriteria()
    c.pressure_tag, c.temperature_tag, c.fuel_rate_tag, c.density_tag = (pressure_tag, temperature_tag,
                                                                         fuel_rate_tag, density_tag)
    c.chemistry, c.box_only, c.has_box = int(bool(chemistry)), int(bool(box_only)), int(box is not None)
    if box is not None:
        for k in range(4):
            c.box[k] = float(box[k])
    c.velocity[0], c.velocity[1] = float(velocity[0]), float(velocity[1])
    return c


class StepFailure(RuntimeError):
    """A failure that BlockAMR::run answers with a rollback and a halved dt
    (BlockAMR.cpp:413-418): an inadmissible face or cell, a failed chemistry cell."""


def _wrap(n, count, periodic):
    """Index n along a direction of `count`: wrapped when periodic, -1 outside."""
    if 0 <= n < count:
        return n
    return n % count if periodic else -1


class Hierarchy:
    def __init__(self, Us, actives, domain, block, chemistry=True, rtol=1e-8, atol=1e-15, crit=None,
                 tag_buffer=1, regrid_interval=0, max_level=None):
        """Us[l]: (ny_l, nx_l, NV) state of level l (read in its active blocks); actives[l]:
        (nby_l, nbx_l) uint8 for l >= 1 (actives[0] is ignored: level 0 is all active);
        domain: the base level's keys (nx, ny, dx, dy, xlo, ylo, periodic, boundary_lo,
        boundary_hi, inlet, wedge_start); crit: criteria(...) for regrids."""
        d = dict(xlo=0.0, ylo=0.0, periodic=(1, 1), boundary_lo=("reflecting", "reflecting"),
                 boundary_hi=("transmissive", "reflecting"), inlet=None, wedge_start=0.0)
        d.update(domain)
        self.d = d
        nx, ny = d["nx"], d["ny"]
        self.nv, self.B = Us[0].shape[2], block
        self.max_level = len(Us) - 1 if max_level is None else max_level
        L = self.max_level + 1
        if block % 2 or (L > 1 and (nx % (block // 2) or ny % (block // 2))):
            raise ValueError("blocks must tile the refined levels")
        self.px, self.py = int(d["periodic"][0]), int(d["periodic"][1])
        self.inlet = np.zeros(self.nv) if d["inlet"] is None else np.asarray(d["inlet"], dtype=np.float64)
        self.shape = [(ny << l, nx << l) for l in range(L)]
        self.dxs = [(d["dx"] / (1 << l), d["dy"] / (1 << l)) for l in range(L)]
        self.g = [self._grid(l, 0, 0, *self.shape[l][::-1]) for l in range(L)]
        self.nb = [((self.shape[l][0] + block - 1) // block, (self.shape[l][1] + block - 1) // block)
                   for l in range(L)]
        self.X = []
        self.acts = [np.ones(self.nb[0], np.uint8)]
        for l in range(L):
            U = np.zeros(self.shape[l] + (self.nv,)) if l >= len(Us) else np.asarray(Us[l], dtype=np.float64)
            if U.shape != self.shape[l] + (self.nv,):
                raise ValueError("level %d has shape %s, expected %s" % (l, U.shape, self.shape[l]))
            self.X.append(oracle.ghosted(U))
            if l:
                a = actives[l] if l < len(actives) and actives[l] is not None else np.zeros(self.nb[l], np.uint8)
                self.acts.append(np.asarray(a, dtype=np.uint8).copy())
        self.finest = 0
        for l in range(1, L):
            if self.acts[l].any():
                self.finest = l
        self.chemistry, self.rtol, self.atol = chemistry, rtol, atol
        self.crit, self.buf, self.interval = crit, tag_buffer, regrid_interval
        self.time, self.steps, self.regrids, self.retries = 0.0, 0, 0, 0
        self._init = []
        self.first_order_stages, self.roundoff_repairs = 0, 0
        self._rebuild()
        self.X = self.average_all(self.X)

    @classmethod
    def from_base(cls, U0, domain, block, crit, max_level=1, tag_buffer=1, regrid_interval=0, levels=None, **kw):
        """The hierarchy the GPU stepper builds from the base level (hf_amr_create): level
        0 = U0, then one regrid per level.  levels: the initial state of levels 1, 2, ...
        ((ny_l, nx_l, NV) or None; hf_amr_create_levels): a new block takes it instead of
        the interpolation, the remap check is skipped, and the levels are then averaged
        down and validated (MakeNewLevelFromScratch, BlockAMR.cpp:124-131; run(), :401)."""
        o = cls([U0], [None], domain, block, crit=crit, tag_buffer=tag_buffer, regrid_interval=regrid_interval,
                max_level=max_level, **kw)
        o._init = [None] + list(levels) if levels else []
        for _ in range(max_level):
            o.regrid()
        if levels:
            o.X = o.average_all(o.X)
            o._check(o.X, "the initial hierarchy")
        o._init = []
        o.regrids = 0
        return o

    # ------------------------------------------------------------ geometry
    def _grid(self, l, i0, j0, nx, ny):
        """Grid of level l's box of nx x ny cells from cell (i0, j0): the domain's
        conditions on the sides that lie on a non-periodic domain edge, transmissive
        (no wall face) elsewhere."""
        d, (NY, NX) = self.d, self.shape[l]
        lo = [BC[d["boundary_lo"][0]], BC[d["boundary_lo"][1]]]
        hi = [BC[d["boundary_hi"][0]], BC[d["boundary_hi"][1]]]
        whole = (i0, j0, nx, ny) == (0, 0, NX, NY)
        if not whole:
            lo[0] = lo[0] if i0 == 0 and not self.px else BC["transmissive"]
            hi[0] = hi[0] if i0 + nx == NX and not self.px else BC["transmissive"]
            lo[1] = lo[1] if j0 == 0 and not self.py else BC["transmissive"]
            hi[1] = hi[1] if j0 + ny == NY and not self.py else BC["transmissive"]
        dx, dy = self.dxs[l]
        return oracle.make_grid(nx, ny, dx, dy, xlo=d["xlo"] + i0 * dx, ylo=d["ylo"] + j0 * dy,
                                periodic=(self.px, self.py) if whole else (0, 0), bc_lo=tuple(lo), bc_hi=tuple(hi),
                                inlet=self.inlet, wedge_start=d["wedge_start"])

    def blocks(self, l):
        """Active blocks (bi, bj) of level l >= 1, row-major."""
        nby, nbx = self.nb[l]
        return [(bi, bj) for bj in range(nby) for bi in range(nbx) if self.acts[l][bj, bi]]

    def _rebuild(self):
        self.regions = [[] for _ in range(self.max_level + 1)]
        B = self.B
        for l in range(1, self.finest + 1):
            nby, nbx = self.nb[l]
            for bi, bj in self.blocks(l):
                ilo, jlo = bi * B, bj * B
                for dj in (-1, 0, 1):
                    for di in (-1, 0, 1):
                        if not di and not dj:
                            continue
                        nbi, nbj = _wrap(bi + di, nbx, self.px), _wrap(bj + dj, nby, self.py)
                        if nbi < 0 or nbj < 0 or self.acts[l][nbj, nbi]:
                            continue
                        i0 = ilo - 2 if di < 0 else (ilo + B if di > 0 else ilo)
                        i1 = ilo - 1 if di < 0 else (ilo + B + 1 if di > 0 else ilo + B - 1)
                        j0 = jlo - 2 if dj < 0 else (jlo + B if dj > 0 else jlo)
                        j1 = jlo - 1 if dj < 0 else (jlo + B + 1 if dj > 0 else jlo + B - 1)
                        self.regions[l].append((i0, j0, i1, j1))

    def leaf_mask(self, l):
        """(ny_l, nx_l) True at the leaf cells of level l."""
        ny, nx = self.shape[l]
        B, h = self.B, self.B // 2
        m = np.ones((ny, nx), bool) if l == 0 else np.kron(self.acts[l], np.ones((B, B), np.uint8)).astype(bool)[
            :ny, :nx]
        if l < self.finest:
            m &= ~np.kron(self.acts[l + 1], np.ones((h, h), np.uint8)).astype(bool)[:ny, :nx]
        return m

    # ------------------------------------------------------------ hierarchy operations
    def _interp(self, f, c, fj, fi):
        """ConservativeInterp child of fine cell (fi, fj) from the ghosted coarse array c."""
        ci, cj = fi >> 1, fj >> 1
        kids, _ = oracle.interp_cell(c[cj + 2, ci + 2], c[cj + 2, ci + 1], c[cj + 2, ci + 3], c[cj + 1, ci + 2],
                                     c[cj + 3, ci + 2])
        f[fj + 2, fi + 2] = kids[(fj & 1) * 2 + (fi & 1)]

    def fill(self, X):
        """Ghosts of every level (coarse levels first)."""
        for l in range(self.finest + 1):
            X[l] = oracle.fill_ghosts(self.g[l], X[l])
            for i0, j0, i1, j1 in self.regions[l]:
                for fj in range(j0, j1 + 1):
                    for fi in range(i0, i1 + 1):
                        self._interp(X[l], X[l - 1], fj, fi)
        return X

    def _averaged(self, l, fine, coarse):
        """coarse with every active level-l block's footprint replaced by the average of
        its children."""
        out = coarse.copy()
        B, h = self.B, self.B // 2
        for bi, bj in self.blocks(l):
            avg = oracle.average_down(fine[2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B])
            out[2 + bj * h:2 + (bj + 1) * h, 2 + bi * h:2 + (bi + 1) * h] = avg
        return out

    def average_all(self, X):
        X = list(X)
        for l in range(self.finest, 0, -1):
            X[l - 1] = self._averaged(l, X[l], X[l - 1])
        return X

    def _active_cells(self, X, l):
        cells = X[l][2:-2, 2:-2]
        if l == 0:
            return cells.reshape(-1, self.nv)
        B = self.B
        return np.concatenate([cells[bj * B:(bj + 1) * B, bi * B:(bi + 1) * B].reshape(-1, self.nv)
                               for bi, bj in self.blocks(l)])

    def _check(self, X, what):
        for l in range(self.finest + 1):
            if np.any(oracle.properties(self._active_cells(X, l))[3]):
                raise StepFailure("inadmissible level-%d cell after %s" % (l, what))

    def _stages(self, Xin, h, first_order):
        """Every level's Euler update from the filled Xin: (out, whole-level face fluxes,
        per-block fine fluxes).  No cell check here: the reference checks the composite
        state after reflux and average_down."""
        out = [x.copy() for x in Xin]
        B = self.B
        FX, FY, fine = [], [], []
        for l in range(self.finest + 1):
            ny, nx = self.shape[l]
            if l == 0:
                o, fx, fy, st = oracle.euler_stage(self.g[0], Xin[0], h, first_order)
                if st:
                    raise StepFailure("level-0 face inadmissible")
                out[0][2:-2, 2:-2] = o[2:-2, 2:-2]
                FX.append(fx)
                FY.append(fy)
                fine.append(None)
                continue
            fxa, fya = np.zeros((ny, nx + 1, self.nv)), np.zeros((ny + 1, nx, self.nv))
            boxes, fxl, fyl = [], [], []
            for bi, bj in self.blocks(l):
                i0, j0 = bi * B, bj * B
                o, fx, fy, st = oracle.euler_stage(self._grid(l, i0, j0, B, B), Xin[l][j0:j0 + B + 4, i0:i0 + B + 4], h,
                                                   first_order)
                if st:
                    raise StepFailure("level-%d face inadmissible" % l)
                out[l][j0 + 2:j0 + 2 + B, i0 + 2:i0 + 2 + B] = o[2:-2, 2:-2]
                fxa[j0:j0 + B, i0:i0 + B + 1] = fx
                fya[j0:j0 + B + 1, i0:i0 + B] = fy
                boxes.append((i0, j0, i0 + B - 1, j0 + B - 1))
                fxl.append(fx)
                fyl.append(fy)
            FX.append(fxa)
            FY.append(fya)
            fine.append((boxes, fxl, fyl))
        return out, FX, FY, fine

    def _patches(self, l):
        """The GPU stepper's patches of level l in table order, as (j0, i0, ny, nx): the
        whole level when every block is active (level 0 always), else the active blocks
        in row-major block order."""
        ny, nx = self.shape[l]
        if l == 0 or self.acts[l].all():
            return [(0, 0, ny, nx)]
        B = self.B
        return [(bj * B, bi * B, B, B) for bi, bj in self.blocks(l)]

    def repair(self, X):
        """repairRoundoff (BlockAMR.cpp:299-334) over the leaf cells of every level, cells
        taken in the order levels, patches (`_patches`), rows: per species the peak partial
        density and the donor (the first cell holding the largest mass, value x volume)
        over all leaf cells; a value below zero by more than 64 ulp of the peak, or not
        finite, is material; smaller ones are zeroed and their deficits (-value x volume)
        added in cell order and taken from the donor, which must hold more mass than the
        deficit.  X is repaired in place.  Returns (ok, number of zeroed values)."""
        ns, eps = self.nv - 3, np.finfo(np.float64).eps
        locs, vols = [], []
        for l in range(self.finest + 1):
            leaf = self.leaf_mask(l)
            vol = self.dxs[l][0] * self.dxs[l][1]
            for j0, i0, pny, pnx in self._patches(l):
                jj, ii = np.mgrid[j0:j0 + pny, i0:i0 + pnx]
                jj, ii = jj.reshape(-1), ii.reshape(-1)
                keep = leaf[jj, ii]
                locs.append((l, jj[keep], ii[keep]))
                vols.append(np.full(int(keep.sum()), vol))
        v = np.concatenate([X[l][jj + 2, ii + 2, :ns] for l, jj, ii in locs])
        vol = np.concatenate(vols)
        neg = ~(v >= 0)
        if not neg.any():
            return True, 0
        peak = np.where(v > 0, v, 0.0).max(0)
        mass = np.where(v > 0, v * vol[:, None], 0.0)
        if np.any(neg & (~np.isfinite(v) | (-v > 64 * eps * peak))):
            return False, 0
        count = 0
        for n in range(ns):
            k = np.nonzero(neg[:, n])[0]
            if not len(k):
                continue
            d = 0.0
            for kk in k:
                d += float(-v[kk, n] * vol[kk])
            v[k, n] = 0.0
            count += len(k)
            if not d > 0:
                continue
            donor = int(np.argmax(mass[:, n]))
            if not mass[donor, n] > d:
                return False, count
            v[donor, n] -= d / vol[donor]
        k = 0
        for l, jj, ii in locs:
            X[l][jj + 2, ii + 2, :ns] = v[k:k + len(jj)]
            k += len(jj)
        self.roundoff_repairs += count
        return True, count

    def _valid(self, X):
        return not any(np.any(oracle.properties(self._active_cells(X, l))[3]) for l in range(self.finest + 1))

    def euler(self, Xin, h):
        """One composite stage (BlockAMR::euler, :202-264): every level's update, then from
        the finest level down reflux and average_down, then repairRoundoff over the leaf
        cells of every level, average_down again when a value was repaired, and validation
        of every level; when the repair or the validation fails the whole stage is redone
        first order (:258-263), and a failing first-order stage fails the step."""
        Xin = self.fill([x.copy() for x in Xin])
        for first_order in (False, True):
            out, FX, FY, fine = self._stages(Xin, h, first_order)
            for l in range(self.finest, 0, -1):
                boxes, fxl, fyl = fine[l]
                dx, dy = self.dxs[l - 1]
                out[l - 1][2:-2, 2:-2] = oracle.reflux(out[l - 1][2:-2, 2:-2], FX[l - 1], FY[l - 1], boxes, fxl, fyl, h,
                                                       dx, dy, periodic=(self.px, self.py))
                out[l - 1] = self._averaged(l, out[l], out[l - 1])
            ok, repaired = self.repair(out)
            if ok and repaired:
                out = self.average_all(out)
            if ok and self._valid(out):
                if first_order:
                    self.first_order_stages += 1
                return out
        raise StepFailure("inadmissible cell after a first-order stage")

    def flow(self, h):
        U = self.X
        S = self.euler(U, h)
        N = self.euler(S, h)
        for l in range(len(N)):
            N[l] = 0.5 * U[l] + 0.5 * N[l]
        N = self.average_all(N)
        self._check(N, "the Heun combination")
        self.X = N

    def react(self, dt):
        if not self.chemistry:
            return
        masks = [self.leaf_mask(l) for l in range(self.finest + 1)]
        batch = np.concatenate([self.X[l][2:-2, 2:-2][masks[l]] for l in range(self.finest + 1)])
        out, bad, _ = oracle.chem_batch(batch, dt, rtol=self.rtol, atol=self.atol)
        if bad >= 0:
            raise StepFailure("chemistry cell %d failed" % bad)
        k = 0
        for l in range(self.finest + 1):
            n = int(masks[l].sum())
            self.X[l][2:-2, 2:-2][masks[l]] = out[k:k + n]
            k += n
        self.X = self.average_all(self.X)
        self._check(self.X, "react")

    def step(self, dt):
        """One Strang step of every level; a failed attempt is rolled back and retried with
        half the step, at most 18 attempts (BlockAMR.cpp:411-419).  Returns the step taken."""
        backup = [x.copy() for x in self.X]
        h = dt
        for _ in range(18):
            try:
                self.flow(0.5 * h)
                self.react(h)
                self.flow(0.5 * h)
                break
            except StepFailure:
                self.X = [x.copy() for x in backup]
                self.retries += 1
                h *= 0.5
        else:
            raise RuntimeError("time advancement failed")
        self.time += h
        self.steps += 1
        if self.interval > 0 and self.steps % self.interval == 0:
            self.regrid()
        return h

    # ------------------------------------------------------------ regrid
    def _regrid_level(self, l):
        B, h, buf = self.B, self.B // 2, self.buf
        self.X = self.fill(self.X)
        c = self.X[l]
        ny, nx = self.shape[l]
        # ErrorEst on the active cells of level l (level 0 as one box, blocks one by one)
        if l == 0:
            tags, st = oracle.tag(self.g[0], c, self.time, self.crit)
            if st:
                raise RuntimeError("ErrorEst: inadmissible level-0 cell")
            tags = tags.astype(bool)
        else:
            tags = np.zeros((ny, nx), bool)
            for bi, bj in self.blocks(l):
                i0, j0 = bi * B, bj * B
                t, st = oracle.tag(self._grid(l, i0, j0, B, B), c[j0:j0 + B + 4, i0:i0 + B + 4], self.time, self.crit)
                if st:
                    raise RuntimeError("ErrorEst: inadmissible level-%d cell" % l)
                tags[j0:j0 + B, i0:i0 + B] = t.astype(bool)
        act = np.ones((ny, nx), bool) if l == 0 else np.kron(self.acts[l], np.ones((B, B), np.uint8)).astype(bool)[
            :ny, :nx]
        nby, nbx = self.nb[l + 1]

        def cells(lo, n, count, periodic):
            idx = [_wrap(k, count, periodic) for k in range(lo, lo + n)]
            return np.array([k for k in idx if k >= 0], dtype=np.int64)

        nxt = np.zeros((nby, nbx), np.uint8)
        for bj in range(nby):
            for bi in range(nbx):
                i0, j0 = bi * h, bj * h
                iw, jw = min(i0 + h, nx) - i0, min(j0 + h, ny) - j0
                rows, cols = cells(j0 - buf, jw + 2 * buf, ny, self.py), cells(i0 - buf, iw + 2 * buf, nx, self.px)
                if not tags[np.ix_(rows, cols)].any():
                    continue
                rows, cols = cells(j0 - 2, jw + 4, ny, self.py), cells(i0 - 2, iw + 4, nx, self.px)
                nxt[bj, bi] = 1 if act[np.ix_(rows, cols)].all() else 0
        prev, had = self.acts[l + 1], self.finest >= l + 1
        self.acts[l + 1] = nxt
        anyb = bool(nxt.any())
        self.finest = max(self.finest, l + 1) if anyb else l
        f = self.X[l + 1]
        init = self._init[l + 1] if l + 1 < len(self._init) else None
        for bj, bi in zip(*np.nonzero(nxt)):
            if had and prev[bj, bi]:
                continue
            if init is not None:
                f[2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B] = init[bj * B:(bj + 1) * B,
                                                                               bi * B:(bi + 1) * B]
                continue
            for fj in range(bj * B, (bj + 1) * B):
                for fi in range(bi * B, (bi + 1) * B):
                    self._interp(f, c, fj, fi)
        if not anyb:
            for q in range(l + 2, self.max_level + 1):
                self.acts[q][:] = 0
        self._rebuild()

    def regrid(self):
        """regridChecked (BlockAMR.cpp:367-373): average_down, the totals, the remap level by
        level, average_down, validation, and the totals again, which must agree to 1e-8 of
        the total of the magnitudes (not checked while the hierarchy is built from given
        level states)."""
        self.X = self.average_all(self.X)
        before, scale = self.totals(), self.totals(absolute=True)
        l = 0
        while l < self.max_level and l <= self.finest:
            self._regrid_level(l)
            l += 1
        self.X = self.average_all(self.X)
        if not self._valid(self.X):
            raise RuntimeError("regridChecked: inadmissible cell after the remap")
        self.regrids += 1
        if self._init:
            return  # building the hierarchy from given level states is not a remap
        after = self.totals()
        if np.any(np.abs(after - before) > 1e-8 * np.maximum(scale, 1e-300)):
            raise RuntimeError("regridChecked: the totals changed in the remap")

    # ------------------------------------------------------------ results
    def totals(self, absolute=False):
        """Conserved totals over the leaf cells of every level (per unit depth); absolute:
        of the magnitudes."""
        a = np.abs if absolute else (lambda x: x)
        t = np.zeros(self.nv)
        for l in range(self.finest + 1):
            dx, dy = self.dxs[l]
            t = t + a(self.X[l][2:-2, 2:-2][self.leaf_mask(l)]).sum(0) * (dx * dy)
        return t

    def level(self, l):
        return self.X[l][2:-2, 2:-2].copy()


class AmrOracle(Hierarchy):
    """Two levels of a domain periodic in x and y (origin 0): U0 (ny, nx, NV), U1
    (2ny, 2nx, NV) read in the active blocks, active (nby, nbx) of level 1."""

    def __init__(self, U0, U1, active, dx, dy, block, **kw):
        ny, nx, nv = np.shape(U0)
        if np.shape(U1) != (2 * ny, 2 * nx, nv):
            raise ValueError("level 1 must be the level-0 domain at ratio 2")
        if np.shape(active) != (2 * ny // block, 2 * nx // block):
            raise ValueError("blocks must tile level 1")
        super().__init__([U0, U1], [None, active], dict(nx=nx, ny=ny, dx=dx, dy=dy, periodic=(1, 1)), block, **kw)

    @classmethod
    def from_base(cls, U0, dx, dy, block, crit, tag_buffer=1, regrid_interval=0, **kw):
        ny, nx, nv = np.shape(U0)
        o = cls(U0, np.zeros((2 * ny, 2 * nx, nv)), np.zeros((2 * ny // block, 2 * nx // block), np.uint8), dx, dy,
                block, crit=crit, tag_buffer=tag_buffer, regrid_interval=regrid_interval, **kw)
        o.regrid()
        o.regrids = 0
        return o

    @property
    def active(self):
        """(nby, nbx) uint8 active blocks of level 1."""
        return self.acts[1]

    def leaf_mask0(self):
        return self.leaf_mask(0)
