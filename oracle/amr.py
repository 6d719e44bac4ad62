"""CPU oracle of the block-AMR composite Strang step.  TEST INFRASTRUCTURE ONLY: tests
import it; the GPU package never does.

A restatement, with the oracle's per-cell functions, of the multi-level stepper's
algorithm at refinement ratio 2 without time subcycling (HyperFlow_V3/src/BlockAMR.cpp:
euler :202-264, flow :266-270, react :271-285, regrid :367-373 with ErrorEst :170-200).
Scope: two levels, periodic in x and y.
- Ghosts: level 0 by the periodic fill; level 1 by the periodic images of its dense
  array, then, in each active block's 2-cell frame part that lies in an inactive block
  (across a periodic edge: the inactive periodic image), ConservativeInterp from level 0
  (src/ConservativeInterp.cpp:18-51, oracle.interp_cell).
- Euler stage: level 0 as one periodic box, level 1 block by block (no wall faces inside
  the periodic domain), then reflux of level 0 from the fine face fluxes
  (FluxRegister, :245-256) and average_down (:256).
- flow(h): two stages, Heun combination, average_down, validation.
- react(dt): the leaf cells of both levels (level-0 cells under no active block, every
  active level-1 cell) through the oracle's ChemistryBatch, then average_down.
- regrid (every regrid_interval steps, and once to build the initial hierarchy from the
  base level alone): ErrorEst tags of level 0; a level-1 block is active when a tagged
  cell lies in its level-0 footprint grown by tag_buffer cells (wrapping across the
  periodic edges; proper nesting always holds under a fully active level 0).  Blocks
  that become active are filled by ConservativeInterp from level 0; blocks that stay
  keep their data; nothing is averaged.  The leaf totals must survive the remap to 1e-8
  of the total of the magnitudes (regridChecked, :369-371).  The block rule is the GPU
  stepper's deterministic choice in place of AMReX's clustering.
States are AoS arrays (..., NS+3); levels are dense ghosted arrays (ny+4, nx+4, NV).
"""
import numpy as np

import oracle


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


class AmrOracle:
    def __init__(self, U0, U1, active, dx, dy, block, chemistry=True, rtol=1e-8, atol=1e-15, crit=None,
                 tag_buffer=1, regrid_interval=0):
        """U0: (ny, nx, NV) level 0; U1: (2ny, 2nx, NV) level 1 (read in active blocks);
        active: (nby, nbx) uint8 of level-1 blocks (block x block fine cells); crit:
        criteria(...) for regrids."""
        ny, nx, nv = U0.shape
        if U1.shape != (2 * ny, 2 * nx, nv):
            raise ValueError("level 1 must be the level-0 domain at ratio 2")
        self.nx, self.ny, self.nv, self.B = nx, ny, nv, block
        self.dx, self.dy = dx, dy
        self.active = np.asarray(active, dtype=np.uint8)
        nby, nbx = self.active.shape
        if nbx * block != 2 * nx or nby * block != 2 * ny:
            raise ValueError("blocks must tile level 1")
        self.blocks = [(bi, bj) for bj in range(nby) for bi in range(nbx) if self.active[bj, bi]]
        self.chemistry, self.rtol, self.atol = chemistry, rtol, atol
        self.crit, self.buf, self.interval = crit, tag_buffer, regrid_interval
        self.time, self.steps, self.regrids = 0.0, 0, 0
        self.g0 = oracle.make_grid(nx, ny, dx, dy, periodic=(1, 1))
        self.g1 = oracle.make_grid(2 * nx, 2 * ny, dx / 2, dy / 2, periodic=(1, 1))
        # one block as its own box: transmissive sides (no wall faces in a periodic domain)
        self.gb = oracle.make_grid(block, block, dx / 2, dy / 2, periodic=(0, 0), bc_lo=(1, 1), bc_hi=(1, 1))
        self.X = [oracle.ghosted(np.array(U0, dtype=np.float64)), oracle.ghosted(np.array(U1, dtype=np.float64))]
        self.regions = self._regions()
        self.X[0][2:-2, 2:-2] = self._averaged(self.X[1], self.X[0])[2:-2, 2:-2]

    @classmethod
    def from_base(cls, U0, dx, dy, block, crit, tag_buffer=1, regrid_interval=0, **kw):
        """The hierarchy the GPU stepper builds from the base level alone: level 0 = U0,
        then one regrid (hf_amr_create)."""
        ny, nx, nv = U0.shape
        o = cls(U0, np.zeros((2 * ny, 2 * nx, nv)), np.zeros((2 * ny // block, 2 * nx // block), np.uint8), dx, dy,
                block, crit=crit, tag_buffer=tag_buffer, regrid_interval=regrid_interval, **kw)
        o.regrid()
        o.regrids = 0
        return o

    # ------------------------------------------------------------ hierarchy
    def _regions(self):
        """Coarse-fine regions (i0, j0, i1, j1) in level-1 indices."""
        B, (nby, nbx) = self.B, self.active.shape
        out = []
        for bi, bj in self.blocks:
            ilo, jlo = bi * B, bj * B
            for dj in (-1, 0, 1):
                for di in (-1, 0, 1):
                    if not di and not dj:
                        continue
                    if self.active[(bj + dj) % nby, (bi + di) % nbx]:
                        continue
                    i0 = ilo - 2 if di < 0 else (ilo + B if di > 0 else ilo)
                    i1 = ilo - 1 if di < 0 else (ilo + B + 1 if di > 0 else ilo + B - 1)
                    j0 = jlo - 2 if dj < 0 else (jlo + B if dj > 0 else jlo)
                    j1 = jlo - 1 if dj < 0 else (jlo + B + 1 if dj > 0 else jlo + B - 1)
                    out.append((i0, j0, i1, j1))
        return out

    def leaf_mask0(self):
        """(ny, nx) True where a level-0 cell lies under no active level-1 block."""
        cov = np.kron(self.active, np.ones((self.B // 2, self.B // 2), dtype=np.uint8)).astype(bool)
        return ~cov

    def fill(self, X):
        X[0] = oracle.fill_ghosts(self.g0, X[0])
        f = X[1]
        inner = f[2:-2, 2:-2]
        f[:] = np.pad(inner, ((2, 2), (2, 2), (0, 0)), mode="wrap")
        c = X[0]
        for i0, j0, i1, j1 in self.regions:
            for fj in range(j0, j1 + 1):
                for fi in range(i0, i1 + 1):
                    ci, cj = fi >> 1, fj >> 1
                    q = c[cj + 2, ci + 2]
                    kids, _ = oracle.interp_cell(q, c[cj + 2, ci + 1], c[cj + 2, ci + 3], c[cj + 1, ci + 2],
                                                 c[cj + 3, ci + 2])
                    f[fj + 2, fi + 2] = kids[(fj & 1) * 2 + (fi & 1)]
        return X

    def _averaged(self, fine, coarse):
        """coarse with every active block's footprint replaced by the average of its children."""
        out = coarse.copy()
        B, h = self.B, self.B // 2
        for bi, bj in self.blocks:
            avg = oracle.average_down(fine[2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B])
            out[2 + bj * h:2 + (bj + 1) * h, 2 + bi * h:2 + (bi + 1) * h] = avg
        return out

    def _check(self, X, what):
        for l in range(2):
            cells = X[l][2:-2, 2:-2]
            if l == 1:
                B = self.B
                cells = np.concatenate([cells[bj * B:(bj + 1) * B, bi * B:(bi + 1) * B].reshape(-1, self.nv)
                                        for bi, bj in self.blocks]) if self.blocks else cells[:0].reshape(-1, self.nv)
            st = oracle.properties(cells.reshape(-1, self.nv))[3]
            if np.any(st):
                raise RuntimeError("inadmissible level-%d cell after %s" % (l, what))

    # ------------------------------------------------------------ step
    def euler(self, Xin, h):
        Xin = self.fill([x.copy() for x in Xin])
        out = [x.copy() for x in Xin]
        o0, fx0, fy0, st = oracle.euler_stage(self.g0, Xin[0], h)
        if st:
            raise RuntimeError("level-0 face inadmissible")
        out[0][2:-2, 2:-2] = o0[2:-2, 2:-2]
        B = self.B
        boxes, fxl, fyl = [], [], []
        for bi, bj in self.blocks:
            i0, j0 = bi * B, bj * B
            ob, fxb, fyb, st = oracle.euler_stage(self.gb, Xin[1][j0:j0 + B + 4, i0:i0 + B + 4], h)
            if st:
                raise RuntimeError("level-1 face inadmissible")
            out[1][j0 + 2:j0 + 2 + B, i0 + 2:i0 + 2 + B] = ob[2:-2, 2:-2]
            boxes.append((i0, j0, i0 + B - 1, j0 + B - 1))
            fxl.append(fxb)
            fyl.append(fyb)
        self._check(out, "a stage")
        if boxes:
            out[0][2:-2, 2:-2] = oracle.reflux(out[0][2:-2, 2:-2], fx0, fy0, boxes, fxl, fyl, h, self.dx, self.dy,
                                               periodic=(1, 1))
        out[0] = self._averaged(out[1], out[0])
        return out

    def flow(self, h):
        U = self.X
        S = self.euler(U, h)
        N = self.euler(S, h)
        for l in range(2):
            N[l] = 0.5 * U[l] + 0.5 * N[l]
        N[0] = self._averaged(N[1], N[0])
        self._check(N, "the Heun combination")
        self.X = N

    def react(self, dt):
        if not self.chemistry:
            return
        B, nv = self.B, self.nv
        m0 = self.leaf_mask0()
        c0 = self.X[0][2:-2, 2:-2]
        cells = [c0[m0]]
        for bi, bj in self.blocks:
            cells.append(self.X[1][2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B].reshape(-1, nv))
        batch = np.concatenate(cells)
        out, bad, _ = oracle.chem_batch(batch, dt, rtol=self.rtol, atol=self.atol)
        if bad >= 0:
            raise RuntimeError("chemistry cell %d failed" % bad)
        n0 = int(m0.sum())
        c0[m0] = out[:n0]
        k = n0
        for bi, bj in self.blocks:
            self.X[1][2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B] = out[k:k + B * B].reshape(B, B, nv)
            k += B * B
        self.X[0] = self._averaged(self.X[1], self.X[0])
        self._check(self.X, "react")

    def step(self, dt):
        self.flow(0.5 * dt)
        self.react(dt)
        self.flow(0.5 * dt)
        self.time += dt
        self.steps += 1
        if self.interval > 0 and self.steps % self.interval == 0:
            self.regrid()

    def regrid(self):
        before, scale = self.totals(), self.totals(absolute=True)
        c = oracle.fill_ghosts(self.g0, self.X[0].copy())
        tags, st = oracle.tag(self.g0, c, self.time, self.crit)
        if st:
            raise RuntimeError("ErrorEst: inadmissible level-0 cell")
        B, h, buf = self.B, self.B // 2, self.buf
        nby, nbx = self.active.shape
        nxt = np.zeros_like(self.active)
        for bj in range(nby):
            for bi in range(nbx):
                rows = np.arange(bj * h - buf, (bj + 1) * h + buf) % self.ny
                cols = np.arange(bi * h - buf, (bi + 1) * h + buf) % self.nx
                nxt[bj, bi] = 1 if tags[np.ix_(rows, cols)].any() else 0
        f = self.X[1]
        for bj, bi in zip(*np.nonzero(nxt & (1 - self.active))):
            for fj in range(bj * B, (bj + 1) * B):
                for fi in range(bi * B, (bi + 1) * B):
                    ci, cj = fi >> 1, fj >> 1
                    kids, _ = oracle.interp_cell(c[cj + 2, ci + 2], c[cj + 2, ci + 1], c[cj + 2, ci + 3],
                                                 c[cj + 1, ci + 2], c[cj + 3, ci + 2])
                    f[fj + 2, fi + 2] = kids[(fj & 1) * 2 + (fi & 1)]
        self.active = nxt
        self.blocks = [(bi, bj) for bj in range(nby) for bi in range(nbx) if self.active[bj, bi]]
        self.regions = self._regions()
        self.regrids += 1
        after = self.totals()
        if np.any(np.abs(after - before) > 1e-8 * scale):
            raise RuntimeError("regridChecked: the totals changed in the remap")

    def totals(self, absolute=False):
        """Conserved totals over the leaf cells of both levels (per unit depth); absolute:
        of the magnitudes."""
        B = self.B
        v0, v1 = self.dx * self.dy, self.dx * self.dy / 4
        a = np.abs if absolute else (lambda x: x)
        t = a(self.X[0][2:-2, 2:-2][self.leaf_mask0()]).sum(0) * v0
        for bi, bj in self.blocks:
            t = t + a(self.X[1][2 + bj * B:2 + (bj + 1) * B, 2 + bi * B:2 + (bi + 1) * B]).reshape(-1, self.nv).sum(0) * v1
        return t

    def level(self, l):
        return self.X[l][2:-2, 2:-2].copy()
