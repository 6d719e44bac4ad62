// Multi-level block-AMR time stepper over the C ABI: the loop of BlockAMR::run
// (HyperFlow_V3/src/BlockAMR.cpp:400-439) on levels 0..max_level at refinement ratio 2
// with no time subcycling (every level advances with the same dt, the reference's
// summary field time_subcycling:false).
//
// Layout: each level is one dense ghosted SoA array over its whole domain (the base
// domain times 2^l), 2 ghost layers; its active blocks (block x block cells, aligned)
// are hf_patch views into that array, so same-level neighbours are read in place.
// Memory is what a GB300 has plenty of; the dense arrays keep every index computation
// affine and make regridding a change of the block list.
//
// Per stage (BlockAMR::euler, :202-264): ghosts of every level are filled (physical
// boundaries and in-place neighbours, coarse-fine ghosts by ConservativeInterp from the
// next coarser level, coarse levels first), every level's active blocks take the Euler
// update with face fluxes kept, then finest to coarsest: reflux of the coarse level from
// the fine fluxes (FluxRegister) and average_down; then repairRoundoff over the leaf
// cells of every level (:299-334), average_down, and validation of every level.  A
// stage that fails the repair or the validation is redone first order on all levels.
// flow(h) = two stages and the Heun combination (:266-270); react(dt) advances the
// leaf cells of every level (:271-285); a failed step rolls back and halves dt.
//
// Regrid (:367-373, AMReX regrid with ErrorEst tags :170-200): for l = 0..max_level-1,
// ErrorEst on level l (ghosts filled); a block of level l+1 is active when a tagged
// level-l cell lies in its footprint grown by tag_buffer cells and its footprint grown
// by 2 coarse cells lies in active level-l blocks (proper nesting for the coarse-fine
// ghost interpolation); both footprints wrap across periodic edges.  Blocks that
// become active are filled by ConservativeInterp from level l; blocks that stay keep
// their data.  The block choice is a deterministic function of the tags (the
// reference's Berger-Rigoutsos clustering lives in AMReX).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "hf_internal.h"
#include "mech_h2li.h"

namespace {

struct AmrLevel {
    hf_level L{};
    hf_patch dom{};                 // the whole level domain as one patch view
    int nbx = 0, nby = 0;
    std::vector<uint8_t> active;    // [nby][nbx]
    std::vector<hf_patch> blocks;   // active blocks, row-major block order
    std::vector<hf_patch> patches;  // the patches of the ABI calls: the blocks, or the
                                    // domain as one patch when every block is active
    int32_t* d_regions = nullptr;   // coarse-fine ghost regions (4 int32 each, device)
    int nregions = 0;
    int64_t region_cells = 1;       // largest coarsened region
    // device tables of the graph-captured step (uploaded at rebuild; capacity: every block)
    hf_patch* d_patches = nullptr;
    int64_t* d_foff = nullptr;      // 3 per patch: x-face offset, y-face offset, first cell
    int64_t* d_xoff = nullptr;      // x-face offset per patch (reflux)
    int64_t* d_yoff = nullptr;      // y-face offset per patch (reflux)
    int64_t* d_base = nullptr;      // first cell per patch (validation, CFL)
    int* cover = nullptr;           // reflux cover map over the level's cells
    // batched chemistry scratch of the graph-captured step (allocated on first capture)
    double* trial = nullptr;
    int* fail = nullptr;
    int32_t* order = nullptr;
    unsigned long long* bins = nullptr;
    size_t bytes = 0;
    double *U = nullptr, *S = nullptr, *N = nullptr, *O = nullptr, *B = nullptr;  // state, stage, next, old, backup
    double *fx = nullptr, *fy = nullptr;  // face fluxes packed per patch (capacity: every block)
    int64_t* cells = nullptr;             // leaf cells (device gather list)
    int64_t nleaf = 0;
    uint8_t* leaf_mask = nullptr;         // per patch cells, 1 = leaf (device)
    hf_chem_history hist{nullptr, nullptr};
};

__global__ void k_lincomb_all(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}

}  // namespace

struct hf_amr {
    hf_ctx* ctx = nullptr;
    hf_amr_opts o{};
    int ns = 9, nv = 12;
    std::vector<AmrLevel> lev;  // 0..max_level, allocated up front
    int finest = 0;
    double time = 0.0;
    int64_t steps = 0, regrids = 0;
    // graph-captured steps: state in U, result in O.  A graph captures the buffer
    // pointers of the moment (the host path swaps U and N, the graph path U and O), so
    // each of the two graphs is keyed by level 0's pointers; both are dropped at regrid
    hf::DevStatus* gst = nullptr;
    hf::DevStatus* gst_host = nullptr;
    hf::DevStatus* sst = nullptr;    // per-cell checks of the flux kernels (not used: the
                                     // composite state is checked after reflux)
    hf::RepairScratch* rep = nullptr;
    double* ddt = nullptr;       // device [dt, dt/2]
    double* ddt_host = nullptr;
    double* key[2][4] = {};      // level 0's U, N, S, O when graph k was captured
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int64_t graph_kernels[2] = {0, 0};
    double graph_cfl = -1.0;
    int use_graph = 1, sm_count = 1;
    int64_t graph_steps = 0, host_steps = 0;
    std::vector<const double*> init;  // per-level initial states while the hierarchy is built
};

namespace {

hf_status cuda_st(cudaError_t e) { return e == cudaSuccess ? HF_OK : HF_ERR_CUDA; }

hf_patch block_patch(const AmrLevel& a, int bi, int bj, int B) {
    hf_patch p = a.dom;
    p.ilo = bi * B;
    p.jlo = bj * B;
    p.nx = std::min(B, a.L.nx - p.ilo);
    p.ny = std::min(B, a.L.ny - p.jlo);
    p.offset = (int64_t)p.jlo * a.dom.pitch + p.ilo;
    return p;
}

hf_status cf_regions(hf_amr* m, int l, cudaStream_t s);

// Rebuilds blocks, patches, leaf lists, leaf masks and coarse-fine ghost regions of
// every level from the active maps.
hf_status rebuild(hf_amr* m, cudaStream_t s) {
    const int B = m->o.block;
    for (int l = 0; l <= m->o.max_level; ++l) {
        AmrLevel& a = m->lev[l];
        a.blocks.clear();
        if (l <= m->finest)
            for (int bj = 0; bj < a.nby; ++bj)
                for (int bi = 0; bi < a.nbx; ++bi)
                    if (a.active[(size_t)bj * a.nbx + bi]) a.blocks.push_back(block_patch(a, bi, bj, B));
        // a fully active level runs as one patch: 3 flux launches instead of 3 per block
        if (!a.blocks.empty() && a.blocks.size() == a.active.size())
            a.patches.assign(1, a.dom);
        else
            a.patches = a.blocks;
    }
    for (int l = 1; l <= m->finest; ++l) {
        hf_status r = cf_regions(m, l, s);
        if (r != HF_OK) return r;
    }
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        const AmrLevel* f = l < m->finest ? &m->lev[l + 1] : nullptr;
        std::vector<int64_t> idx;
        std::vector<uint8_t> mask;
        for (const hf_patch& p : a.patches)
            for (int j = 0; j < p.ny; ++j)
                for (int i = 0; i < p.nx; ++i) {
                    const int gi = p.ilo + i, gj = p.jlo + j;
                    // covered when the fine block over (2gi, 2gj) is active
                    const bool covered = f && f->active[(size_t)((2 * gj) / B) * f->nbx + (2 * gi) / B];
                    mask.push_back(covered ? 0 : 1);
                    if (!covered) idx.push_back((int64_t)(gj + a.dom.ng) * a.dom.pitch + (gi + a.dom.ng));
                }
        a.nleaf = (int64_t)idx.size();
        if (cudaMemcpyAsync(a.cells, idx.data(), sizeof(int64_t) * idx.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(a.leaf_mask, mask.data(), mask.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemsetAsync(a.hist.h, 0, sizeof(double) * std::max<int64_t>(a.nleaf, 1), s) != cudaSuccess ||
            cudaMemsetAsync(a.hist.cost, 0, sizeof(int32_t) * std::max<int64_t>(a.nleaf, 1), s) != cudaSuccess)
            return HF_ERR_CUDA;
    }
    // device tables of the graph-captured step (face arrays packed per patch as
    // hf_flux_update packs them); the graphs captured for the old blocks are stale
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        const int np = (int)a.patches.size();
        std::vector<int64_t> foff(3 * (size_t)np), xo(np), yo(np), base(np);
        int64_t ox = 0, oy = 0, b = 0;
        for (int p = 0; p < np; ++p) {
            const hf_patch& P = a.patches[p];
            foff[3 * p] = xo[p] = ox;
            foff[3 * p + 1] = yo[p] = oy;
            foff[3 * p + 2] = base[p] = b;
            ox += (int64_t)m->nv * (P.nx + 1) * P.ny;
            oy += (int64_t)m->nv * P.nx * (P.ny + 1);
            b += (int64_t)P.nx * P.ny;
        }
        if (np && (cudaMemcpyAsync(a.d_patches, a.patches.data(), sizeof(hf_patch) * np, cudaMemcpyHostToDevice, s) !=
                       cudaSuccess ||
                   cudaMemcpyAsync(a.d_foff, foff.data(), sizeof(int64_t) * foff.size(), cudaMemcpyHostToDevice, s) !=
                       cudaSuccess ||
                   cudaMemcpyAsync(a.d_xoff, xo.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                   cudaMemcpyAsync(a.d_yoff, yo.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                   cudaMemcpyAsync(a.d_base, base.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s) != cudaSuccess))
            return HF_ERR_CUDA;
    }
    for (auto& g : m->exec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return cuda_st(cudaStreamSynchronize(s));
}

// Block index nb along a direction with nblk blocks: wrapped when the direction is
// periodic, -1 when it lies outside a non-periodic domain.
int wrap_block(int nb, int nblk, int periodic) {
    if (nb >= 0 && nb < nblk) return nb;
    return periodic ? (nb + nblk) % nblk : -1;
}

// Cell index g along a direction with n cells: wrapped when periodic, -1 outside.
int wrap_cell(int g, int n, int periodic) {
    if (g >= 0 && g < n) return g;
    return periodic ? ((g % n) + n) % n : -1;
}

// Coarse-fine ghost regions of level l's blocks: the 2-cell frame parts that lie in
// inactive blocks (across a periodic boundary: the inactive periodic image), filled by
// ConservativeInterp from level l-1.  A frame part outside a non-periodic domain edge
// holds physical ghosts.  Across a periodic edge the region is interpolated in place
// from the coarse level's ghost frame, which holds the periodic image.  Regions are in
// level-l indices of the dense level array; uploaded once per rebuild.
hf_status cf_regions(hf_amr* m, int l, cudaStream_t s) {
    AmrLevel& a = m->lev[l];
    const AmrLevel& c = m->lev[l - 1];
    const int B = m->o.block;
    std::vector<int32_t> reg;
    int64_t cells = 1;
    for (const hf_patch& p : a.blocks) {
        const int bi = p.ilo / B, bj = p.jlo / B;
        for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
                if (!di && !dj) continue;
                const int nbi = wrap_block(bi + di, a.nbx, a.L.periodic[0]);
                const int nbj = wrap_block(bj + dj, a.nby, a.L.periodic[1]);
                if (nbi < 0 || nbj < 0) continue;                   // outside: physical ghosts
                if (a.active[(size_t)nbj * a.nbx + nbi]) continue;  // in place (or periodic copy)
                int32_t r[4];
                r[0] = di < 0 ? p.ilo - 2 : (di > 0 ? p.ilo + p.nx : p.ilo);
                r[2] = di < 0 ? p.ilo - 1 : (di > 0 ? p.ilo + p.nx + 1 : p.ilo + p.nx - 1);
                r[1] = dj < 0 ? p.jlo - 2 : (dj > 0 ? p.jlo + p.ny : p.jlo);
                r[3] = dj < 0 ? p.jlo - 1 : (dj > 0 ? p.jlo + p.ny + 1 : p.jlo + p.ny - 1);
                // inside the fine array's ghosted box; the coarsened box grown by one
                // inside the coarse array's ghosted box
                if (r[0] < -2 || r[1] < -2 || r[2] > a.L.nx + 1 || r[3] > a.L.ny + 1 || (r[0] >> 1) - 1 < -2 ||
                    (r[1] >> 1) - 1 < -2 || (r[2] >> 1) + 1 > c.L.nx + 1 || (r[3] >> 1) + 1 > c.L.ny + 1)
                    return HF_ERR_ARG;
                reg.insert(reg.end(), r, r + 4);
                cells = std::max<int64_t>(cells, (int64_t)((r[2] >> 1) - (r[0] >> 1) + 1) * ((r[3] >> 1) - (r[1] >> 1) + 1));
            }
    }
    a.nregions = (int)(reg.size() / 4);
    a.region_cells = cells;
    if (reg.empty()) return HF_OK;
    return cuda_st(cudaMemcpyAsync(a.d_regions, reg.data(), sizeof(int32_t) * reg.size(), cudaMemcpyHostToDevice, s)) ==
                   HF_OK
               ? cuda_st(cudaStreamSynchronize(s))
               : HF_ERR_CUDA;
}

// Coarse-fine ghosts of level l in X[l] from X[l-1]: every region in one launch.
hf_status fill_cf(hf_amr* m, int l, double* Uf, const double* Uc, cudaStream_t s) {
    const AmrLevel& a = m->lev[l];
    const AmrLevel& c = m->lev[l - 1];
    int64_t nl = 0;
    if (hf::launch_interp_regions(m->ns, c.dom, Uc, a.dom, Uf, a.d_regions, a.nregions, a.region_cells, s, &nl) !=
        cudaSuccess)
        return HF_ERR_CUDA;
    hf::ctx_add_launches(m->ctx, nl, 0, 0);
    return HF_OK;
}

// Ghosts of every level of the arrays X[l] (coarse levels first).
hf_status fill_all(hf_amr* m, double* const* X, cudaStream_t s) {
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        hf_status r = hf_fill_ghosts(m->ctx, &a.L, a.patches.data(), (int)a.patches.size(), X[l], s);
        if (r == HF_OK && l > 0) r = fill_cf(m, l, X[l], X[l - 1], s);
        if (r != HF_OK) return r;
    }
    return HF_OK;
}

hf_status average_all(hf_amr* m, double* const* X, cudaStream_t s) {
    for (int l = m->finest; l > 0; --l) {
        AmrLevel &f = m->lev[l], &c = m->lev[l - 1];
        hf_status r = hf_average_down(m->ctx, f.patches.data(), (int)f.patches.size(), X[l], c.patches.data(),
                                      (int)c.patches.size(), X[l - 1], s);
        if (r != HF_OK) return r;
    }
    return HF_OK;
}

hf_status validate_all(hf_amr* m, double* const* X, cudaStream_t s) {
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        int64_t bad = -1;
        hf_status r = hf_validate(m->ctx, &a.L, a.patches.data(), (int)a.patches.size(), X[l], &bad, s);
        if (r != HF_OK) return r;
    }
    return HF_OK;
}

cudaError_t g_stage(hf_amr* m, double* const* in, double* const* out, double h, const double* hdev, int first_order,
                    cudaStream_t s, int64_t* nl);

// One composite Euler stage in -> out with host control (BlockAMR::euler, :202-264):
// second order, or, when the repair or the validation of the composite state fails,
// first order on every level (:258-263).  A face that falls back to an inadmissible
// cell is properties() throwing inside the face loop: no redo, the step rolls back.
hf_status euler(hf_amr* m, double* const* in, double* const* out, double h, cudaStream_t s) {
    for (int fo = 0; fo < 2; ++fo) {
        int64_t nl = 0;
        cudaError_t e = cudaMemsetAsync(m->gst, 0, sizeof(hf::DevStatus), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(&m->gst->bad_cell, 0xff, sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = g_stage(m, in, out, h, nullptr, fo, s, &nl);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m->gst_host, m->gst, sizeof(hf::DevStatus), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        hf::ctx_add_launches(m->ctx, nl, 0, 0);
        if (e != cudaSuccess) return HF_ERR_CUDA;
        const unsigned f = m->gst_host->flags;
        hf::ctx_add_repairs(m->ctx, (int64_t)m->gst_host->repairs);
        if (f & hf::ST_FACE_BAD) {
            hf::ctx_set_error(m->ctx, "amr_step: inadmissible cell state at a face");
            return HF_ERR_FACE;
        }
        if (!f) {
            if (fo) hf::ctx_add_counters(m->ctx, 1, 0);
            return HF_OK;
        }
    }
    hf::ctx_set_error(m->ctx, "amr_step: inadmissible composite state after a first-order stage");
    return HF_ERR_INADMISSIBLE;
}

template <class F>
void arrays(hf_amr* m, F pick, double** X) {
    for (int l = 0; l <= m->o.max_level; ++l) X[l] = pick(m->lev[l]);
}

// flow(h): U <- (U + E(E(U)))/2 on every level (BlockAMR::flow, :266-270).
hf_status flow(hf_amr* m, double h, cudaStream_t s) {
    double *U[8], *S[8], *N[8];
    arrays(m, [](AmrLevel& a) { return a.U; }, U);
    arrays(m, [](AmrLevel& a) { return a.S; }, S);
    arrays(m, [](AmrLevel& a) { return a.N; }, N);
    hf_status r = euler(m, U, S, h, s);
    if (r == HF_OK) r = euler(m, S, N, h, s);
    if (r != HF_OK) return r;
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        const int64_t n = (int64_t)(a.bytes / sizeof(double));
        k_lincomb_all<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 0.5, a.U, 0.5, a.N);
        if (cudaGetLastError() != cudaSuccess) return HF_ERR_CUDA;
    }
    r = average_all(m, N, s);
    if (r == HF_OK) r = validate_all(m, N, s);
    if (r != HF_OK) return HF_ERR_COMBINE;
    for (int l = 0; l <= m->finest; ++l) std::swap(m->lev[l].U, m->lev[l].N);
    return HF_OK;
}

// react(dt) on the leaf cells of every level (BlockAMR::react, :271-285).
hf_status react(hf_amr* m, double dt, cudaStream_t s) {
    if (!m->o.chemistry) return HF_OK;
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        if (!a.nleaf) continue;
        int64_t first = -1;
        hf_status r = m->o.chem_form == HF_CHEM_PERSISTENT
                          ? hf_chem_advance_batched(m->ctx, a.U, a.dom.comp_stride, a.cells, a.nleaf, dt, nullptr,
                                                    m->o.rtol, m->o.atol, &a.hist, &first, s)
                          : hf_chem_advance(m->ctx, a.U, a.dom.comp_stride, a.cells, a.nleaf, dt, nullptr, m->o.rtol,
                                            m->o.atol, m->o.chem_form, &first, s);
        if (r != HF_OK) return r;
    }
    double* U[8];
    arrays(m, [](AmrLevel& a) { return a.U; }, U);
    hf_status r = average_all(m, U, s);
    if (r == HF_OK) r = validate_all(m, U, s);
    return r;
}

hf_status totals(hf_amr* m, double* out, cudaStream_t s, int absolute = 0) {
    for (int n = 0; n < m->nv; ++n) out[n] = 0.0;
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        double t[16];
        hf_status r = hf_totals(m->ctx, a.patches.data(), (int)a.patches.size(), a.U, a.leaf_mask, a.L.dx * a.L.dy,
                                absolute, t, s);
        if (r != HF_OK) return r;
        for (int n = 0; n < m->nv; ++n) out[n] += t[n];
    }
    return HF_OK;
}

// ---------------------------------------------------------------- graph-captured step
// The whole Strang step of every level as one CUDA graph: the same kernels as the
// host-driven path above (multi-patch flux, validation and CFL launches, batched
// coarse-fine interpolation, reflux and average_down, batched leaf chemistry) with dt
// computed on the device, every failure a flag in one status block.  The state U of
// each level is only read; the result goes to O, and the host swaps U and O after a
// step without flags.  A flagged step is re-run from the untouched U by the host path
// (first-order redo, repair, rollback and dt halving).

// Ghosts of every level of X (fill_all).
cudaError_t g_fill_all(hf_amr* m, double* const* X, cudaStream_t s, int64_t* nl) {
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        const hf::Level L = hf::make_level(a.L);
        cudaError_t e = hf::launch_fill(m->ns, L, a.patches.data(), a.d_patches, (int)a.patches.size(), X[l], s, nl);
        if (e == cudaSuccess && l > 0)
            e = hf::launch_interp_regions(m->ns, m->lev[l - 1].dom, X[l - 1], a.dom, X[l], a.d_regions, a.nregions,
                                          a.region_cells, s, nl);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// average_down of X, finest to coarsest.
cudaError_t g_average_all(hf_amr* m, double* const* X, cudaStream_t s, int64_t* nl) {
    for (int l = m->finest; l > 0; --l) {
        AmrLevel &f = m->lev[l], &c = m->lev[l - 1];
        cudaError_t e = hf::launch_average_down(f.d_patches, f.patches.data(), (int)f.patches.size(), X[l],
                                                c.d_patches, (int)c.patches.size(), X[l - 1], m->nv, s, nl);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t g_validate_all(hf_amr* m, double* const* X, cudaStream_t s, int64_t* nl) {
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        cudaError_t e = hf::launch_validate_multi(m->ns, a.patches.data(), a.d_patches, (int)a.patches.size(),
                                                  a.d_base, X[l], m->gst, s, nl);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

__global__ void k_merge_face(const hf::DevStatus* from, hf::DevStatus* to) {
    if (from->flags & hf::ST_FACE_BAD) {
        atomicOr(&to->flags, hf::ST_FACE_BAD);
        atomicMin(&to->bad_cell, from->bad_cell);
    }
}

// The leaf cells of every level of X for the composite repair.
hf::RepairLevels repair_levels(hf_amr* m, double* const* X) {
    hf::RepairLevels R{};
    R.nlev = m->finest + 1;
    for (int l = 0; l <= m->finest; ++l) {
        const AmrLevel& a = m->lev[l];
        int64_t mc = 1;
        for (const hf_patch& p : a.patches) mc = std::max<int64_t>(mc, (int64_t)p.nx * p.ny);
        R.lev[l] = hf::RepairLevel{a.d_patches, a.d_base, a.leaf_mask, X[l], (int)a.patches.size(), mc,
                                   a.L.dx * a.L.dy};
    }
    return R;
}

// One composite Euler stage in -> out (BlockAMR::euler, :202-264) with the stage length
// h, or read from hdev (graph-captured steps): ghosts of every level; every level's
// update with its face fluxes (the flux kernels' own per-cell checks go to sst and are
// not used: the reference checks the composite state after reflux); reflux and
// average_down from the finest level down; repairRoundoff over the leaf cells of every
// level; average_down again (a no-op bit for bit when nothing was repaired, so it runs
// unconditionally); validation of every level.  Face failures, material negatives and
// inadmissible cells are flags of gst.
cudaError_t g_stage(hf_amr* m, double* const* in, double* const* out, double h, const double* hdev, int first_order,
                    cudaStream_t s, int64_t* nl) {
    cudaError_t e = g_fill_all(m, in, s, nl);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->sst, 0, sizeof(hf::DevStatus), s);
    for (int l = 0; e == cudaSuccess && l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        e = hf::launch_flux_multi(m->ns, hf::make_level(a.L), a.patches.data(), a.d_patches, (int)a.patches.size(),
                                  a.d_foff, in[l], nullptr, out[l], a.fx, a.fy, h, first_order, m->sst, s, nl, hdev);
    }
    if (e == cudaSuccess) {
        k_merge_face<<<1, 1, 0, s>>>(m->sst, m->gst);
        ++*nl;
        e = cudaGetLastError();
    }
    for (int l = m->finest; e == cudaSuccess && l > 0; --l) {
        AmrLevel &f = m->lev[l], &c = m->lev[l - 1];
        e = hf::launch_reflux(hf::make_level(c.L), c.d_patches, c.patches.data(), (int)c.patches.size(), c.d_xoff,
                              c.d_yoff, c.fx, c.fy, out[l - 1], f.d_patches, f.patches.data(), (int)f.patches.size(),
                              f.d_xoff, f.d_yoff, f.fx, f.fy, c.cover, h, m->nv, s, nl, hdev);
        if (e == cudaSuccess)
            e = hf::launch_average_down(f.d_patches, f.patches.data(), (int)f.patches.size(), out[l], c.d_patches,
                                        (int)c.patches.size(), out[l - 1], m->nv, s, nl);
    }
    if (e == cudaSuccess) e = hf::launch_composite_repair(m->ns, repair_levels(m, out), m->rep, m->gst, s, nl);
    if (e == cudaSuccess) e = g_average_all(m, out, s, nl);
    if (e == cudaSuccess) e = g_validate_all(m, out, s, nl);
    return e;
}

// flow(dt/2) in -> out (S stage buffers): two stages, Heun combination, average_down,
// validation.
cudaError_t g_flow(hf_amr* m, double* const* in, double* const* S, double* const* out, cudaStream_t s, int64_t* nl) {
    const double* half = m->ddt + 1;
    cudaError_t e = g_stage(m, in, S, 0.0, half, 0, s, nl);
    if (e == cudaSuccess) e = g_stage(m, S, out, 0.0, half, 0, s, nl);
    for (int l = 0; e == cudaSuccess && l <= m->finest; ++l) {
        const int64_t n = (int64_t)(m->lev[l].bytes / sizeof(double));
        k_lincomb_all<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 0.5, in[l], 0.5, out[l]);
        ++*nl;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = g_average_all(m, out, s, nl);
    if (e == cudaSuccess) e = g_validate_all(m, out, s, nl);
    return e;
}

// react(dt) on the leaf cells of every level of X (react()).
cudaError_t g_react(hf_amr* m, double* const* X, cudaStream_t s, int64_t* nl) {
    cudaError_t e = cudaSuccess;
    for (int l = 0; e == cudaSuccess && l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        if (!a.nleaf) continue;
        e = cudaMemsetAsync(&m->gst->counter, 0, 2 * sizeof(unsigned long long), s);  // work-queue heads
        if (e == cudaSuccess)
            e = hf::launch_chem_batched(m->ns, X[l], a.dom.comp_stride, a.cells, a.nleaf, 0.0, m->ddt, nullptr,
                                        m->o.rtol, m->o.atol, a.hist.h, a.hist.cost, a.order, a.bins, a.trial, a.fail,
                                        m->gst, m->sm_count, s, nl);
        if (e == cudaSuccess) e = hf::launch_chem_commit(m->ns, X[l], a.dom.comp_stride, a.cells, a.nleaf, a.trial, s, nl);
    }
    if (e == cudaSuccess) e = g_average_all(m, X, s, nl);
    if (e == cudaSuccess) e = g_validate_all(m, X, s, nl);
    return e;
}

cudaError_t g_enqueue_step(hf_amr* m, double cfl, cudaStream_t s, int64_t* nl) {
    double *U[8], *S[8], *N[8], *O[8];
    arrays(m, [](AmrLevel& a) { return a.U; }, U);
    arrays(m, [](AmrLevel& a) { return a.S; }, S);
    arrays(m, [](AmrLevel& a) { return a.N; }, N);
    arrays(m, [](AmrLevel& a) { return a.O; }, O);
    cudaError_t e = cudaMemsetAsync(m->gst, 0, sizeof(hf::DevStatus), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(&m->gst->bad_cell, 0xff, sizeof(unsigned long long), s);
    // stableDt over every level (the max rate over all levels' cells)
    for (int l = 0; e == cudaSuccess && l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        e = hf::launch_cfl_multi(m->ns, hf::make_level(a.L), a.patches.data(), a.d_patches, (int)a.patches.size(),
                                 a.d_base, U[l], m->gst, s, nl);
    }
    if (e == cudaSuccess) e = hf::launch_dt_from_rate(m->gst, cfl, m->ddt, s, nl);
    if (e == cudaSuccess) e = g_flow(m, U, S, N, s, nl);  // flow(dt/2): U -> N
    if (e == cudaSuccess && m->o.chemistry) e = g_react(m, N, s, nl);
    if (e == cudaSuccess) e = g_flow(m, N, S, O, s, nl);  // flow(dt/2): N -> O
    return e;
}

// Scratch of the graph path (chemistry per level over its whole dense domain).
hf_status g_alloc(hf_amr* m) {
    for (int l = 0; l <= m->o.max_level; ++l) {
        AmrLevel& a = m->lev[l];
        if (a.trial) continue;
        const size_t nc = (size_t)a.L.nx * a.L.ny;
        if (cudaMalloc(&a.trial, sizeof(double) * m->nv * nc) != cudaSuccess ||
            cudaMalloc(&a.fail, sizeof(int) * nc) != cudaSuccess ||
            cudaMalloc(&a.order, sizeof(int32_t) * nc) != cudaSuccess ||
            cudaMalloc(&a.bins, hf::CHEM_BINS * sizeof(unsigned long long)) != cudaSuccess)
            return HF_ERR_CUDA;
    }
    return HF_OK;
}

// One graph step: HF_OK with *dt, HF_ERR_INADMISSIBLE with *dt = the graph's dt when the
// host path must re-run the step, HF_ERR_CUDA when no graph could be made.
hf_status g_step(hf_amr* m, double cfl, double* dt, cudaStream_t s) {
    if (m->graph_cfl != cfl)
        for (auto& g : m->exec)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    m->graph_cfl = cfl;
    const AmrLevel& a0 = m->lev[0];
    const double* now[4] = {a0.U, a0.N, a0.S, a0.O};
    int k = -1;
    for (int q = 0; q < 2 && k < 0; ++q)
        if (m->exec[q] && std::equal(now, now + 4, m->key[q])) k = q;
    if (k < 0) {  // capture into a free slot (or replace slot 0)
        k = !m->exec[0] ? 0 : (!m->exec[1] ? 1 : 0);
        if (m->exec[k]) {
            cudaGraphExecDestroy(m->exec[k]);
            m->exec[k] = nullptr;
        }
    }
    if (!m->exec[k]) {
        if (g_alloc(m) != HF_OK) return HF_ERR_CUDA;
        cudaStream_t cs = nullptr;
        cudaGraph_t g = nullptr;
        int64_t nl = 0;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t q = g_enqueue_step(m, cfl, cs, &nl);
            e = cudaStreamEndCapture(cs, &g);
            if (q != cudaSuccess) e = q;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&m->exec[k], g, 0);
        if (g) cudaGraphDestroy(g);
        if (cs) cudaStreamDestroy(cs);
        if (e != cudaSuccess) {
            cudaGetLastError();
            m->exec[k] = nullptr;
            return HF_ERR_CUDA;
        }
        m->graph_kernels[k] = nl;
        for (int q = 0; q < 4; ++q) m->key[k][q] = const_cast<double*>(now[q]);
    }
    if (cudaGraphLaunch(m->exec[k], s) != cudaSuccess ||
        cudaMemcpyAsync(m->gst_host, m->gst, sizeof(hf::DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(m->ddt_host, m->ddt, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return HF_ERR_CUDA;
    int64_t leaf = 0;
    for (int l = 0; l <= m->finest; ++l) leaf += m->lev[l].nleaf;
    hf::ctx_add_launches(m->ctx, m->graph_kernels[k], m->o.chemistry ? leaf : 0, (int64_t)m->gst_host->steps);
    hf::ctx_add_coop(m->ctx, (int64_t)m->gst_host->coop_cells);
    *dt = m->ddt_host[0];
    return m->gst_host->flags ? HF_ERR_INADMISSIBLE : HF_OK;
}

// New active blocks of level l+1 from the tags of level l.
hf_status regrid_level(hf_amr* m, int l, cudaStream_t s) {
    AmrLevel& c = m->lev[l];
    AmrLevel& f = m->lev[l + 1];
    const int B = m->o.block, half = B / 2, buf = m->o.tag_buffer;
    double* U[8];
    arrays(m, [](AmrLevel& a) { return a.U; }, U);
    hf_status r = fill_all(m, U, s);  // ErrorEst reads the neighbours
    if (r != HF_OK) return r;
    int64_t ncell = 0;
    for (const hf_patch& p : c.patches) ncell += (int64_t)p.nx * p.ny;
    uint8_t* dtags = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&dtags), std::max<int64_t>(ncell, 1), s) != cudaSuccess)
        return HF_ERR_CUDA;
    r = hf_tag_cells(m->ctx, &c.L, c.patches.data(), (int)c.patches.size(), c.U, m->time, &m->o.tags, dtags, s);
    std::vector<uint8_t> tags(ncell);
    if (r == HF_OK)
        r = cuda_st(cudaMemcpyAsync(tags.data(), dtags, ncell, cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(dtags, s);
    if (r == HF_OK) r = cuda_st(cudaStreamSynchronize(s));
    if (r != HF_OK) return r;
    // tagged and active maps of level l (cell resolution)
    std::vector<uint8_t> tag((size_t)c.L.nx * c.L.ny, 0), act((size_t)c.L.nx * c.L.ny, 0);
    int64_t k = 0;
    for (const hf_patch& p : c.patches)
        for (int j = 0; j < p.ny; ++j)
            for (int i = 0; i < p.nx; ++i, ++k) {
                const size_t g = (size_t)(p.jlo + j) * c.L.nx + (p.ilo + i);
                tag[g] = tags[k];
                act[g] = 1;
            }
    std::vector<uint8_t> next(f.active.size(), 0);
    for (int bj = 0; bj < f.nby; ++bj)
        for (int bi = 0; bi < f.nbx; ++bi) {
            // footprint of the fine block on level l
            const int i0 = bi * half, j0 = bj * half;
            const int i1 = std::min(i0 + half, c.L.nx) - 1, j1 = std::min(j0 + half, c.L.ny) - 1;
            // both footprints wrap across periodic edges and are cut at the others
            const int px = c.L.periodic[0], py = c.L.periodic[1];
            bool tagged = false;
            for (int jj = j0 - buf; !tagged && jj <= j1 + buf; ++jj)
                for (int ii = i0 - buf; ii <= i1 + buf; ++ii) {
                    const int i = wrap_cell(ii, c.L.nx, px), j = wrap_cell(jj, c.L.ny, py);
                    if (i >= 0 && j >= 0 && tag[(size_t)j * c.L.nx + i]) { tagged = true; break; }
                }
            if (!tagged) continue;
            bool nested = true;
            for (int jj = j0 - 2; nested && jj <= j1 + 2; ++jj)
                for (int ii = i0 - 2; ii <= i1 + 2; ++ii) {
                    const int i = wrap_cell(ii, c.L.nx, px), j = wrap_cell(jj, c.L.ny, py);
                    if (i >= 0 && j >= 0 && !act[(size_t)j * c.L.nx + i]) { nested = false; break; }
                }
            next[(size_t)bj * f.nbx + bi] = nested ? 1 : 0;
        }
    // blocks that become active: ConservativeInterp from level l, or, while the
    // hierarchy is built, the caller's initial state of level l+1 when it gave one
    // (MakeNewLevelFromScratch evaluates the initial condition on every level)
    const double* init = l + 1 < (int)m->init.size() ? m->init[l + 1] : nullptr;
    std::vector<uint8_t> prev = f.active;
    const bool had = m->finest >= l + 1;
    f.active = next;
    int any = 0;
    for (uint8_t v : next) any |= v;
    m->finest = any ? std::max(m->finest, l + 1) : l;
    for (int bj = 0; bj < f.nby; ++bj)
        for (int bi = 0; bi < f.nbx; ++bi) {
            const size_t b = (size_t)bj * f.nbx + bi;
            if (!next[b] || (had && prev[b])) continue;
            const hf_patch p = block_patch(f, bi, bj, B);
            if (init) {
                const int64_t nc = (int64_t)f.L.nx * f.L.ny;
                for (int n = 0; n < m->nv; ++n)
                    if (cudaMemcpy2DAsync(f.U + n * f.dom.comp_stride + (int64_t)(p.jlo + f.dom.ng) * f.dom.pitch +
                                              (p.ilo + f.dom.ng),
                                          f.dom.pitch * sizeof(double),
                                          init + n * nc + (int64_t)p.jlo * f.L.nx + p.ilo, f.L.nx * sizeof(double),
                                          p.nx * sizeof(double), p.ny, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                        return HF_ERR_CUDA;
                continue;
            }
            const int32_t reg[4] = {p.ilo, p.jlo, p.ilo + p.nx - 1, p.jlo + p.ny - 1};
            r = hf_interp_coarse_to_fine(m->ctx, &c.dom, c.U, &p, f.U, reg, s);
            if (r != HF_OK) return r;
        }
    if (!any)
        for (int q = l + 2; q <= m->o.max_level; ++q) std::fill(m->lev[q].active.begin(), m->lev[q].active.end(), 0);
    return rebuild(m, s);
}

}  // namespace

extern "C" {

hf_status hf_amr_regrid(hf_amr* m, void* stream) {
    if (!m) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // regridChecked (:367-373): average_down, totals, remap, average_down, validate,
    // totals; the totals must survive the remap (relative to the total of the
    // magnitudes, so that a component summing to ~0 is judged fairly)
    double* U[8];
    arrays(m, [](AmrLevel& a) { return a.U; }, U);
    double before[16], after[16], scale[16];
    hf_status r = average_all(m, U, s);
    if (r == HF_OK) r = totals(m, before, s);
    if (r == HF_OK) r = totals(m, scale, s, 1);
    for (int l = 0; r == HF_OK && l < m->o.max_level && l <= m->finest; ++l) r = regrid_level(m, l, s);
    if (r == HF_OK) r = average_all(m, U, s);
    if (r == HF_OK) {
        r = validate_all(m, U, s);
        if (r == HF_ERR_INADMISSIBLE) hf::ctx_set_error(m->ctx, "regrid: inadmissible cell after the remap");
    }
    if (r == HF_OK) r = totals(m, after, s);
    if (r != HF_OK) return r;
    ++m->regrids;
    // building the hierarchy from given level states is InitFromScratch, not a remap
    if (!m->init.empty()) return HF_OK;
    double defect = 0.0;
    for (int n = 0; n < m->nv; ++n) defect = std::max(defect, std::fabs(after[n] - before[n]) / std::max(scale[n], 1e-300));
    if (defect > 1e-8) {
        char msg[96];
        snprintf(msg, sizeof msg, "regrid: nonconservative remap (relative defect %.3e)", defect);
        hf::ctx_set_error(m->ctx, msg);
        return HF_ERR_INADMISSIBLE;
    }
    return HF_OK;
}

hf_status hf_amr_create(hf_ctx* ctx, const hf_level* base, const double* U0, const hf_amr_opts* o, hf_amr** out,
                        void* stream) {
    return hf_amr_create_levels(ctx, base, &U0, 1, o, out, stream);
}

hf_status hf_amr_create_levels(hf_ctx* ctx, const hf_level* base, const double* const* U_levels, int nlevels,
                               const hf_amr_opts* o, hf_amr** out, void* stream) {
    if (out) *out = nullptr;
    if (!U_levels || nlevels < 1 || !o || nlevels > o->max_level + 1) return HF_ERR_ARG;
    const double* U0 = U_levels[0];
    if (!ctx || !base || !U0 || !o || !out || o->max_level < 0 || o->max_level > 6 || o->block < 8 ||
        (o->block & 1) || base->nx % (o->block / 2) || base->ny % (o->block / 2) || o->tag_buffer < 0 ||
        !(o->rtol > 0) || !(o->atol > 0))
        return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hf_amr* m = new hf_amr();
    m->ctx = ctx;
    m->o = *o;
    m->ns = hf_nspecies(ctx);
    m->nv = m->ns + 3;
    m->lev.resize(o->max_level + 1);
    bool ok = true;
    for (int l = 0; ok && l <= o->max_level; ++l) {
        AmrLevel& a = m->lev[l];
        a.L = *base;
        a.L.nx = base->nx << l;
        a.L.ny = base->ny << l;
        a.L.dx = base->dx / (1 << l);
        a.L.dy = base->dy / (1 << l);
        hf_patch& d = a.dom;
        d.ilo = d.jlo = 0;
        d.nx = a.L.nx;
        d.ny = a.L.ny;
        d.ng = 2;
        d.pitch = (d.nx + 2 * d.ng + 1) & ~int64_t(1);
        d.comp_stride = (d.pitch * (d.ny + 2 * d.ng) + 31) & ~int64_t(31);
        d.offset = 0;
        a.nbx = (a.L.nx + o->block - 1) / o->block;
        a.nby = (a.L.ny + o->block - 1) / o->block;
        a.active.assign((size_t)a.nbx * a.nby, l == 0 ? 1 : 0);
        a.bytes = sizeof(double) * (size_t)d.comp_stride * m->nv;
        const int64_t nc = (int64_t)a.L.nx * a.L.ny;
        const size_t fb = sizeof(double) * (size_t)m->nv * ((size_t)(a.L.nx + a.nbx) * a.L.ny);
        const size_t gb = sizeof(double) * (size_t)m->nv * ((size_t)a.L.nx * (a.L.ny + a.nby));
        for (double** p : {&a.U, &a.S, &a.N, &a.O, &a.B})
            ok = ok && cudaMalloc(p, a.bytes) == cudaSuccess && cudaMemset(*p, 0, a.bytes) == cudaSuccess;
        ok = ok && cudaMalloc(&a.fx, fb) == cudaSuccess && cudaMalloc(&a.fy, gb) == cudaSuccess &&
             cudaMalloc(&a.cells, sizeof(int64_t) * nc) == cudaSuccess && cudaMalloc(&a.leaf_mask, nc) == cudaSuccess &&
             cudaMalloc(&a.hist.h, sizeof(double) * nc) == cudaSuccess &&
             cudaMalloc(&a.hist.cost, sizeof(int32_t) * nc) == cudaSuccess &&
             cudaMalloc(&a.d_regions, sizeof(int32_t) * 4 * 8 * (size_t)a.nbx * a.nby) == cudaSuccess;
        const size_t cap = (size_t)a.nbx * a.nby;
        ok = ok && cudaMalloc(&a.d_patches, sizeof(hf_patch) * cap) == cudaSuccess &&
             cudaMalloc(&a.d_foff, sizeof(int64_t) * 3 * cap) == cudaSuccess &&
             cudaMalloc(&a.d_xoff, sizeof(int64_t) * cap) == cudaSuccess &&
             cudaMalloc(&a.d_yoff, sizeof(int64_t) * cap) == cudaSuccess &&
             cudaMalloc(&a.d_base, sizeof(int64_t) * cap) == cudaSuccess &&
             cudaMalloc(&a.cover, sizeof(int) * (size_t)nc) == cudaSuccess;
    }
    int dev = 0;
    ok = ok && cudaGetDevice(&dev) == cudaSuccess &&
         cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
         cudaMalloc(&m->gst, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMemset(m->gst, 0, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMallocHost(&m->gst_host, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMalloc(&m->ddt, 2 * sizeof(double)) == cudaSuccess &&
         cudaMallocHost(&m->ddt_host, 2 * sizeof(double)) == cudaSuccess &&
         cudaMalloc(&m->sst, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMemset(m->sst, 0, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMalloc(&m->rep, hf::repair_scratch_bytes()) == cudaSuccess;
    if (ok) {
        AmrLevel& a = m->lev[0];
        const int64_t nc = (int64_t)a.L.nx * a.L.ny;
        for (int n = 0; ok && n < m->nv; ++n)
            ok = cudaMemcpy2DAsync(a.U + n * a.dom.comp_stride + a.dom.ng * a.dom.pitch + a.dom.ng,
                                   a.dom.pitch * sizeof(double), U0 + (size_t)n * nc, a.L.nx * sizeof(double),
                                   a.L.nx * sizeof(double), a.L.ny, cudaMemcpyDeviceToDevice, s) == cudaSuccess;
    }
    hf_status r = ok ? rebuild(m, s) : HF_ERR_CUDA;
    // initial hierarchy: one regrid per level (new blocks from the given level states)
    if (nlevels > 1) m->init.assign(U_levels, U_levels + nlevels);
    for (int k = 0; r == HF_OK && k < o->max_level; ++k) r = hf_amr_regrid(m, stream);
    if (r == HF_OK && nlevels > 1) {
        // run() (:401): average(state) after InitFromScratch, then validate(state)
        double* U[8];
        arrays(m, [](AmrLevel& a) { return a.U; }, U);
        r = average_all(m, U, s);
        if (r == HF_OK) r = validate_all(m, U, s);
    }
    m->init.clear();
    m->regrids = 0;
    if (r != HF_OK) {
        hf_amr_destroy(m);
        return r;
    }
    *out = m;
    return HF_OK;
}

void hf_amr_destroy(hf_amr* m) {
    if (!m) return;
    for (AmrLevel& a : m->lev) {
        for (double* p : {a.U, a.S, a.N, a.O, a.B, a.fx, a.fy}) cudaFree(p);
        cudaFree(a.cells);
        cudaFree(a.leaf_mask);
        cudaFree(a.hist.h);
        cudaFree(a.hist.cost);
        cudaFree(a.d_regions);
        cudaFree(a.d_patches);
        cudaFree(a.d_foff);
        cudaFree(a.d_xoff);
        cudaFree(a.d_yoff);
        cudaFree(a.d_base);
        cudaFree(a.cover);
        cudaFree(a.trial);
        cudaFree(a.fail);
        cudaFree(a.order);
        cudaFree(a.bins);
    }
    for (auto g : m->exec)
        if (g) cudaGraphExecDestroy(g);
    cudaFree(m->gst);
    cudaFreeHost(m->gst_host);
    cudaFree(m->sst);
    cudaFree(m->rep);
    cudaFree(m->ddt);
    cudaFreeHost(m->ddt_host);
    delete m;
}

hf_status hf_amr_cfl_dt(hf_amr* m, double cfl, double* dt, void* stream) {
    if (!m || !dt || !(cfl > 0)) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double h = INFINITY;
    for (int l = 0; l <= m->finest; ++l) {
        AmrLevel& a = m->lev[l];
        double d = 0.0;
        const hf_status r = hf_cfl_dt(m->ctx, &a.L, a.patches.data(), (int)a.patches.size(), a.U, cfl, &d, s);
        if (r != HF_OK) return r;
        h = std::min(h, d);
    }
    *dt = h;
    return HF_OK;
}

hf_status hf_amr_step(hf_amr* m, double cfl, double* dt, void* stream) {
    if (!m || !dt) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double h = *dt;
    if (!(h > 0) && m->use_graph && (!m->o.chemistry || m->o.chem_form == HF_CHEM_PERSISTENT)) {
        double hg = 0.0;
        const hf_status r = g_step(m, cfl, &hg, s);
        if (r == HF_OK) {
            for (int l = 0; l <= m->finest; ++l) std::swap(m->lev[l].U, m->lev[l].O);
            m->time += hg;
            *dt = hg;
            ++m->steps;
            ++m->graph_steps;
            if (m->o.regrid_interval > 0 && m->steps % m->o.regrid_interval == 0) return hf_amr_regrid(m, stream);
            return HF_OK;
        }
        if (r == HF_ERR_CUDA) {
            m->use_graph = 0;  // no graph: the host-driven path from here on
            cudaGetLastError();
        } else {
            h = hg;  // re-run this step with host control from the untouched U
        }
    }
    if (!(h > 0)) {
        // stableDt over the leaf cells of every level (:335-346): the finest level's
        // cells bind (the coarse cells under them are their averages)
        h = INFINITY;
        for (int l = 0; l <= m->finest; ++l) {
            AmrLevel& a = m->lev[l];
            double d = 0.0;
            hf_status r = hf_cfl_dt(m->ctx, &a.L, a.patches.data(), (int)a.patches.size(), a.U, cfl, &d, s);
            if (r != HF_OK) return r;
            h = std::min(h, d);
        }
    }
    for (int l = 0; l <= m->finest; ++l)
        if (cudaMemcpyAsync(m->lev[l].B, m->lev[l].U, m->lev[l].bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return HF_ERR_CUDA;
    for (int attempt = 0; attempt < 18; ++attempt) {
        hf_status r = flow(m, 0.5 * h, s);
        if (r == HF_OK) r = react(m, h, s);
        if (r == HF_OK) r = flow(m, 0.5 * h, s);
        if (r == HF_OK) {
            m->time += h;
            *dt = h;
            ++m->steps;
            ++m->host_steps;
            if (m->o.regrid_interval > 0 && m->steps % m->o.regrid_interval == 0) return hf_amr_regrid(m, stream);
            return HF_OK;
        }
        if (r == HF_ERR_ARG || r == HF_ERR_CUDA || r == HF_ERR_TIMEOUT) return r;
        hf::ctx_add_counters(m->ctx, 0, 1);
        for (int l = 0; l <= m->finest; ++l)
            if (cudaMemcpyAsync(m->lev[l].U, m->lev[l].B, m->lev[l].bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return HF_ERR_CUDA;
        h *= 0.5;  // rollback (:413-418)
    }
    std::string msg = std::string("amr_step: time advancement failed; last attempt: ") + hf_last_error(m->ctx);
    hf::ctx_set_error(m->ctx, msg.c_str());
    return HF_ERR_INADMISSIBLE;
}

hf_status hf_amr_info(const hf_amr* m, int lev, int32_t* nx, int32_t* ny, int32_t* nbx, int32_t* nby,
                      int32_t* finest, int64_t* leaf_cells) {
    if (!m || lev < 0 || lev > m->o.max_level) return HF_ERR_ARG;
    const AmrLevel& a = m->lev[lev];
    if (nx) *nx = a.L.nx;
    if (ny) *ny = a.L.ny;
    if (nbx) *nbx = a.nbx;
    if (nby) *nby = a.nby;
    if (finest) *finest = m->finest;
    if (leaf_cells) *leaf_cells = lev <= m->finest ? a.nleaf : 0;
    return HF_OK;
}

hf_status hf_amr_get_level(hf_amr* m, int lev, double* U, uint8_t* active, void* stream) {
    if (!m || lev < 0 || lev > m->o.max_level) return HF_ERR_ARG;
    const AmrLevel& a = m->lev[lev];
    const int64_t nc = (int64_t)a.L.nx * a.L.ny;
    if (U)
        for (int n = 0; n < m->nv; ++n)
            if (cudaMemcpy2DAsync(U + (size_t)n * nc, a.L.nx * sizeof(double),
                                  a.U + n * a.dom.comp_stride + a.dom.ng * a.dom.pitch + a.dom.ng,
                                  a.dom.pitch * sizeof(double), a.L.nx * sizeof(double), a.L.ny,
                                  cudaMemcpyDeviceToDevice, reinterpret_cast<cudaStream_t>(stream)) != cudaSuccess)
                return HF_ERR_CUDA;
    if (active)
        for (size_t b = 0; b < a.active.size(); ++b) active[b] = lev <= m->finest ? a.active[b] : 0;
    return HF_OK;
}

hf_status hf_amr_totals(hf_amr* m, double* out, void* stream) {
    if (!m || !out) return HF_ERR_ARG;
    return totals(m, out, reinterpret_cast<cudaStream_t>(stream));
}

double hf_amr_time(const hf_amr* m) { return m ? m->time : 0.0; }

void hf_amr_set_graph(hf_amr* m, int enable) {
    if (m) m->use_graph = enable ? 1 : 0;
}

void hf_amr_stats(const hf_amr* m, int64_t* graph_steps, int64_t* host_steps) {
    if (graph_steps) *graph_steps = m ? m->graph_steps : 0;
    if (host_steps) *host_steps = m ? m->host_steps : 0;
}

}  // extern "C"
