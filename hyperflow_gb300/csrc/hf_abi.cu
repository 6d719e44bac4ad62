// C ABI of libhyperflow_gpu.so (declared in include/hyperflow_gpu.h): context,
// scratch management, status read-back and dispatch to the kernels of hf_flux.cu
// and hf_chem.cu.  Error behaviour mirrors the reference's exceptions as return
// codes (see the header for the mapping).
#include <cuda.h>
#include <cstdio>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "hf_internal.h"
#include "mech_h2li.h"

using namespace hf;

struct hf_ctx {
    int ns = 9;
    int device = 0;
    int sm_count = 1;
    std::string err;
    hf_counters cnt{};
    DevStatus* st = nullptr;       // device status block
    DevStatus* st_host = nullptr;  // pinned mirror
    void* scratch = nullptr;       // grown on demand
    size_t scratch_bytes = 0;
    hf_patch* d_patches = nullptr;
    int d_patch_cap = 0;
    int64_t* d_off = nullptr;  // per-patch offsets of the multi-patch flux launches
    int d_off_cap = 0;
    RepairScratch* rep = nullptr;  // roundoff repair scratch (fixed size)
    // tensor-map cache for the fused flux kernel
    struct TMap { const double* base; hf_patch P; alignas(64) unsigned char map[128]; };
    std::vector<TMap> tmaps;
    // second scratch area for the block-AMR operations (tables, cover map, partial sums)
    void* aux = nullptr;
    size_t aux_bytes = 0;
    // optional per-class device timing
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool pending = false;
    int pending_class = 0;
    double ms[3] = {0, 0, 0};
    int64_t launches[3] = {0, 0, 0};
};

namespace {

hf_status fail(hf_ctx* c, hf_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}
hf_status cuda_fail(hf_ctx* c, cudaError_t e, const char* where) {
    return fail(c, HF_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define HF_CUDA(call)                                             \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

cudaError_t reset_status(hf_ctx* ctx, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(ctx->st, 0, sizeof(DevStatus), s);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(&ctx->st->bad_cell, 0xff, sizeof(unsigned long long), s);
}
// Timing brackets: tic() before a class's launches, toc() after them; the elapsed
// time is collected at the next stream synchronisation (read_status).
void tic(hf_ctx* ctx, int cls, cudaStream_t s) {
    if (!ctx->timing) return;
    cudaEventRecord(ctx->ev0, s);
    ctx->pending_class = cls;
}
void toc(hf_ctx* ctx, cudaStream_t s, int64_t nlaunch) {
    if (!ctx->timing) return;
    cudaEventRecord(ctx->ev1, s);
    ctx->pending = true;
    ctx->launches[ctx->pending_class] += nlaunch;
}
cudaError_t read_status(hf_ctx* ctx, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(ctx->st_host, ctx->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && ctx->pending) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) == cudaSuccess) ctx->ms[ctx->pending_class] += t;
        else (void)cudaGetLastError();  // leave no pending error for the caller's next call
        ctx->pending = false;
    }
    return e;
}
void* scratch(hf_ctx* ctx, size_t bytes) {
    if (bytes > ctx->scratch_bytes) {
        if (ctx->scratch) cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        if (cudaMalloc(&ctx->scratch, bytes) != cudaSuccess) return nullptr;
        ctx->scratch_bytes = bytes;
    }
    return ctx->scratch;
}
cudaError_t upload_patches(hf_ctx* ctx, const hf_patch* p, int n, cudaStream_t s) {
    if (n > ctx->d_patch_cap) {
        if (ctx->d_patches) cudaFree(ctx->d_patches);
        ctx->d_patches = nullptr;
        cudaError_t e = cudaMalloc(&ctx->d_patches, sizeof(hf_patch) * n);
        if (e != cudaSuccess) return e;
        ctx->d_patch_cap = n;
    }
    cudaError_t e = cudaMemcpyAsync(ctx->d_patches, p, sizeof(hf_patch) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}
static cudaError_t upload_offsets(hf_ctx* ctx, const int64_t* v, int n, cudaStream_t s) {
    if (n > ctx->d_off_cap) {
        if (ctx->d_off) cudaFree(ctx->d_off);
        ctx->d_off = nullptr;
        cudaError_t e = cudaMalloc(&ctx->d_off, sizeof(int64_t) * n);
        if (e != cudaSuccess) return e;
        ctx->d_off_cap = n;
    }
    cudaError_t e = cudaMemcpyAsync(ctx->d_off, v, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}
bool patch_ok(const hf_patch& P) {
    return P.nx > 0 && P.ny > 0 && P.ng >= 2 && P.pitch >= P.nx + 2 * P.ng &&
           P.comp_stride >= P.pitch * (P.ny + 2 * P.ng) && P.offset >= 0;
}
bool level_ok(const hf_level& L) {
    if (L.nx <= 0 || L.ny <= 0 || !(L.dx > 0) || !(L.dy > 0)) return false;
    for (int d = 0; d < 2; ++d) {
        if (L.bc_lo[d] < 0 || L.bc_lo[d] > 3 || L.bc_hi[d] < 0 || L.bc_hi[d] > 2) return false;
        if (L.bc_lo[d] == HF_BC_WEDGE && (d != 1 || L.periodic[1])) return false;
    }
    return true;
}
const void* tensor_map(hf_ctx* ctx, const double* base, const hf_patch& P) {
    for (auto& t : ctx->tmaps)
        if (t.base == base && !memcmp(&t.P, &P, sizeof(P))) return t.map;
    hf_ctx::TMap t;
    t.base = base;
    t.P = P;
    if (!make_tensor_map(t.map, base, P, ctx->ns + 3)) return nullptr;
    if (ctx->tmaps.size() > 64) ctx->tmaps.erase(ctx->tmaps.begin());
    ctx->tmaps.push_back(t);
    return ctx->tmaps.back().map;
}

}  // namespace

namespace hf {
void ctx_add_counters(hf_ctx* ctx, int64_t first_order_stages, int64_t retries) {
    ctx->cnt.first_order_stages += first_order_stages;
    ctx->cnt.retries += retries;
}
void ctx_add_repairs(hf_ctx* ctx, int64_t repairs) { ctx->cnt.roundoff_repairs += repairs; }
void ctx_add_coop(hf_ctx* ctx, int64_t coop_cells) { ctx->cnt.chem_coop_cells += coop_cells; }
void ctx_set_error(hf_ctx* ctx, const char* msg) {
    if (ctx) ctx->err = msg;
}
void ctx_add_launches(hf_ctx* ctx, int64_t kernels, int64_t chem_cells, int64_t chem_steps) {
    ctx->cnt.kernel_launches += kernels;
    ctx->cnt.chem_cell_calls += chem_cells;
    ctx->cnt.chem_steps += chem_steps;
}
bool ctx_timing_enabled(const hf_ctx* ctx) { return ctx->timing; }
void ctx_add_timing(hf_ctx* ctx, double flux_ms, double chem_ms, double other_ms, int64_t flux_launches,
                    int64_t chem_launches, int64_t other_launches) {
    ctx->ms[0] += flux_ms;
    ctx->ms[1] += chem_ms;
    ctx->ms[2] += other_ms;
    ctx->launches[0] += flux_launches;
    ctx->launches[1] += chem_launches;
    ctx->launches[2] += other_launches;
}
}  // namespace hf

extern "C" {

hf_status hf_init(const char* mechanism, int device, hf_ctx** out) {
    if (!out) return HF_ERR_ARG;
    *out = nullptr;
    int ns = 9;
    if (mechanism && *mechanism) {
        std::string m(mechanism);
        auto ends = [&](const std::string& suf) {
            return m.size() >= suf.size() && m.compare(m.size() - suf.size(), suf.size(), suf) == 0;
        };
        if (m == "H2_Li" || ends("H2_Li.yaml")) ns = 9;
        else if (m == "H2_Li+AR") ns = 10;
        else return HF_ERR_ARG;
    }
    hf_ctx* ctx = new hf_ctx();
    ctx->ns = ns;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->st, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->st_host, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->rep, repair_scratch_bytes());
    if (e == cudaSuccess) e = chem_set_rate_scale(nullptr);
    if (e == cudaSuccess) e = chem_prefer_l1();
    if (e == cudaSuccess) e = adjoint_set_rate_scale(nullptr);
    if (e != cudaSuccess) {
        hf_destroy(ctx);
        return HF_ERR_CUDA;
    }
    *out = ctx;
    return HF_OK;
}

void hf_set_timing(hf_ctx* ctx, int enable) {
    if (!ctx) return;
    if (enable && !ctx->ev0) {
        cudaEventCreate(&ctx->ev0);
        cudaEventCreate(&ctx->ev1);
    }
    ctx->timing = enable != 0 && ctx->ev0;
    ctx->pending = false;
    for (int k = 0; k < 3; ++k) { ctx->ms[k] = 0; ctx->launches[k] = 0; }
}
void hf_get_timing(const hf_ctx* ctx, double ms[3], int64_t launches[3]) {
    for (int k = 0; k < 3; ++k) {
        if (ms) ms[k] = ctx ? ctx->ms[k] : 0.0;
        if (launches) launches[k] = ctx ? ctx->launches[k] : 0;
    }
}

void hf_destroy(hf_ctx* ctx) {
    if (!ctx) return;
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->st) cudaFree(ctx->st);
    if (ctx->st_host) cudaFreeHost(ctx->st_host);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->aux) cudaFree(ctx->aux);
    if (ctx->d_patches) cudaFree(ctx->d_patches);
    if (ctx->d_off) cudaFree(ctx->d_off);
    if (ctx->rep) cudaFree(ctx->rep);
    delete ctx;
}

int hf_nspecies(const hf_ctx* ctx) { return ctx ? ctx->ns : 0; }
const char* hf_last_error(const hf_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
void hf_get_counters(const hf_ctx* ctx, hf_counters* out) {
    if (ctx && out) *out = ctx->cnt;
}

hf_status hf_set_rate_scale(hf_ctx* ctx, const double* scale) {
    if (!ctx) return HF_ERR_ARG;
    HF_CUDA(cudaSetDevice(ctx->device));
    HF_CUDA(chem_set_rate_scale(scale));
    HF_CUDA(adjoint_set_rate_scale(scale));
    return HF_OK;
}

hf_status hf_properties(hf_ctx* ctx, const double* q, int64_t stride, int64_t count, double* p, double* a, double* T,
                        int32_t* status, void* stream) {
    if (!ctx || !q || !p || !a || !T || !status || count < 0 || stride < count) return fail(ctx, HF_ERR_ARG, "properties: bad arguments");
    if (count == 0) return HF_OK;
    HF_CUDA(reset_status(ctx, S(stream)));
    HF_CUDA(launch_properties(ctx->ns, q, stride, count, p, a, T, status, ctx->st, S(stream), &ctx->cnt.kernel_launches));
    HF_CUDA(read_status(ctx, S(stream)));
    return ctx->st_host->flags ? HF_ERR_INADMISSIBLE : HF_OK;
}

hf_status hf_hllc(hf_ctx* ctx, const double* l, const double* r, const double* pl, const double* pr, int64_t stride,
                  int64_t count, int dir, double* f, void* stream) {
    if (!ctx || !l || !r || !pl || !pr || !f || count < 0 || stride < count || (dir != 0 && dir != 1))
        return fail(ctx, HF_ERR_ARG, "hllc: bad arguments");
    if (count == 0) return HF_OK;
    HF_CUDA(launch_hllc(ctx->ns, l, r, pl, pr, stride, count, dir, f, S(stream), &ctx->cnt.kernel_launches));
    return HF_OK;
}

hf_status hf_fill_ghosts(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, double* U,
                         void* stream) {
    if (!ctx || !level || !patches || npatch <= 0 || !U || !level_ok(*level)) return fail(ctx, HF_ERR_ARG, "fill_ghosts: bad arguments");
    for (int p = 0; p < npatch; ++p)
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "fill_ghosts: bad patch");
    HF_CUDA(upload_patches(ctx, patches, npatch, S(stream)));
    const Level L = make_level(*level);
    HF_CUDA(launch_fill(ctx->ns, L, patches, ctx->d_patches, npatch, U, S(stream), &ctx->cnt.kernel_launches));
    return HF_OK;
}

hf_status hf_interp_coarse_to_fine(hf_ctx* ctx, const hf_patch* coarse, const double* Uc, const hf_patch* fine,
                                   double* Uf, const int32_t region[4], void* stream) {
    if (!ctx || !coarse || !Uc || !fine || !Uf || !region || !patch_ok(*coarse) || !patch_ok(*fine))
        return fail(ctx, HF_ERR_ARG, "interp: bad arguments");
    if (region[2] < region[0] || region[3] < region[1]) return fail(ctx, HF_ERR_ARG, "interp: empty region");
    // the coarsened region grown by one must lie in the coarse patch's ghosted box,
    // the region itself in the fine patch's ghosted box
    const int ci0 = (region[0] >> 1) - 1, cj0 = (region[1] >> 1) - 1, ci1 = (region[2] >> 1) + 1, cj1 = (region[3] >> 1) + 1;
    if (ci0 < coarse->ilo - coarse->ng || cj0 < coarse->jlo - coarse->ng || ci1 >= coarse->ilo + coarse->nx + coarse->ng ||
        cj1 >= coarse->jlo + coarse->ny + coarse->ng)
        return fail(ctx, HF_ERR_ARG, "interp: coarse patch does not hold the coarsened region");
    if (region[0] < fine->ilo - fine->ng || region[1] < fine->jlo - fine->ng || region[2] >= fine->ilo + fine->nx + fine->ng ||
        region[3] >= fine->jlo + fine->ny + fine->ng)
        return fail(ctx, HF_ERR_ARG, "interp: region outside the fine patch");
    HF_CUDA(launch_interp(ctx->ns, *coarse, Uc, *fine, Uf, region, S(stream), &ctx->cnt.kernel_launches));
    return HF_OK;
}

static char* aux_scratch(hf_ctx* ctx, size_t bytes);

// Roundoff repair (the composite kernels over one level, every cell a leaf) + validation
// of one level after a stage (BlockAMR.cpp:257, 299-334).
static hf_status repair_and_validate(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, double* U,
                                     cudaStream_t s, int64_t* bad_cell) {
    std::vector<int64_t> base(npatch);
    int64_t b = 0, mc = 1;
    for (int p = 0; p < npatch; ++p) {
        base[p] = b;
        b += (int64_t)patches[p].nx * patches[p].ny;
        mc = std::max<int64_t>(mc, (int64_t)patches[p].nx * patches[p].ny);
    }
    HF_CUDA(upload_patches(ctx, patches, npatch, s));
    HF_CUDA(upload_offsets(ctx, base.data(), npatch, s));
    RepairLevels R{};
    R.nlev = 1;
    R.lev[0] = RepairLevel{ctx->d_patches, ctx->d_off, nullptr, U, npatch, mc, level->dx * level->dy};
    HF_CUDA(reset_status(ctx, s));
    HF_CUDA(launch_composite_repair(ctx->ns, R, ctx->rep, ctx->st, s, &ctx->cnt.kernel_launches));
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags & ST_MATERIAL) return fail(ctx, HF_ERR_NEGATIVE, "materially negative species after a stage");
    ctx->cnt.roundoff_repairs += (int64_t)ctx->st_host->repairs;
    HF_CUDA(reset_status(ctx, s));
    int64_t vb = 0;
    for (int p = 0; p < npatch; ++p) {
        HF_CUDA(launch_validate(ctx->ns, patches[p], U, vb, ctx->st, s, &ctx->cnt.kernel_launches));
        vb += (int64_t)patches[p].nx * patches[p].ny;
    }
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags) {
        if (bad_cell) *bad_cell = (int64_t)ctx->st_host->bad_cell;
        return fail(ctx, HF_ERR_INADMISSIBLE, "inadmissible state after a stage");
    }
    return HF_OK;
}

hf_status hf_repair_roundoff(hf_ctx* ctx, int nlev, const hf_level* levels, const hf_patch* const* patches,
                             const int* npatch, double* const* U, const uint8_t* const* leaf, int64_t* repairs,
                             void* stream) {
    if (repairs) *repairs = 0;
    if (!ctx || nlev < 1 || nlev > REPAIR_MAX_LEVELS || !levels || !patches || !npatch || !U)
        return fail(ctx, HF_ERR_ARG, "repair_roundoff: bad arguments");
    for (int l = 0; l < nlev; ++l) {
        if (!level_ok(levels[l]) || !patches[l] || npatch[l] <= 0 || !U[l])
            return fail(ctx, HF_ERR_ARG, "repair_roundoff: bad level");
        for (int p = 0; p < npatch[l]; ++p)
            if (!patch_ok(patches[l][p])) return fail(ctx, HF_ERR_ARG, "repair_roundoff: bad patch");
    }
    const cudaStream_t s = S(stream);
    // per-level device tables: patches | first-cell offsets, in the aux scratch
    size_t bytes = 0;
    for (int l = 0; l < nlev; ++l) bytes += ((sizeof(hf_patch) + sizeof(int64_t)) * (size_t)npatch[l] + 255) & ~size_t(255);
    char* w = aux_scratch(ctx, bytes);
    if (!w) return fail(ctx, HF_ERR_CUDA, "repair_roundoff: scratch allocation failed");
    RepairLevels R{};
    R.nlev = nlev;
    size_t off = 0;
    for (int l = 0; l < nlev; ++l) {
        const int np = npatch[l];
        std::vector<int64_t> base(np);
        int64_t b = 0, mc = 1;
        for (int p = 0; p < np; ++p) {
            base[p] = b;
            b += (int64_t)patches[l][p].nx * patches[l][p].ny;
            mc = std::max<int64_t>(mc, (int64_t)patches[l][p].nx * patches[l][p].ny);
        }
        hf_patch* dp = reinterpret_cast<hf_patch*>(w + off);
        int64_t* db = reinterpret_cast<int64_t*>(w + off + sizeof(hf_patch) * np);
        off += ((sizeof(hf_patch) + sizeof(int64_t)) * (size_t)np + 255) & ~size_t(255);
        HF_CUDA(cudaMemcpyAsync(dp, patches[l], sizeof(hf_patch) * np, cudaMemcpyHostToDevice, s));
        HF_CUDA(cudaMemcpyAsync(db, base.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s));
        HF_CUDA(cudaStreamSynchronize(s));
        R.lev[l] = RepairLevel{dp, db, leaf ? leaf[l] : nullptr, U[l], np, mc, levels[l].dx * levels[l].dy};
    }
    HF_CUDA(reset_status(ctx, s));
    HF_CUDA(launch_composite_repair(ctx->ns, R, ctx->rep, ctx->st, s, &ctx->cnt.kernel_launches));
    HF_CUDA(read_status(ctx, s));
    if (repairs) *repairs = (int64_t)ctx->st_host->repairs;
    if (ctx->st_host->flags & ST_MATERIAL)
        return fail(ctx, HF_ERR_NEGATIVE, "repair_roundoff: materially negative species or insufficient donor");
    ctx->cnt.roundoff_repairs += (int64_t)ctx->st_host->repairs;
    return HF_OK;
}

hf_status hf_flux_update(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, const double* U_in,
                         const double* U_old, double* U_out, double* fx, double* fy, double h, int first_order,
                         int form, int64_t* bad_cell, void* stream) {
    if (bad_cell) *bad_cell = -1;
    if (!ctx || !level || !patches || npatch <= 0 || !U_in || !U_out || U_in == U_out || !level_ok(*level) ||
        !(h > 0) || (form != HF_FLUX_PLAIN && form != HF_FLUX_FUSED))
        return fail(ctx, HF_ERR_ARG, "flux_update: bad arguments");
    for (int p = 0; p < npatch; ++p)
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "flux_update: bad patch");
    const cudaStream_t s = S(stream);
    const Level L = make_level(*level);
    const int nv = ctx->ns + 3;
    if (form == HF_FLUX_FUSED) {
        const hf_patch& P = patches[0];
        if (npatch != 1 || P.ilo != 0 || P.jlo != 0 || P.nx != level->nx || P.ny != level->ny || (P.ng & 1) || fx || fy)
            return fail(ctx, HF_ERR_ARG, "flux_update: the fused form takes one domain-covering patch, even ng, no face output");
    }
    // face flux storage for the plain form
    int64_t nfx_tot = 0, nfy_tot = 0;
    for (int p = 0; p < npatch; ++p) {
        nfx_tot += (int64_t)nv * (patches[p].nx + 1) * patches[p].ny;
        nfy_tot += (int64_t)nv * patches[p].nx * (patches[p].ny + 1);
    }
    double* FX = fx;
    double* FY = fy;
    if (form == HF_FLUX_PLAIN && (!fx || !fy)) {
        double* w = static_cast<double*>(scratch(ctx, sizeof(double) * (size_t)(nfx_tot + nfy_tot)));
        if (!w) return fail(ctx, HF_ERR_CUDA, "flux_update: scratch allocation failed");
        if (!FX) FX = w;
        if (!FY) FY = w + nfx_tot;
    }
    auto run = [&](const double* uold) -> hf_status {
        HF_CUDA(reset_status(ctx, s));
        const int64_t l0 = ctx->cnt.kernel_launches;
        tic(ctx, 0, s);
        if (form == HF_FLUX_FUSED) {
            const void* tm = tensor_map(ctx, U_in, patches[0]);
            if (!tm) return fail(ctx, HF_ERR_ARG, "flux_update: TMA descriptor rejected (alignment/pitch)");
            HF_CUDA(launch_flux_fused(ctx->ns, L, patches[0], tm, U_in, uold, U_out, h, nullptr, first_order, 0, ctx->st, s,
                                      &ctx->cnt.kernel_launches));
        } else if (npatch == 1) {
            HF_CUDA(launch_flux_plain(ctx->ns, L, patches[0], 0, U_in, uold, U_out, FX, FY, h, first_order, 0, ctx->st,
                                      s, &ctx->cnt.kernel_launches));
        } else {
            // every patch in one launch per kernel: face arrays packed per patch in patch order
            std::vector<int64_t> off(3 * (size_t)npatch);
            int64_t base = 0, ox = 0, oy = 0;
            for (int p = 0; p < npatch; ++p) {
                const hf_patch& P = patches[p];
                off[3 * p] = ox;
                off[3 * p + 1] = oy;
                off[3 * p + 2] = base;
                base += (int64_t)P.nx * P.ny;
                ox += (int64_t)nv * (P.nx + 1) * P.ny;
                oy += (int64_t)nv * P.nx * (P.ny + 1);
            }
            HF_CUDA(upload_patches(ctx, patches, npatch, s));
            HF_CUDA(upload_offsets(ctx, off.data(), 3 * npatch, s));
            HF_CUDA(launch_flux_multi(ctx->ns, L, patches, ctx->d_patches, npatch, ctx->d_off, U_in, uold, U_out, FX, FY,
                                      h, first_order, ctx->st, s, &ctx->cnt.kernel_launches));
        }
        toc(ctx, s, ctx->cnt.kernel_launches - l0);
        HF_CUDA(read_status(ctx, s));
        return HF_OK;
    };
    hf_status r = run(U_old);
    if (r != HF_OK) return r;
    unsigned f = ctx->st_host->flags;
    if (bad_cell && f) *bad_cell = (int64_t)ctx->st_host->bad_cell;
    if (f & ST_TIMEOUT) return fail(ctx, HF_ERR_TIMEOUT, "flux_update: TMA wait timed out");
    if (f & ST_FACE_BAD) return fail(ctx, HF_ERR_FACE, "flux_update: inadmissible cell state at a face");
    if (f & ST_STAGE_BAD) return fail(ctx, HF_ERR_INADMISSIBLE, "flux_update: inadmissible stage output");
    if (f & ST_NEGATIVE) {
        // roundoff repair path: recompute the pure stage output if it was combined
        if (U_old) {
            r = run(nullptr);
            if (r != HF_OK) return r;
        }
        r = repair_and_validate(ctx, level, patches, npatch, U_out, s, bad_cell);
        if (r != HF_OK) return r;
        if (U_old) {
            HF_CUDA(reset_status(ctx, s));
            int64_t base = 0;
            for (int p = 0; p < npatch; ++p) {
                HF_CUDA(launch_combine(ctx->ns, patches[p], U_old, U_out, base, ctx->st, s, &ctx->cnt.kernel_launches));
                base += (int64_t)patches[p].nx * patches[p].ny;
            }
            HF_CUDA(read_status(ctx, s));
            if (ctx->st_host->flags) {
                if (bad_cell) *bad_cell = (int64_t)ctx->st_host->bad_cell;
                return fail(ctx, HF_ERR_COMBINE, "flux_update: inadmissible Heun combination");
            }
        }
        return HF_OK;
    }
    if (f & ST_COMBINE_BAD) return fail(ctx, HF_ERR_COMBINE, "flux_update: inadmissible Heun combination");
    return HF_OK;
}

hf_status hf_flux_adjoint(hf_ctx* ctx, const hf_level* level, const hf_patch* patch, const double* U,
                          const double* Ubar_out, double h, int first_order, double* Ubar_in, void* stream) {
    if (!ctx || !level || !patch || !U || !Ubar_out || !Ubar_in || !level_ok(*level) || !patch_ok(*patch) || !(h > 0))
        return fail(ctx, HF_ERR_ARG, "flux_adjoint: bad arguments");
    const hf_patch& P = *patch;
    if (P.ilo != 0 || P.jlo != 0 || P.nx != level->nx || P.ny != level->ny || P.ng != 2)
        return fail(ctx, HF_ERR_ARG, "flux_adjoint: one domain-covering patch with 2 ghost layers");
    for (int d = 0; d < 2; ++d)
        if (level->bc_lo[d] == HF_BC_WEDGE || level->bc_hi[d] == HF_BC_WEDGE)
            return fail(ctx, HF_ERR_ARG, "flux_adjoint: no wedge boundary");
    const int nv = ctx->ns + 3;
    const size_t nfa = 4 * (size_t)nv * (P.nx + 1) * P.ny, nfb = 4 * (size_t)nv * P.nx * (P.ny + 1);
    const size_t nug = (size_t)P.offset + (size_t)nv * P.comp_stride;
    double* w = static_cast<double*>(scratch(ctx, sizeof(double) * (nfa + nfb + nug)));
    if (!w) return fail(ctx, HF_ERR_CUDA, "flux_adjoint: scratch allocation failed");
    const cudaStream_t s = S(stream);
    HF_CUDA(reset_status(ctx, s));
    HF_CUDA(launch_stage_adjoint(ctx->ns, make_level(*level), P, U, Ubar_out, 1.0, h, first_order ? 1 : 0, w, w + nfa,
                                 w + nfa + nfb, Ubar_in, ctx->st, s, &ctx->cnt.kernel_launches));
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags & ST_FACE_BAD) return fail(ctx, HF_ERR_FACE, "flux_adjoint: inadmissible face state");
    return HF_OK;
}

static hf_status chem_common(hf_ctx* ctx, double* U, int64_t comp_stride, const int64_t* cell_index, int64_t count,
                             double dt, const double* dt_cell, double rtol, double atol, int form,
                             const hf_chem_history* hist, int64_t* first_failed, void* stream) {
    if (first_failed) *first_failed = -1;
    if (!ctx || (!U && count > 0) || count < 0 || count > INT32_MAX || (!cell_index && comp_stride < count) ||
        (!dt_cell && (!(dt > 0) || !std::isfinite(dt))) || !(rtol > 0) || !(atol > 0) ||
        (form != HF_CHEM_PLAIN && form != HF_CHEM_PERSISTENT && form != 2))
        return fail(ctx, HF_ERR_ARG, "chem_advance: invalid batch extent, interval or tolerances");
    if (count == 0) return HF_OK;
    const cudaStream_t s = S(stream);
    const int nv = ctx->ns + 3;
    // scratch: trial states | fail codes | queue order | bucket offsets
    const size_t b_trial = sizeof(double) * (size_t)nv * count;
    const size_t b_fail = (sizeof(int) * (size_t)count + 15) & ~size_t(15);
    const size_t b_order = (sizeof(int32_t) * (size_t)count + 15) & ~size_t(15);
    char* w = static_cast<char*>(scratch(ctx, b_trial + b_fail + b_order + CHEM_BINS * sizeof(unsigned long long)));
    if (!w) return fail(ctx, HF_ERR_CUDA, "chem_advance: scratch allocation failed");
    double* trial = reinterpret_cast<double*>(w);
    int* failv = reinterpret_cast<int*>(w + b_trial);
    int32_t* order = reinterpret_cast<int32_t*>(w + b_trial + b_fail);
    unsigned long long* bins = reinterpret_cast<unsigned long long*>(w + b_trial + b_fail + b_order);
    HF_CUDA(reset_status(ctx, s));
    tic(ctx, 1, s);
    const int64_t l0 = ctx->cnt.kernel_launches;
    if (form == 2)
        HF_CUDA(launch_chem_batched(ctx->ns, U, comp_stride, cell_index, count, dt, nullptr, dt_cell, rtol, atol,
                                    hist ? hist->h : nullptr, hist ? hist->cost : nullptr, order, bins, trial, failv,
                                    ctx->st, ctx->sm_count, s, &ctx->cnt.kernel_launches));
    else
        HF_CUDA(launch_chem(ctx->ns, form, U, comp_stride, cell_index, count, dt, dt_cell, rtol, atol, trial, failv,
                            ctx->st, ctx->sm_count, s, &ctx->cnt.kernel_launches));
    toc(ctx, s, ctx->cnt.kernel_launches - l0);
    HF_CUDA(read_status(ctx, s));
    ctx->cnt.chem_steps += (int64_t)ctx->st_host->steps;
    ctx->cnt.chem_coop_cells += (int64_t)ctx->st_host->coop_cells;
    const unsigned f = ctx->st_host->flags;
    if (f & (ST_CHEM_FAIL | ST_MAXSTEPS)) {
        if (first_failed) *first_failed = (int64_t)ctx->st_host->bad_cell;
        char msg[96];
        snprintf(msg, sizeof msg, "chemistry cell %lld: %s", (long long)ctx->st_host->bad_cell,
                 (f & ST_MAXSTEPS) && !(f & ST_CHEM_FAIL) ? "step limit" : "integration failed");
        return fail(ctx, (f & ST_CHEM_FAIL) ? HF_ERR_CHEM_FAIL : HF_ERR_MAXSTEPS, msg);
    }
    HF_CUDA(launch_chem_commit(ctx->ns, U, comp_stride, cell_index, count, trial, s, &ctx->cnt.kernel_launches));
    ctx->cnt.chem_cell_calls += count;
    return HF_OK;
}

hf_status hf_chem_advance(hf_ctx* ctx, double* U, int64_t comp_stride, const int64_t* cell_index, int64_t count,
                          double dt, const double* dt_cell, double rtol, double atol, int form, int64_t* first_failed,
                          void* stream) {
    if (form != HF_CHEM_PLAIN && form != HF_CHEM_PERSISTENT) {
        if (first_failed) *first_failed = -1;
        return fail(ctx, HF_ERR_ARG, "chem_advance: unknown form");
    }
    return chem_common(ctx, U, comp_stride, cell_index, count, dt, dt_cell, rtol, atol, form, nullptr, first_failed,
                       stream);
}

hf_status hf_chem_advance_batched(hf_ctx* ctx, double* U, int64_t comp_stride, const int64_t* cell_index,
                                  int64_t count, double dt, const double* dt_cell, double rtol, double atol,
                                  const hf_chem_history* history, int64_t* first_failed, void* stream) {
    return chem_common(ctx, U, comp_stride, cell_index, count, dt, dt_cell, rtol, atol, 2, history, first_failed,
                       stream);
}

// Objective (backward = false) or objective + discrete adjoint of 0D chemistry runs.
// The checkpoint / segment / tape scratch is taken from the stream-ordered allocator
// for the call only, in chunks of cells that fit half the free device memory (16 GiB
// at most).
static hf_status chem_sensitivity(hf_ctx* ctx, const double* U0, int64_t comp_stride, int64_t count, double dt,
                                  int32_t ncalls, const hf_adjoint_opts* o, double* J, double* dJdp, double* dJdy0,
                                  int64_t* first_failed, void* stream, bool backward) {
    if (first_failed) *first_failed = -1;
    if (!ctx || !U0 || !J || !o || count < 0 || count > INT32_MAX || comp_stride < count || !(dt > 0) ||
        !std::isfinite(dt) || ncalls < 1 || o->objective < HF_OBJ_IGNITION_DELAY || o->objective > HF_OBJ_FINAL_T ||
        o->checkpoint_every < 1 || !(o->rtol > 0) || !(o->atol > 0) || !std::isfinite(o->ignition_dT) ||
        (backward && !dJdp))
        return fail(ctx, HF_ERR_ARG, "chem_adjoint: invalid batch extent, interval, options or outputs");
    if (count == 0) return HF_OK;
    const cudaStream_t s = S(stream);
    const int ns = ctx->ns, nv = ns + 3;
    AdjointArgs a{};
    a.U0 = U0;
    a.cs = comp_stride;
    a.count = count;
    a.dt = dt;
    a.dT = o->ignition_dT;
    a.rtol = o->rtol;
    a.atol = o->atol;
    a.ncalls = ncalls;
    a.K = o->checkpoint_every < ncalls ? o->checkpoint_every : ncalls;
    a.objective = o->objective;
    a.cap = 5000;  // >= the accepted-step limit of one call
    a.backward = backward ? 1 : 0;
    a.J = J;
    a.dJdp = dJdp;
    a.dJdy0 = dJdy0;
    int* failv = static_cast<int*>(scratch(ctx, sizeof(int) * (size_t)count));
    if (!failv) return fail(ctx, HF_ERR_CUDA, "chem_adjoint: scratch allocation failed");
    a.fail = failv;
    a.st = ctx->st;
    int64_t chunk = count;
    size_t per = 0;
    if (backward) {
        per = adjoint_bytes_per_cell(ns, ncalls, a.K, a.cap);
        size_t fr = 0, tot = 0;
        HF_CUDA(cudaMemGetInfo(&fr, &tot));
        size_t budget = fr / 2;
        if (budget > (size_t(16) << 30)) budget = size_t(16) << 30;
        chunk = (int64_t)(budget / per);
        if (chunk < 1) return fail(ctx, HF_ERR_CUDA, "chem_adjoint: not enough device memory for one cell");
        if (chunk > count) chunk = count;
    }
    char* w = nullptr;
    if (backward) {
        const size_t bytes = per * (size_t)chunk + 1024;
        HF_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&w), bytes, s));
        const int nck = (ncalls + a.K - 1) / a.K;
        size_t off = 0;
        auto take = [&](size_t b) { char* p = w + off; off += (b + 255) & ~size_t(255); return p; };
        a.ckpt = reinterpret_cast<double*>(take(sizeof(double) * (size_t)nck * nv * chunk));
        a.seg = reinterpret_cast<double*>(take(sizeof(double) * (size_t)(a.K + 1) * nv * chunk));
        a.tape = reinterpret_cast<double*>(take(sizeof(double) * (size_t)a.cap * (ns + 1) * chunk));
        a.nstep = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * (size_t)a.K * chunk));
        a.clipm = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)a.K * chunk));
    }
    hf_status rc = HF_OK;
    cudaError_t e = reset_status(ctx, s);
    tic(ctx, 1, s);
    const int64_t l0 = ctx->cnt.kernel_launches;
    for (int64_t i0 = 0; e == cudaSuccess && i0 < count; i0 += chunk) {
        a.i0 = i0;
        a.chunk = count - i0 < chunk ? count - i0 : chunk;
        e = launch_chem_adjoint(ns, a, s, &ctx->cnt.kernel_launches);
    }
    toc(ctx, s, ctx->cnt.kernel_launches - l0);
    if (w) {
        const cudaError_t e2 = cudaFreeAsync(w, s);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "chem_adjoint launch");
    HF_CUDA(read_status(ctx, s));
    ctx->cnt.chem_steps += (int64_t)ctx->st_host->steps;
    ctx->cnt.chem_coop_cells += (int64_t)ctx->st_host->coop_cells;
    const unsigned f = ctx->st_host->flags;
    if (f & (ST_CHEM_FAIL | ST_MAXSTEPS)) {
        if (first_failed) *first_failed = (int64_t)ctx->st_host->bad_cell;
        char msg[96];
        snprintf(msg, sizeof msg, "chemistry cell %lld: %s", (long long)ctx->st_host->bad_cell,
                 (f & ST_MAXSTEPS) && !(f & ST_CHEM_FAIL) ? "step limit" : "integration failed");
        rc = fail(ctx, (f & ST_CHEM_FAIL) ? HF_ERR_CHEM_FAIL : HF_ERR_MAXSTEPS, msg);
    }
    return rc;
}

hf_status hf_chem_objective(hf_ctx* ctx, const double* U0, int64_t comp_stride, int64_t count, double dt,
                            int32_t ncalls, const hf_adjoint_opts* opts, double* objective, int64_t* first_failed,
                            void* stream) {
    return chem_sensitivity(ctx, U0, comp_stride, count, dt, ncalls, opts, objective, nullptr, nullptr, first_failed,
                            stream, false);
}

hf_status hf_chem_adjoint(hf_ctx* ctx, const double* U0, int64_t comp_stride, int64_t count, double dt,
                          int32_t ncalls, const hf_adjoint_opts* opts, double* objective, double* dJ_dlnA,
                          double* dJ_dY0, int64_t* first_failed, void* stream) {
    return chem_sensitivity(ctx, U0, comp_stride, count, dt, ncalls, opts, objective, dJ_dlnA, dJ_dY0, first_failed,
                            stream, true);
}

hf_status hf_cfl_dt(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, const double* U, double cfl,
                    double* dt, void* stream) {
    if (!ctx || !level || !patches || npatch <= 0 || !U || !dt || !(cfl > 0) || !level_ok(*level))
        return fail(ctx, HF_ERR_ARG, "cfl_dt: bad arguments");
    for (int p = 0; p < npatch; ++p)
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "cfl_dt: bad patch");
    const cudaStream_t s = S(stream);
    const Level L = make_level(*level);
    std::vector<int64_t> base;
    if (npatch > 1) {  // every patch in one launch
        base.resize(npatch);
        int64_t b = 0;
        for (int p = 0; p < npatch; ++p) {
            base[p] = b;
            b += (int64_t)patches[p].nx * patches[p].ny;
        }
        HF_CUDA(upload_patches(ctx, patches, npatch, s));
        HF_CUDA(upload_offsets(ctx, base.data(), npatch, s));
    }
    HF_CUDA(reset_status(ctx, s));
    tic(ctx, 2, s);
    if (npatch == 1)
        HF_CUDA(launch_cfl(ctx->ns, L, patches[0], U, ctx->st, s, &ctx->cnt.kernel_launches));
    else
        HF_CUDA(launch_cfl_multi(ctx->ns, L, patches, ctx->d_patches, npatch, ctx->d_off, U, ctx->st, s,
                                 &ctx->cnt.kernel_launches));
    toc(ctx, s, 1);
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags) return fail(ctx, HF_ERR_INADMISSIBLE, "cfl_dt: inadmissible cell");
    double rate;
    memcpy(&rate, &ctx->st_host->rate_bits, sizeof rate);
    *dt = cfl / rate;
    return HF_OK;
}

hf_status hf_validate(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, const double* U,
                      int64_t* bad_cell, void* stream) {
    if (bad_cell) *bad_cell = -1;
    if (!ctx || !level || !patches || npatch <= 0 || !U) return fail(ctx, HF_ERR_ARG, "validate: bad arguments");
    for (int p = 0; p < npatch; ++p)
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "validate: bad patch");
    const cudaStream_t s = S(stream);
    std::vector<int64_t> base(npatch);
    int64_t b = 0;
    for (int p = 0; p < npatch; ++p) {
        base[p] = b;
        b += (int64_t)patches[p].nx * patches[p].ny;
    }
    if (npatch > 1) {  // every patch in one launch
        HF_CUDA(upload_patches(ctx, patches, npatch, s));
        HF_CUDA(upload_offsets(ctx, base.data(), npatch, s));
    }
    HF_CUDA(reset_status(ctx, s));
    tic(ctx, 2, s);
    if (npatch == 1)
        HF_CUDA(launch_validate(ctx->ns, patches[0], U, 0, ctx->st, s, &ctx->cnt.kernel_launches));
    else
        HF_CUDA(launch_validate_multi(ctx->ns, patches, ctx->d_patches, npatch, ctx->d_off, U, ctx->st, s,
                                      &ctx->cnt.kernel_launches));
    toc(ctx, s, 1);
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags) {
        if (bad_cell) *bad_cell = (int64_t)ctx->st_host->bad_cell;
        return fail(ctx, HF_ERR_INADMISSIBLE, "validate: inadmissible cell");
    }
    return HF_OK;
}


// ---------------------------------------------------------------- block-AMR operations
static char* aux_scratch(hf_ctx* ctx, size_t bytes) {
    if (bytes > ctx->aux_bytes) {
        if (ctx->aux) cudaFree(ctx->aux);
        ctx->aux = nullptr;
        ctx->aux_bytes = 0;
        if (cudaMalloc(&ctx->aux, bytes) != cudaSuccess) return nullptr;
        ctx->aux_bytes = bytes;
    }
    return static_cast<char*>(ctx->aux);
}
static size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

hf_status hf_totals(hf_ctx* ctx, const hf_patch* patches, int npatch, const double* U, const uint8_t* leaf_mask,
                    double cell_volume, int absolute, double* out, void* stream) {
    if (!ctx || !patches || npatch <= 0 || !U || !out) return fail(ctx, HF_ERR_ARG, "totals: bad arguments");
    int64_t total = 0;
    for (int p = 0; p < npatch; ++p) {
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "totals: bad patch");
        total += (int64_t)patches[p].nx * patches[p].ny;
    }
    const int nv = ctx->ns + 3;
    const cudaStream_t s = S(stream);
    const size_t bp = align16(sizeof(hf_patch) * npatch), bt = align16(totals_scratch_bytes(nv));
    char* w = aux_scratch(ctx, bp + bt + sizeof(double) * 16);
    if (!w) return fail(ctx, HF_ERR_CUDA, "totals: scratch allocation failed");
    HF_CUDA(cudaMemcpyAsync(w, patches, sizeof(hf_patch) * npatch, cudaMemcpyHostToDevice, s));
    double* out_dev = reinterpret_cast<double*>(w + bp + bt);
    HF_CUDA(launch_totals(reinterpret_cast<hf_patch*>(w), npatch, total, U, leaf_mask, nv, cell_volume, absolute,
                          w + bp, out_dev, s, &ctx->cnt.kernel_launches));
    HF_CUDA(cudaMemcpyAsync(out, out_dev, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
    HF_CUDA(cudaStreamSynchronize(s));
    return HF_OK;
}

hf_status hf_average_down(hf_ctx* ctx, const hf_patch* fine, int nfine, const double* Uf, const hf_patch* coarse,
                          int ncoarse, double* Uc, void* stream) {
    if (!ctx || !fine || nfine <= 0 || !Uf || !coarse || ncoarse <= 0 || !Uc)
        return fail(ctx, HF_ERR_ARG, "average_down: bad arguments");
    for (int p = 0; p < nfine; ++p)
        if (!patch_ok(fine[p]) || (fine[p].ilo & 1) || (fine[p].jlo & 1) || (fine[p].nx & 1) || (fine[p].ny & 1))
            return fail(ctx, HF_ERR_ARG, "average_down: fine patches must be aligned to the ratio 2");
    for (int p = 0; p < ncoarse; ++p)
        if (!patch_ok(coarse[p])) return fail(ctx, HF_ERR_ARG, "average_down: bad coarse patch");
    const cudaStream_t s = S(stream);
    const size_t bf = align16(sizeof(hf_patch) * nfine), bc = align16(sizeof(hf_patch) * ncoarse);
    char* w = aux_scratch(ctx, bf + bc);
    if (!w) return fail(ctx, HF_ERR_CUDA, "average_down: scratch allocation failed");
    HF_CUDA(cudaMemcpyAsync(w, fine, sizeof(hf_patch) * nfine, cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(w + bf, coarse, sizeof(hf_patch) * ncoarse, cudaMemcpyHostToDevice, s));
    HF_CUDA(launch_average_down(reinterpret_cast<hf_patch*>(w), fine, nfine, Uf, reinterpret_cast<hf_patch*>(w + bf),
                                ncoarse, Uc, ctx->ns + 3, s, &ctx->cnt.kernel_launches));
    HF_CUDA(cudaStreamSynchronize(s));  // the tables live in scratch until the kernel is done
    return HF_OK;
}

hf_status hf_reflux(hf_ctx* ctx, const hf_level* coarse_level, const hf_patch* coarse, int ncoarse, double* Uc,
                    const double* fxc, const double* fyc, const hf_patch* fine, int nfine, const double* fxf,
                    const double* fyf, double h, void* stream) {
    if (!ctx || !coarse_level || !level_ok(*coarse_level) || !coarse || ncoarse <= 0 || !Uc || !fxc || !fyc ||
        !fine || nfine <= 0 || !fxf || !fyf || !(h > 0))
        return fail(ctx, HF_ERR_ARG, "reflux: bad arguments");
    const int nv = ctx->ns + 3;
    std::vector<int64_t> off(2 * (ncoarse + nfine));
    int64_t ox = 0, oy = 0;
    for (int p = 0; p < ncoarse; ++p) {
        const hf_patch& C = coarse[p];
        if (!patch_ok(C) || C.ilo < 0 || C.jlo < 0 || C.ilo + C.nx > coarse_level->nx || C.jlo + C.ny > coarse_level->ny)
            return fail(ctx, HF_ERR_ARG, "reflux: coarse patch outside the level");
        off[p] = ox;
        off[ncoarse + p] = oy;
        ox += (int64_t)nv * (C.nx + 1) * C.ny;
        oy += (int64_t)nv * C.nx * (C.ny + 1);
    }
    ox = oy = 0;
    for (int p = 0; p < nfine; ++p) {
        const hf_patch& F = fine[p];
        if (!patch_ok(F) || (F.ilo & 1) || (F.jlo & 1) || (F.nx & 1) || (F.ny & 1) || F.ilo < 0 || F.jlo < 0 ||
            F.ilo + F.nx > 2 * coarse_level->nx || F.jlo + F.ny > 2 * coarse_level->ny)
            return fail(ctx, HF_ERR_ARG, "reflux: fine patches must be aligned to the ratio 2 inside the level");
        off[2 * ncoarse + p] = ox;
        off[2 * ncoarse + nfine + p] = oy;
        ox += (int64_t)nv * (F.nx + 1) * F.ny;
        oy += (int64_t)nv * F.nx * (F.ny + 1);
    }
    const cudaStream_t s = S(stream);
    const size_t bc = align16(sizeof(hf_patch) * ncoarse), bf = align16(sizeof(hf_patch) * nfine);
    const size_t bo = align16(sizeof(int64_t) * off.size());
    const size_t bm = sizeof(int) * (size_t)coarse_level->nx * coarse_level->ny;
    char* w = aux_scratch(ctx, bc + bf + bo + bm);
    if (!w) return fail(ctx, HF_ERR_CUDA, "reflux: scratch allocation failed");
    HF_CUDA(cudaMemcpyAsync(w, coarse, sizeof(hf_patch) * ncoarse, cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(w + bc, fine, sizeof(hf_patch) * nfine, cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(w + bc + bf, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, s));
    const int64_t* o = reinterpret_cast<const int64_t*>(w + bc + bf);
    HF_CUDA(launch_reflux(make_level(*coarse_level), reinterpret_cast<hf_patch*>(w), coarse, ncoarse, o, o + ncoarse,
                          fxc, fyc, Uc, reinterpret_cast<hf_patch*>(w + bc), fine, nfine, o + 2 * ncoarse,
                          o + 2 * ncoarse + nfine, fxf, fyf, reinterpret_cast<int*>(w + bc + bf + bo), h, nv, s,
                          &ctx->cnt.kernel_launches));
    HF_CUDA(cudaStreamSynchronize(s));  // pageable offset table and scratch stay valid until here
    return HF_OK;
}

hf_status hf_tag_cells(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch, const double* U,
                       double time, const hf_tag_criteria* criteria, uint8_t* tags, void* stream) {
    if (!ctx || !level || !level_ok(*level) || !patches || npatch <= 0 || !U || !criteria || !tags)
        return fail(ctx, HF_ERR_ARG, "tag_cells: bad arguments");
    std::vector<int64_t> off(npatch);
    int64_t o = 0;
    for (int p = 0; p < npatch; ++p) {
        if (!patch_ok(patches[p])) return fail(ctx, HF_ERR_ARG, "tag_cells: bad patch");
        off[p] = o;
        o += (int64_t)patches[p].nx * patches[p].ny;
    }
    const cudaStream_t s = S(stream);
    const size_t bp = align16(sizeof(hf_patch) * npatch);
    char* w = aux_scratch(ctx, bp + sizeof(int64_t) * npatch);
    if (!w) return fail(ctx, HF_ERR_CUDA, "tag_cells: scratch allocation failed");
    HF_CUDA(cudaMemcpyAsync(w, patches, sizeof(hf_patch) * npatch, cudaMemcpyHostToDevice, s));
    HF_CUDA(cudaMemcpyAsync(w + bp, off.data(), sizeof(int64_t) * npatch, cudaMemcpyHostToDevice, s));
    HF_CUDA(reset_status(ctx, s));
    HF_CUDA(launch_tag(ctx->ns, make_level(*level), reinterpret_cast<hf_patch*>(w), patches, npatch, U, time, *criteria,
                       tags, reinterpret_cast<int64_t*>(w + bp), ctx->st, s, &ctx->cnt.kernel_launches));
    HF_CUDA(read_status(ctx, s));
    if (ctx->st_host->flags) return fail(ctx, HF_ERR_INADMISSIBLE, "tag_cells: inadmissible cell on a stencil");
    return HF_OK;
}

// FP64 roofline probe: independent FMA chains, 8 per thread, on every SM.
static __global__ void __launch_bounds__(256) k_fp64_peak(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1e-3 * threadIdx.x + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == -1.0) out[blockIdx.x] = s;  // never true; keeps the chains live
}

hf_status hf_fp64_peak(hf_ctx* ctx, double* gflops, void* stream) {
    if (!ctx || !gflops) return fail(ctx, HF_ERR_ARG, "fp64_peak: bad arguments");
    const cudaStream_t s = S(stream);
    double* out = static_cast<double*>(scratch(ctx, sizeof(double) * 4096));
    if (!out) return fail(ctx, HF_ERR_CUDA, "fp64_peak: scratch allocation failed");
    cudaEvent_t e0, e1;
    HF_CUDA(cudaEventCreate(&e0));
    HF_CUDA(cudaEventCreate(&e1));
    const int blocks = ctx->sm_count * 8, threads = 256, iters = 8192;
    float best = 1e30f;
    cudaError_t e = cudaSuccess;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        k_fp64_peak<<<blocks, threads, 0, s>>>(out, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && t < best) best = t;  // the first launch is a warm-up
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fp64_peak");
    ctx->cnt.kernel_launches += 4;
    *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
    return HF_OK;
}

}  // extern "C"
