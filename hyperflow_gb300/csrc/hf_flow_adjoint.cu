// Discrete adjoint of a run of Strang steps on a one-patch level (a build-defined
// extension: the reference has no sensitivity code).
//
// hf_flow_record replays the loop of BlockAMR::run (HyperFlow_V3/src/BlockAMR.cpp:
// 409-419) with the plain forms (filled ghosts + face/update kernels, one thread per
// cell chemistry): per step flow(dt/2), react(dt), flow(dt/2), each Euler stage
// redone first order when its second-order output is inadmissible (:257-263).  It
// records the step sizes, the first-order flags and the state every K steps.
//
// hf_flow_adjoint runs the reverse sweep from a cotangent of the final state: per
// segment of K steps it recomputes the step-start states from the checkpoint, then
// for each step, last first, recomputes the step's intermediates
//     A1 = E(S0), X = (S0 + E(A1))/2, C = react(X), A2 = E(C), S2 = (C + E(A2))/2
// and applies the transposes of the four stages and of the chemistry calls.  The
// step sizes and every branch of the forward are held fixed (the frozen map);
// roundoff repairs are taken as the identity.
#include <cuda_runtime.h>
#include <cstring>
#include <vector>
#include "hf_internal.h"
#include "mech_h2li.h"

struct hf_flow_tape {
    hf_ctx* ctx = nullptr;
    hf_level L{};
    hf_patch P{};
    int ns = 9, nv = 12;
    int nsteps = 0, K = 1;
    int chemistry = 1;
    double rtol = 1e-8, atol = 1e-15;
    size_t bytes = 0;                 // one ghosted state
    std::vector<double> dts;
    std::vector<unsigned char> fo;    // first-order flag of each stage, 4 per step
    std::vector<double*> ck;          // state at steps 0, K, 2K, ...
    int64_t* cells = nullptr;         // interior gather list (chemistry)
};

namespace {

using hf::DevStatus;

constexpr int TAPE_CAP = 5000;  // >= the accepted-step limit of one chemistry call

__global__ void k_lincomb(hf_patch P, int nv, double a, const double* __restrict__ x, double b,
                          const double* __restrict__ y, double* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
    for (int n = 0; n < nv; ++n) {
        const int64_t k = g + n * P.comp_stride;
        out[k] = a * x[k] + (y ? b * y[k] : 0.0);
    }
}

// out[r] = sum over cells of pcell[r][cell], a fixed-order tree per row.
__global__ void k_sum_rows(const double* __restrict__ pcell, int64_t n, double* __restrict__ out) {
    __shared__ double sh[256];
    const double* row = pcell + (int64_t)blockIdx.x * n;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += row[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

hf_status cuda_status(cudaError_t e) { return e == cudaSuccess ? HF_OK : HF_ERR_CUDA; }

hf_status copy_interior(const hf_flow_tape* t, double* dst_ghosted, const double* src_soa, cudaStream_t s,
                        bool in) {
    const hf_patch& P = t->P;
    const int64_t nc = (int64_t)P.nx * P.ny;
    for (int n = 0; n < t->nv; ++n) {
        double* g = dst_ghosted + n * P.comp_stride + P.ng * P.pitch + P.ng;
        cudaError_t e = in ? cudaMemcpy2DAsync(g, P.pitch * sizeof(double), src_soa + (size_t)n * nc,
                                               P.nx * sizeof(double), P.nx * sizeof(double), P.ny,
                                               cudaMemcpyDeviceToDevice, s)
                           : cudaMemcpy2DAsync(const_cast<double*>(src_soa) + (size_t)n * nc, P.nx * sizeof(double),
                                               g, P.pitch * sizeof(double), P.nx * sizeof(double), P.ny,
                                               cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return HF_ERR_CUDA;
    }
    return HF_OK;
}

// One Euler stage out = E(in) (old: Heun with old) with filled ghosts; fo in/out:
// replay uses the recorded flag, otherwise the stage is redone first order when its
// second-order output is inadmissible.
hf_status stage_fwd(hf_flow_tape* t, double* in, const double* old, double* out, double h, unsigned char& fo,
                    bool replay, cudaStream_t s) {
    hf_status r = hf_fill_ghosts(t->ctx, &t->L, &t->P, 1, in, s);
    if (r != HF_OK) return r;
    int64_t bad = -1;
    if (replay) return hf_flux_update(t->ctx, &t->L, &t->P, 1, in, old, out, nullptr, nullptr, h, fo, HF_FLUX_PLAIN,
                                      &bad, s);
    for (int f = 0; f < 2; ++f) {
        r = hf_flux_update(t->ctx, &t->L, &t->P, 1, in, old, out, nullptr, nullptr, h, f, HF_FLUX_PLAIN, &bad, s);
        if (r == HF_OK) {
            fo = (unsigned char)f;
            return HF_OK;
        }
        if (r != HF_ERR_INADMISSIBLE && r != HF_ERR_NEGATIVE) return r;
    }
    return HF_ERR_INADMISSIBLE;
}

// Strang step n from S0; the intermediates go to w[0..3] = A1, X, C, A2 and the
// result to S2.
hf_status step_fwd(hf_flow_tape* t, int n, double* S0, double* const* w, double* S2, bool replay, cudaStream_t s) {
    const double h = t->dts[n], hh = 0.5 * h;
    unsigned char* fo = &t->fo[(size_t)4 * n];
    double *A1 = w[0], *X = w[1], *C = w[2], *A2 = w[3];
    hf_status r = stage_fwd(t, S0, nullptr, A1, hh, fo[0], replay, s);
    if (r == HF_OK) r = stage_fwd(t, A1, S0, X, hh, fo[1], replay, s);
    if (r != HF_OK) return r;
    if (cudaMemcpyAsync(C, X, t->bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return HF_ERR_CUDA;
    if (t->chemistry) {
        int64_t first = -1;
        r = hf_chem_advance(t->ctx, C, t->P.comp_stride, t->cells, (int64_t)t->P.nx * t->P.ny, h, nullptr, t->rtol,
                            t->atol, HF_CHEM_PLAIN, &first, s);
        if (r != HF_OK) return r;
    }
    r = stage_fwd(t, C, nullptr, A2, hh, fo[2], replay, s);
    if (r == HF_OK && S2) r = stage_fwd(t, A2, C, S2, hh, fo[3], replay, s);
    if (r == HF_OK && !S2) r = hf_fill_ghosts(t->ctx, &t->L, &t->P, 1, A2, s);  // A2's ghosts for the reverse
    return r;
}

struct Bufs {
    std::vector<double*> all;
    double* get(size_t bytes, cudaStream_t s) {
        void* p = nullptr;
        if (cudaMallocAsync(&p, bytes, s) != cudaSuccess) return nullptr;
        if (cudaMemsetAsync(p, 0, bytes, s) != cudaSuccess) return nullptr;
        all.push_back(static_cast<double*>(p));
        return static_cast<double*>(p);
    }
    void release(cudaStream_t s) {
        for (double* p : all) cudaFreeAsync(p, s);
        all.clear();
    }
};

}  // namespace

extern "C" {

hf_status hf_flow_record(hf_ctx* ctx, const hf_level* level, const double* U0, int32_t nsteps, const double* dts,
                         double cfl, int32_t checkpoint_every, int chemistry, double rtol, double atol,
                         double* U_final, double* dts_out, hf_flow_tape** out, void* stream) {
    if (out) *out = nullptr;
    if (!ctx || !level || !U0 || !out || nsteps < 1 || checkpoint_every < 1 || (!dts && !(cfl > 0)) ||
        !(rtol > 0) || !(atol > 0) || level->nx <= 0 || level->ny <= 0 || level->bc_lo[1] == HF_BC_WEDGE)
        return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    hf_flow_tape* t = new hf_flow_tape();
    t->ctx = ctx;
    t->L = *level;
    t->ns = hf_nspecies(ctx);
    t->nv = t->ns + 3;
    t->nsteps = nsteps;
    t->K = checkpoint_every < nsteps ? checkpoint_every : nsteps;
    t->chemistry = chemistry;
    t->rtol = rtol;
    t->atol = atol;
    hf_patch& P = t->P;
    P.ilo = P.jlo = 0;
    P.nx = level->nx;
    P.ny = level->ny;
    P.ng = 2;
    P.pitch = (P.nx + 2 * P.ng + 1) & ~int64_t(1);
    P.comp_stride = (P.pitch * (P.ny + 2 * P.ng) + 31) & ~int64_t(31);
    P.offset = 0;
    t->bytes = sizeof(double) * (size_t)P.comp_stride * t->nv;
    t->dts.assign(nsteps, 0.0);
    if (dts) std::memcpy(t->dts.data(), dts, sizeof(double) * nsteps);
    t->fo.assign((size_t)4 * nsteps, 0);
    const int64_t nc = (int64_t)P.nx * P.ny;
    bool ok = cudaMalloc(&t->cells, sizeof(int64_t) * nc) == cudaSuccess;
    if (ok) {
        std::vector<int64_t> idx(nc);
        for (int64_t j = 0; j < P.ny; ++j)
            for (int64_t i = 0; i < P.nx; ++i) idx[j * P.nx + i] = (j + P.ng) * P.pitch + (i + P.ng);
        ok = cudaMemcpy(t->cells, idx.data(), sizeof(int64_t) * nc, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    const int nck = (nsteps + t->K - 1) / t->K;
    for (int k = 0; ok && k < nck; ++k) {
        double* p = nullptr;
        ok = cudaMalloc(&p, t->bytes) == cudaSuccess && cudaMemset(p, 0, t->bytes) == cudaSuccess;
        t->ck.push_back(p);
    }
    if (!ok) {
        hf_flow_tape_destroy(t);
        return HF_ERR_CUDA;
    }
    Bufs b;
    double* w[4];
    double *cur = b.get(t->bytes, s), *nxt = b.get(t->bytes, s);
    for (int k = 0; k < 4; ++k) w[k] = b.get(t->bytes, s);
    hf_status r = (cur && nxt && w[0] && w[1] && w[2] && w[3]) ? copy_interior(t, cur, U0, s, true) : HF_ERR_CUDA;
    for (int n = 0; r == HF_OK && n < nsteps; ++n) {
        if (n % t->K == 0) r = cuda_status(cudaMemcpyAsync(t->ck[n / t->K], cur, t->bytes, cudaMemcpyDeviceToDevice, s));
        if (r == HF_OK && !dts) r = hf_cfl_dt(ctx, &t->L, &t->P, 1, cur, cfl, &t->dts[n], s);
        if (r == HF_OK) r = step_fwd(t, n, cur, w, nxt, false, s);
        std::swap(cur, nxt);
    }
    if (r == HF_OK && U_final) r = copy_interior(t, cur, U_final, s, false);
    if (r == HF_OK && dts_out) std::memcpy(dts_out, t->dts.data(), sizeof(double) * nsteps);
    b.release(s);
    if (r == HF_OK) r = cuda_status(cudaStreamSynchronize(s));
    if (r != HF_OK) {
        hf_flow_tape_destroy(t);
        return r;
    }
    *out = t;
    return HF_OK;
}

hf_status hf_flow_adjoint(hf_flow_tape* t, const double* seed, double* U0_bar, double* dJ_dlnA, void* stream) {
    if (!t || !seed) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const hf_patch& P = t->P;
    const hf::Level L = hf::make_level(t->L);
    const int64_t nc = (int64_t)P.nx * P.ny;
    const int64_t nfx = (int64_t)(P.nx + 1) * P.ny, nfy = (int64_t)P.nx * (P.ny + 1);
    int64_t chunk = (int64_t)((size_t(4) << 30) / (sizeof(double) * (size_t)TAPE_CAP * (t->ns + 1)));
    if (chunk > nc) chunk = nc;
    if (chunk < 1) chunk = 1;
    Bufs b;
    std::vector<double*> seg(t->K + 1);
    for (auto& p : seg) p = b.get(t->bytes, s);
    // the intermediates of every step of a segment are kept when 4K states fit in a
    // quarter of the free memory (one forward recomputation in all); otherwise each
    // step's intermediates are recomputed from its start state before its transpose
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const bool keep = (size_t)4 * t->K * t->bytes <= fr / 4;
    std::vector<double*> inter((size_t)4 * (keep ? t->K : 1));
    for (auto& p : inter) p = b.get(t->bytes, s);
    double *ub = b.get(t->bytes, s), *t1 = b.get(t->bytes, s), *t2 = b.get(t->bytes, s);
    double *cC = b.get(t->bytes, s), *cX = b.get(t->bytes, s), *UG = b.get(t->bytes, s);
    double* FAx = b.get(sizeof(double) * 4 * t->nv * nfx, s);
    double* FAy = b.get(sizeof(double) * 4 * t->nv * nfy, s);
    double* tape = t->chemistry ? b.get(sizeof(double) * (size_t)TAPE_CAP * (t->ns + 1) * chunk, s) : nullptr;
    double* pcell = b.get(sizeof(double) * hfmech::NR * nc, s);
    double* psum = b.get(sizeof(double) * hfmech::NR, s);
    DevStatus* dst = reinterpret_cast<DevStatus*>(b.get(sizeof(DevStatus), s));
    bool have = ub && t1 && t2 && cC && cX && UG && FAx && FAy && pcell && psum && dst && (tape || !t->chemistry);
    for (auto p : seg) have = have && p;
    for (auto p : inter) have = have && p;
    hf_status r = have ? copy_interior(t, ub, seed, s, true) : HF_ERR_CUDA;
    if (r == HF_OK) r = cuda_status(cudaMemsetAsync(&dst->bad_cell, 0xff, sizeof(unsigned long long), s));
    int64_t nl = 0;
    const unsigned gridc = (unsigned)((nc + 127) / 128);
    const int nseg = (t->nsteps + t->K - 1) / t->K;
    for (int sg = nseg - 1; r == HF_OK && sg >= 0; --sg) {
        const int n0 = sg * t->K, n1 = n0 + t->K < t->nsteps ? n0 + t->K : t->nsteps;
        r = cuda_status(cudaMemcpyAsync(seg[0], t->ck[sg], t->bytes, cudaMemcpyDeviceToDevice, s));
        for (int n = n0; r == HF_OK && n < n1 - 1; ++n)
            r = step_fwd(t, n, seg[n - n0], &inter[keep ? (size_t)4 * (n - n0) : 0], seg[n - n0 + 1], true, s);
        for (int n = n1 - 1; r == HF_OK && n >= n0; --n) {
            double* S0 = seg[n - n0];
            double* const* w = &inter[keep ? (size_t)4 * (n - n0) : 0];
            // A1, X, C, A2 with filled ghosts: recomputed unless kept (the segment's last
            // step was not stepped above)
            if (!keep || n == n1 - 1) r = step_fwd(t, n, S0, w, nullptr, true, s);
            if (r != HF_OK) break;
            const double hh = 0.5 * t->dts[n];
            const unsigned char* fo = &t->fo[(size_t)4 * n];
            cudaError_t e;
            // S2 = (C + E(A2))/2
            e = hf::launch_stage_adjoint(t->ns, L, P, w[3], ub, 0.5, hh, fo[3], FAx, FAy, UG, t1, dst, s, &nl);
            if (e == cudaSuccess) {
                k_lincomb<<<gridc, 128, 0, s>>>(P, t->nv, 0.5, ub, 0.0, nullptr, cC);
                e = cudaGetLastError();
            }
            // A2 = E(C)
            if (e == cudaSuccess)
                e = hf::launch_stage_adjoint(t->ns, L, P, w[2], t1, 1.0, hh, fo[2], FAx, FAy, UG, t2, dst, s, &nl);
            if (e == cudaSuccess) {
                k_lincomb<<<gridc, 128, 0, s>>>(P, t->nv, 1.0, cC, 1.0, t2, cC);
                e = cudaGetLastError();
            }
            // C = react(X)
            if (e == cudaSuccess) {
                if (t->chemistry) {
                    for (int64_t i0 = 0; e == cudaSuccess && i0 < nc; i0 += chunk)
                        e = hf::launch_chem_call_adjoint(t->ns, P, w[1], cC, cX, t->dts[n], t->rtol, t->atol, tape,
                                                         TAPE_CAP, i0, nc - i0 < chunk ? nc - i0 : chunk, pcell, dst,
                                                         s, &nl);
                } else {
                    e = cudaMemcpyAsync(cX, cC, t->bytes, cudaMemcpyDeviceToDevice, s);
                }
            }
            // X = (S0 + E(A1))/2
            if (e == cudaSuccess)
                e = hf::launch_stage_adjoint(t->ns, L, P, w[0], cX, 0.5, hh, fo[1], FAx, FAy, UG, t1, dst, s, &nl);
            // A1 = E(S0)
            if (e == cudaSuccess)
                e = hf::launch_stage_adjoint(t->ns, L, P, S0, t1, 1.0, hh, fo[0], FAx, FAy, UG, t2, dst, s, &nl);
            if (e == cudaSuccess) {
                k_lincomb<<<gridc, 128, 0, s>>>(P, t->nv, 0.5, cX, 1.0, t2, ub);
                e = cudaGetLastError();
            }
            r = cuda_status(e);
        }
    }
    DevStatus st_host;
    if (r == HF_OK) {
        k_sum_rows<<<hfmech::NR, 256, 0, s>>>(pcell, nc, psum);
        r = cuda_status(cudaGetLastError());
    }
    if (r == HF_OK && U0_bar) r = copy_interior(t, ub, U0_bar, s, false);
    double ps[hfmech::NR];
    if (r == HF_OK) r = cuda_status(cudaMemcpyAsync(ps, psum, sizeof(ps), cudaMemcpyDeviceToHost, s));
    if (r == HF_OK) r = cuda_status(cudaMemcpyAsync(&st_host, dst, sizeof(st_host), cudaMemcpyDeviceToHost, s));
    if (r == HF_OK) r = cuda_status(cudaStreamSynchronize(s));
    b.release(s);
    if (r != HF_OK) return r;
    if (st_host.flags & hf::ST_CHEM_FAIL) return HF_ERR_CHEM_FAIL;
    if (st_host.flags & hf::ST_FACE_BAD) return HF_ERR_FACE;
    if (dJ_dlnA) std::memcpy(dJ_dlnA, ps, sizeof(ps));
    return HF_OK;
}

void hf_flow_tape_destroy(hf_flow_tape* t) {
    if (!t) return;
    for (double* p : t->ck) cudaFree(p);
    cudaFree(t->cells);
    delete t;
}

}  // extern "C"
