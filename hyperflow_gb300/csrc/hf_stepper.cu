// Host time stepper over the C ABI for a uniform one-patch level: the loop body of
// BlockAMR::run (HyperFlow_V3/src/BlockAMR.cpp:409-419) with flow() (:266-270),
// euler() first-order redo (:257-263) and react() (:271-285).  The step-start
// state stays untouched until the step is accepted, so a failed attempt rolls back
// by discarding the work buffers (the reference clones the state, :413, :416).
#include <cuda_runtime.h>
#include <cstring>
#include <vector>
#include "hf_internal.h"

struct hf_stepper {
    hf_ctx* ctx = nullptr;
    hf_level L{};
    hf_patch P{};
    int nv = 12;
    int chemistry = 1;
    double rtol = 1e-8, atol = 1e-15;
    int flux_form = HF_FLUX_FUSED, chem_form = HF_CHEM_PERSISTENT;
    double* buf[4] = {nullptr, nullptr, nullptr, nullptr};  // [0] = current state
    int64_t* cells = nullptr;                                // valid-cell gather list
    hf_chem_history hist{nullptr, nullptr};                  // batched chemistry history
    double time = 0.0;
};

namespace {

hf_status stage(hf_stepper* st, const double* in, const double* old, double* out, double h, cudaStream_t s) {
    if (st->flux_form == HF_FLUX_PLAIN) {
        hf_status r = hf_fill_ghosts(st->ctx, &st->L, &st->P, 1, const_cast<double*>(in), s);
        if (r != HF_OK) return r;
    }
    for (int fo = 0; fo < 2; ++fo) {
        int64_t bad = -1;
        hf_status r = hf_flux_update(st->ctx, &st->L, &st->P, 1, in, old, out, nullptr, nullptr, h, fo, st->flux_form,
                                     &bad, s);
        if (r == HF_OK) {
            if (fo) hf::ctx_add_counters(st->ctx, 1, 0);
            return HF_OK;
        }
        // domain_error of the stage output -> redo the stage first order (BlockAMR.cpp:258-263)
        if (r != HF_ERR_INADMISSIBLE && r != HF_ERR_NEGATIVE) return r;
    }
    return HF_ERR_INADMISSIBLE;
}

// flow(h): out = [in + E(E(in))]/2 (BlockAMR.cpp:266-269); in is not modified.
hf_status flow(hf_stepper* st, const double* in, double* tmp, double* out, double h, cudaStream_t s) {
    hf_status r = stage(st, in, nullptr, tmp, h, s);
    if (r != HF_OK) return r;
    return stage(st, tmp, in, out, h, s);
}

}  // namespace

extern "C" {

hf_status hf_stepper_create(hf_ctx* ctx, const hf_level* level, const double* U0, int chemistry, double rtol,
                            double atol, int flux_form, int chem_form, hf_stepper** out) {
    if (!ctx || !level || !out || level->nx <= 0 || level->ny <= 0) return HF_ERR_ARG;
    *out = nullptr;
    hf_stepper* st = new hf_stepper();
    st->ctx = ctx;
    st->L = *level;
    st->nv = hf_nspecies(ctx) + 3;
    st->chemistry = chemistry;
    st->rtol = rtol;
    st->atol = atol;
    st->flux_form = flux_form;
    st->chem_form = chem_form;
    hf_patch& P = st->P;
    P.ilo = P.jlo = 0;
    P.nx = level->nx;
    P.ny = level->ny;
    P.ng = 2;
    P.pitch = (P.nx + 2 * P.ng + 1) & ~int64_t(1);
    P.comp_stride = (P.pitch * (P.ny + 2 * P.ng) + 31) & ~int64_t(31);
    P.offset = 0;
    const size_t bytes = sizeof(double) * (size_t)P.comp_stride * st->nv;
    for (int b = 0; b < 4; ++b) {
        if (cudaMalloc(&st->buf[b], bytes) != cudaSuccess) { hf_stepper_destroy(st); return HF_ERR_CUDA; }
        cudaMemset(st->buf[b], 0, bytes);
    }
    const int64_t nc = (int64_t)P.nx * P.ny;
    std::vector<int64_t> idx(nc);
    for (int64_t j = 0; j < P.ny; ++j)
        for (int64_t i = 0; i < P.nx; ++i) idx[j * P.nx + i] = (j + P.ng) * P.pitch + (i + P.ng);
    if (cudaMalloc(&st->cells, sizeof(int64_t) * nc) != cudaSuccess ||
        cudaMemcpy(st->cells, idx.data(), sizeof(int64_t) * nc, cudaMemcpyHostToDevice) != cudaSuccess) {
        hf_stepper_destroy(st);
        return HF_ERR_CUDA;
    }
    if (cudaMalloc(&st->hist.h, sizeof(double) * nc) != cudaSuccess ||
        cudaMalloc(&st->hist.cost, sizeof(int32_t) * nc) != cudaSuccess ||
        cudaMemset(st->hist.h, 0, sizeof(double) * nc) != cudaSuccess ||
        cudaMemset(st->hist.cost, 0, sizeof(int32_t) * nc) != cudaSuccess) {
        hf_stepper_destroy(st);
        return HF_ERR_CUDA;
    }
    if (U0) {
        for (int n = 0; n < st->nv; ++n) {
            cudaError_t e = cudaMemcpy2D(st->buf[0] + n * P.comp_stride + P.ng * P.pitch + P.ng, P.pitch * sizeof(double),
                                         U0 + (size_t)n * nc, P.nx * sizeof(double), P.nx * sizeof(double), P.ny,
                                         cudaMemcpyDeviceToDevice);
            if (e != cudaSuccess) { hf_stepper_destroy(st); return HF_ERR_CUDA; }
        }
    }
    *out = st;
    return HF_OK;
}

void hf_stepper_destroy(hf_stepper* st) {
    if (!st) return;
    for (auto b : st->buf)
        if (b) cudaFree(b);
    if (st->cells) cudaFree(st->cells);
    if (st->hist.h) cudaFree(st->hist.h);
    if (st->hist.cost) cudaFree(st->hist.cost);
    delete st;
}

hf_status hf_stepper_step(hf_stepper* st, double cfl, double* dt, void* stream) {
    if (!st || !dt) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double h = *dt;
    if (!(h > 0)) {
        hf_status r = hf_cfl_dt(st->ctx, &st->L, &st->P, 1, st->buf[0], cfl, &h, s);
        if (r != HF_OK) return r;
    }
    for (int attempt = 0; attempt < 18; ++attempt) {
        double* S0 = st->buf[0];
        double* T1 = st->buf[1];
        double* X = st->buf[2];
        double* S2 = st->buf[3];
        hf_status r = flow(st, S0, T1, X, 0.5 * h, s);
        if (r == HF_OK && st->chemistry) {
            int64_t first = -1;
            const int64_t nc = (int64_t)st->P.nx * st->P.ny;
            if (st->chem_form == HF_CHEM_PERSISTENT)
                r = hf_chem_advance_batched(st->ctx, X, st->P.comp_stride, st->cells, nc, h, nullptr, st->rtol,
                                            st->atol, &st->hist, &first, s);
            else
                r = hf_chem_advance(st->ctx, X, st->P.comp_stride, st->cells, nc, h, nullptr, st->rtol, st->atol,
                                    st->chem_form, &first, s);
            if (r == HF_OK) {
                int64_t bad = -1;
                r = hf_validate(st->ctx, &st->L, &st->P, 1, X, &bad, s);
            }
        }
        if (r == HF_OK) r = flow(st, X, T1, S2, 0.5 * h, s);
        if (r == HF_OK) {
            st->buf[0] = S2;
            st->buf[3] = S0;
            st->time += h;
            *dt = h;
            return HF_OK;
        }
        if (r == HF_ERR_ARG || r == HF_ERR_CUDA || r == HF_ERR_TIMEOUT) return r;
        hf::ctx_add_counters(st->ctx, 0, 1);
        h *= 0.5;  // rollback: buf[0] was never written (BlockAMR.cpp:416)
    }
    return HF_ERR_INADMISSIBLE;
}

hf_status hf_stepper_get(hf_stepper* st, double* U, void* stream) {
    if (!st || !U) return HF_ERR_ARG;
    const hf_patch& P = st->P;
    const int64_t nc = (int64_t)P.nx * P.ny;
    for (int n = 0; n < st->nv; ++n) {
        cudaError_t e = cudaMemcpy2DAsync(U + (size_t)n * nc, P.nx * sizeof(double),
                                          st->buf[0] + n * P.comp_stride + P.ng * P.pitch + P.ng, P.pitch * sizeof(double),
                                          P.nx * sizeof(double), P.ny, cudaMemcpyDeviceToDevice,
                                          reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return HF_ERR_CUDA;
    }
    return HF_OK;
}

hf_status hf_stepper_set_host(hf_stepper* st, const double* U, void* stream) {
    if (!st || !U) return HF_ERR_ARG;
    const hf_patch& P = st->P;
    const int64_t nc = (int64_t)P.nx * P.ny;
    for (int n = 0; n < st->nv; ++n) {
        cudaError_t e = cudaMemcpy2DAsync(st->buf[0] + n * P.comp_stride + P.ng * P.pitch + P.ng, P.pitch * sizeof(double),
                                          U + (size_t)n * nc, P.nx * sizeof(double), P.nx * sizeof(double), P.ny,
                                          cudaMemcpyHostToDevice, reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return HF_ERR_CUDA;
    }
    return HF_OK;
}

hf_status hf_stepper_get_host(hf_stepper* st, double* U, void* stream) {
    if (!st || !U) return HF_ERR_ARG;
    const hf_patch& P = st->P;
    const int64_t nc = (int64_t)P.nx * P.ny;
    for (int n = 0; n < st->nv; ++n) {
        cudaError_t e = cudaMemcpy2DAsync(U + (size_t)n * nc, P.nx * sizeof(double),
                                          st->buf[0] + n * P.comp_stride + P.ng * P.pitch + P.ng, P.pitch * sizeof(double),
                                          P.nx * sizeof(double), P.ny, cudaMemcpyDeviceToHost,
                                          reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return HF_ERR_CUDA;
    }
    return cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)) == cudaSuccess ? HF_OK : HF_ERR_CUDA;
}

double hf_stepper_time(const hf_stepper* st) { return st ? st->time : 0.0; }

}  // extern "C"
