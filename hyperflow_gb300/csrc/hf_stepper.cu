// Host time stepper over the C ABI for a uniform one-patch level: the loop body of
// BlockAMR::run (HyperFlow_V3/src/BlockAMR.cpp:409-419) with flow() (:266-270),
// euler() first-order redo (:257-263) and react() (:271-285).  The step-start
// state stays untouched until the step is accepted, so a failed attempt rolls back
// by discarding the work buffers (the reference clones the state, :413, :416).
//
// Two ways through a step:
//  * graph path (CFL dt, either chemistry form): the whole Strang step - CFL
//    reduction, dt on the device, four Euler stages (fused kernel, or ghost fill + face
//    + update kernels of the plain form), the chemistry (ordered batched kernel, or one
//    thread per cell), commit, validation - is one CUDA graph.  Every phase ORs its failure flags
//    into one status block; the host reads it once per step.  Any flag discards the
//    step and the host-controlled path below re-runs it.
//  * host-controlled path: the ABI calls one by one with a status read after each,
//    first-order redo of a failed stage, rollback and dt halving up to 18 attempts.
//
// hf_stepper_run enqueues many graph steps with no host round trip between them:
// each step's last kernel records its dt, flags, attempt count and phase timestamps
// in a device run record and, if the step failed, raises the status block's
// abort_run word, after which every step kernel of the later steps returns at entry
// (so the failed step's start state - the other ping-pong buffer - stays intact).
// The host reads the record once per batch, accepts the steps before the failure and
// re-runs the failed one on the host-controlled path.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstring>
#include <utility>
#include <vector>
#include "hf_internal.h"

namespace {
constexpr int RUN_CAP = 256;  // steps per device-resident batch
// Device record of a batch of graph steps.
struct RunRec {
    unsigned int n, pad;
    double dt[RUN_CAP];
    unsigned int flags[RUN_CAP];
    unsigned long long steps[RUN_CAP];   // chemistry step attempts
    unsigned long long coop[RUN_CAP];    // cells of the cooperative chemistry queue
    unsigned long long t[RUN_CAP][4];    // %globaltimer at the phase boundaries (ns)
};
}  // namespace

struct hf_stepper {
    hf_ctx* ctx = nullptr;
    hf_level L{};
    hf_patch P{};
    int ns = 9, nv = 12;
    int chemistry = 1;
    double rtol = 1e-8, atol = 1e-15;
    int flux_form = HF_FLUX_FUSED, chem_form = HF_CHEM_PERSISTENT;
    double* buf[4] = {nullptr, nullptr, nullptr, nullptr};  // [0] = current state
    int64_t* cells = nullptr;                                // valid-cell gather list
    hf_chem_history hist{nullptr, nullptr};                  // batched chemistry history
    double time = 0.0;
    // graph path
    int sm_count = 1;
    hf::DevStatus* gst = nullptr;       // step status (device)
    hf::DevStatus* gst_host = nullptr;  // pinned mirror
    double* ddt = nullptr;              // device [dt, dt/2]
    double* ddt_host = nullptr;         // pinned mirror
    double* trial = nullptr;            // chemistry scratch owned by the stepper
    int* fail = nullptr;
    int32_t* order = nullptr;
    unsigned long long* bins = nullptr;
    alignas(64) unsigned char tmap[4][128];  // TMA descriptors of the four buffers (fused form)
    hf_patch* d_patch = nullptr;             // the level patch in device memory (plain form)
    double *fx = nullptr, *fy = nullptr;     // face fluxes of one stage (plain form)
    double* base[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // by which buffer holds the state
    int64_t graph_kernels[2] = {0, 0};             // kernels in each graph
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // recorded inside the graph
    double graph_cfl = -1.0;
    int use_graph = 1;
    int64_t graph_steps = 0, host_steps = 0;
    unsigned last_graph_flags = 0;   // status flags of the last graph step (0: it was accepted)
    unsigned* phase_flags = nullptr;  // device: the step's flags at its 4 phase boundaries
    unsigned phase_flags_host[4] = {0, 0, 0, 0};
    int capture_error = 0;           // cudaError_t of a failed capture (the graph path is then off)
    // device-resident runs
    RunRec* rec = nullptr;
    RunRec* rec_host = nullptr;
    cudaGraphExec_t exec_run[2] = {nullptr, nullptr};
    int64_t run_kernels[2] = {0, 0};
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

int buf_index(const hf_stepper* st, const double* p) {
    for (int k = 0; k < 4; ++k)
        if (st->base[k] == p) return k;
    return 0;
}

__global__ void k_run_mark(const hf::DevStatus* st, RunRec* rec, int slot) {
    if (st->abort_run) return;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    const unsigned n = rec->n;
    if (n < RUN_CAP) rec->t[n][slot] = t;
}
__global__ void k_run_record(hf::DevStatus* st, const double* ddt, RunRec* rec) {
    if (st->abort_run) return;
    const unsigned n = rec->n;
    if (n < RUN_CAP) {
        rec->dt[n] = ddt[0];
        rec->flags[n] = st->flags;
        rec->steps[n] = st->steps;
        rec->coop[n] = st->coop_cells;
    }
    rec->n = n + 1;
    if (st->flags) st->abort_run = 1;
}

__global__ void k_phase_flags(const hf::DevStatus* st, unsigned* out, int k) { out[k] = st->flags; }

// Phase boundary k of a step: an event-record node and the status flags so far (single
// steps), or a timestamp in the run record (device-resident runs, whose graphs are
// launched many times).
cudaError_t phase_mark(hf_stepper* st, RunRec* rec, int k, cudaStream_t s, int64_t* nl) {
    if (!rec) {
        k_phase_flags<<<1, 1, 0, s>>>(st->gst, st->phase_flags, k);
        ++*nl;
        const cudaError_t e = cudaGetLastError();
        return e != cudaSuccess ? e : cudaEventRecordWithFlags(st->ev[k], s, cudaEventRecordExternal);
    }
    k_run_mark<<<1, 1, 0, s>>>(st->gst, rec, k);
    ++*nl;
    return cudaGetLastError();
}

// The graph path's Strang step from S0 into S2 (T1 and X are work buffers); rec
// non-null: the step of a device-resident run.
cudaError_t enqueue_step(hf_stepper* st, double cfl, double* S0, double* T1, double* X, double* S2, cudaStream_t s,
                         int64_t* nl, RunRec* rec = nullptr) {
    using namespace hf;
    const Level L = make_level(st->L);
    const hf_patch& P = st->P;
    const int64_t nc = (int64_t)P.nx * P.ny;
    cudaError_t e;
#define HF_Q(call)                                \
    do {                                          \
        if ((e = (call)) != cudaSuccess) return e; \
    } while (0)
    HF_Q(cudaMemsetAsync(st->gst, 0, offsetof(DevStatus, abort_run), s));  // abort_run persists over a run
    HF_Q(cudaMemsetAsync(&st->gst->bad_cell, 0xff, sizeof(unsigned long long), s));
    HF_Q(phase_mark(st, rec, 0, s, nl));  // per-phase device time
    HF_Q(launch_cfl(st->ns, L, P, S0, st->gst, s, nl));
    HF_Q(launch_dt_from_rate(st->gst, cfl, st->ddt, s, nl));
    const double* half = st->ddt + 1;
    auto tm = [&](const double* b) { return (const void*)st->tmap[buf_index(st, b)]; };
    // one Euler stage in -> out (Heun combine with old when non-null), h = dt/2 on the device
    auto euler = [&](const double* in, const double* old, double* out) -> cudaError_t {
        if (st->flux_form == HF_FLUX_FUSED)
            return launch_flux_fused(st->ns, L, P, tm(in), in, old, out, 0.0, half, 0, 0, st->gst, s, nl);
        cudaError_t q = launch_fill(st->ns, L, &P, st->d_patch, 1, const_cast<double*>(in), s, nl);
        if (q != cudaSuccess) return q;
        return launch_flux_plain(st->ns, L, P, 0, in, old, out, st->fx, st->fy, 0.0, 0, 0, st->gst, s, nl, half);
    };
    // flow(dt/2)
    HF_Q(euler(S0, nullptr, T1));
    HF_Q(euler(T1, S0, X));
    HF_Q(phase_mark(st, rec, 1, s, nl));
    // react(dt): work-queue head reset, then the chemistry kernel of the stepper's form,
    // commit, validate
    HF_Q(cudaMemsetAsync(&st->gst->counter, 0, 2 * sizeof(unsigned long long), s));  // work-queue heads
    if (st->chemistry) {
        if (st->chem_form == HF_CHEM_PLAIN) {  // the drop-in form: one thread per cell
            HF_Q(launch_chem(st->ns, HF_CHEM_PLAIN, X, P.comp_stride, st->cells, nc, 0.0, nullptr, st->rtol, st->atol,
                             st->trial, st->fail, st->gst, st->sm_count, s, nl, st->ddt));
        } else {
            HF_Q(launch_chem_batched(st->ns, X, P.comp_stride, st->cells, nc, 0.0, st->ddt, nullptr, st->rtol,
                                     st->atol, st->hist.h, st->hist.cost, st->order, st->bins, st->trial, st->fail,
                                     st->gst, st->sm_count, s, nl));
        }
        HF_Q(launch_chem_commit(st->ns, X, P.comp_stride, st->cells, nc, st->trial, s, nl));
        HF_Q(launch_validate(st->ns, P, X, 0, st->gst, s, nl));
    }
    HF_Q(phase_mark(st, rec, 2, s, nl));
    // flow(dt/2)
    HF_Q(euler(X, nullptr, T1));
    HF_Q(euler(T1, X, S2));
    HF_Q(phase_mark(st, rec, 3, s, nl));
    if (rec) {
        k_run_record<<<1, 1, 0, s>>>(st->gst, st->ddt, rec);
        ++*nl;
        HF_Q(cudaGetLastError());
    }
#undef HF_Q
    return cudaSuccess;
}

bool graph_ready(const hf_stepper* st) { return st->use_graph != 0; }

// One step through the graph.  Returns HF_OK with the accepted dt, HF_ERR_INADMISSIBLE
// with *dt = the graph's dt when the step must be re-run on the host-controlled path,
// or HF_ERR_CUDA when no graph could be made.
// Drops the instantiated graphs when the CFL number changes (it is baked into them).
void graphs_for_cfl(hf_stepper* st, double cfl) {
    if (st->graph_cfl == cfl) return;
    for (auto& g : st->exec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (auto& g : st->exec_run)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    st->graph_cfl = cfl;
}

// Captures the step of parity k (k = 0: state in base[0] -> base[3]; k = 1: the
// reverse) as a graph; rec non-null for a device-resident run.
cudaError_t capture_step(hf_stepper* st, double cfl, int k, RunRec* rec, cudaGraphExec_t* exec, int64_t* nl) {
    double* S0 = st->base[k ? 3 : 0];
    double* S2 = st->base[k ? 0 : 3];
    cudaGraph_t g = nullptr;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    *nl = 0;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t q = enqueue_step(st, cfl, S0, st->base[1], st->base[2], S2, cs, nl, rec);
        e = cudaStreamEndCapture(cs, &g);
        if (q != cudaSuccess) e = q;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    return e;
}

hf_status graph_step(hf_stepper* st, double cfl, double* dt, cudaStream_t s) {
    const int k = st->buf[0] == st->base[0] ? 0 : 1;
    graphs_for_cfl(st, cfl);
    if (!st->exec[k]) {
        int64_t nl = 0;
        const cudaError_t ce = capture_step(st, cfl, k, nullptr, &st->exec[k], &nl);
        if (ce != cudaSuccess) {
            st->capture_error = (int)ce;
            st->use_graph = 0;  // host-controlled path from here on
            cudaGetLastError();
            return HF_ERR_CUDA;
        }
        st->graph_kernels[k] = nl;
    }
    if (cudaGraphLaunch(st->exec[k], s) != cudaSuccess ||
        cudaMemcpyAsync(st->gst_host, st->gst, sizeof(hf::DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(st->ddt_host, st->ddt, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(st->phase_flags_host, st->phase_flags, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return HF_ERR_CUDA;
    hf::ctx_add_launches(st->ctx, st->graph_kernels[k], st->chemistry ? (int64_t)st->P.nx * st->P.ny : 0,
                         (int64_t)st->gst_host->steps);
    hf::ctx_add_coop(st->ctx, (int64_t)st->gst_host->coop_cells);
    if (hf::ctx_timing_enabled(st->ctx)) {
        // ev0..ev1: CFL + dt + first flow; ev1..ev2: chemistry (order, kernel, commit,
        // validate); ev2..ev3: second flow
        float a = 0.f, b = 0.f, c = 0.f;
        if (cudaEventElapsedTime(&a, st->ev[0], st->ev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&b, st->ev[1], st->ev[2]) == cudaSuccess &&
            cudaEventElapsedTime(&c, st->ev[2], st->ev[3]) == cudaSuccess)
            hf::ctx_add_timing(st->ctx, a + c, b, 0.0, 4, st->chemistry ? 1 : 0, 2);
        else
            (void)cudaGetLastError();  // leave no pending error for the caller's next call
    }
    *dt = st->ddt_host[0];
    st->last_graph_flags = st->gst_host->flags;
    return st->gst_host->flags ? HF_ERR_INADMISSIBLE : HF_OK;
}

hf_status host_step(hf_stepper* st, double cfl, double* dt, cudaStream_t s) {
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
            ++st->host_steps;
            return HF_OK;
        }
        if (r == HF_ERR_ARG || r == HF_ERR_CUDA || r == HF_ERR_TIMEOUT) return r;
        hf::ctx_add_counters(st->ctx, 0, 1);
        h *= 0.5;  // rollback: buf[0] was never written (BlockAMR.cpp:416)
    }
    return HF_ERR_INADMISSIBLE;
}

// Up to RUN_CAP graph steps enqueued back to back, then one read of the run record.
// Returns the number of steps taken (accepted graph steps, plus one host-controlled
// step when a graph step failed) in *taken.
hf_status run_batch(hf_stepper* st, int nsteps, double cfl, cudaStream_t s, int* taken) {
    *taken = 0;
    graphs_for_cfl(st, cfl);
    for (int k = 0; k < 2; ++k)
        if (!st->exec_run[k]) {
            int64_t nl = 0;
            if (capture_step(st, cfl, k, st->rec, &st->exec_run[k], &nl) != cudaSuccess) {
                cudaGetLastError();
                return HF_ERR_CUDA;
            }
            st->run_kernels[k] = nl;
        }
    const int batch = nsteps < RUN_CAP ? nsteps : RUN_CAP;
    if (cudaMemsetAsync(&st->gst->abort_run, 0, sizeof(unsigned int), s) != cudaSuccess ||
        cudaMemsetAsync(&st->rec->n, 0, sizeof(unsigned int), s) != cudaSuccess)
        return HF_ERR_CUDA;
    int k = st->buf[0] == st->base[0] ? 0 : 1;
    for (int i = 0; i < batch; ++i, k ^= 1)
        if (cudaGraphLaunch(st->exec_run[k], s) != cudaSuccess) return HF_ERR_CUDA;
    if (cudaMemcpyAsync(st->rec_host, st->rec, sizeof(RunRec), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return HF_ERR_CUDA;
    const RunRec& r = *st->rec_host;
    const int n = (int)(r.n < (unsigned)batch ? r.n : (unsigned)batch);
    const bool failed = n > 0 && r.flags[n - 1] != 0;
    const int acc = failed ? n - 1 : n;
    double flux_ms = 0.0, chem_ms = 0.0;
    int64_t attempts = 0, coop = 0;
    for (int i = 0; i < acc; ++i) {
        st->time += r.dt[i];
        attempts += (int64_t)r.steps[i];
        coop += (int64_t)r.coop[i];
        flux_ms += 1e-6 * (double)((r.t[i][1] - r.t[i][0]) + (r.t[i][3] - r.t[i][2]));
        chem_ms += 1e-6 * (double)(r.t[i][2] - r.t[i][1]);
    }
    const int64_t nc = (int64_t)st->P.nx * st->P.ny;
    hf::ctx_add_launches(st->ctx, (st->run_kernels[0] + st->run_kernels[1]) / 2 * acc, st->chemistry ? nc * acc : 0,
                         attempts);
    hf::ctx_add_coop(st->ctx, coop);
    if (hf::ctx_timing_enabled(st->ctx)) hf::ctx_add_timing(st->ctx, flux_ms, chem_ms, 0.0, 4 * acc, acc, 0);
    if (acc & 1) std::swap(st->buf[0], st->buf[3]);
    st->graph_steps += acc;
    *taken = acc;
    if (failed) {
        double h = r.dt[n - 1];  // re-run the failed step with host control from its start state
        const hf_status q = host_step(st, cfl, &h, s);
        if (q != HF_OK) return q;
        *taken = acc + 1;
    }
    return HF_OK;
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
    st->ns = hf_nspecies(ctx);
    st->nv = st->ns + 3;
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
    const int64_t nc = (int64_t)P.nx * P.ny;
    int dev = 0;
    bool ok = cudaGetDevice(&dev) == cudaSuccess &&
              cudaDeviceGetAttribute(&st->sm_count, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess;
    for (int b = 0; ok && b < 4; ++b) {
        ok = cudaMalloc(&st->buf[b], bytes) == cudaSuccess && cudaMemset(st->buf[b], 0, bytes) == cudaSuccess;
        st->base[b] = st->buf[b];
    }
    ok = ok && cudaMalloc(&st->cells, sizeof(int64_t) * nc) == cudaSuccess &&
         cudaMalloc(&st->hist.h, sizeof(double) * nc) == cudaSuccess &&
         cudaMalloc(&st->hist.cost, sizeof(int32_t) * nc) == cudaSuccess &&
         cudaMemset(st->hist.h, 0, sizeof(double) * nc) == cudaSuccess &&
         cudaMemset(st->hist.cost, 0, sizeof(int32_t) * nc) == cudaSuccess &&
         cudaMalloc(&st->gst, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMalloc(&st->phase_flags, 4 * sizeof(unsigned)) == cudaSuccess &&
         cudaMemset(st->phase_flags, 0, 4 * sizeof(unsigned)) == cudaSuccess &&
         cudaMemset(st->gst, 0, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMalloc(&st->rec, sizeof(RunRec)) == cudaSuccess &&
         cudaMallocHost(&st->rec_host, sizeof(RunRec)) == cudaSuccess &&
         cudaMallocHost(&st->gst_host, sizeof(hf::DevStatus)) == cudaSuccess &&
         cudaMalloc(&st->ddt, 2 * sizeof(double)) == cudaSuccess &&
         cudaMallocHost(&st->ddt_host, 2 * sizeof(double)) == cudaSuccess &&
         cudaMalloc(&st->trial, sizeof(double) * st->nv * nc) == cudaSuccess &&
         cudaMalloc(&st->fail, sizeof(int) * nc) == cudaSuccess &&
         cudaMalloc(&st->order, sizeof(int32_t) * nc) == cudaSuccess &&
         cudaMalloc(&st->bins, hf::CHEM_BINS * sizeof(unsigned long long)) == cudaSuccess;
    for (int k = 0; ok && k < 4; ++k) ok = cudaEventCreate(&st->ev[k]) == cudaSuccess;
    if (ok) {
        std::vector<int64_t> idx(nc);
        for (int64_t j = 0; j < P.ny; ++j)
            for (int64_t i = 0; i < P.nx; ++i) idx[j * P.nx + i] = (j + P.ng) * P.pitch + (i + P.ng);
        ok = cudaMemcpy(st->cells, idx.data(), sizeof(int64_t) * nc, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && flux_form == HF_FLUX_FUSED)
        for (int b = 0; ok && b < 4; ++b) ok = hf::make_tensor_map(st->tmap[b], st->buf[b], P, st->nv);
    if (ok && flux_form == HF_FLUX_PLAIN) {
        const size_t fxb = sizeof(double) * st->nv * (size_t)(P.nx + 1) * P.ny;
        const size_t fyb = sizeof(double) * st->nv * (size_t)P.nx * (P.ny + 1);
        ok = cudaMalloc(&st->d_patch, sizeof(hf_patch)) == cudaSuccess &&
             cudaMemcpy(st->d_patch, &P, sizeof(hf_patch), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMalloc(&st->fx, fxb) == cudaSuccess && cudaMalloc(&st->fy, fyb) == cudaSuccess;
    }
    if (ok && U0) {
        for (int n = 0; ok && n < st->nv; ++n)
            ok = cudaMemcpy2D(st->buf[0] + n * P.comp_stride + P.ng * P.pitch + P.ng, P.pitch * sizeof(double),
                              U0 + (size_t)n * nc, P.nx * sizeof(double), P.nx * sizeof(double), P.ny,
                              cudaMemcpyDeviceToDevice) == cudaSuccess;
    }
    if (!ok) {
        hf_stepper_destroy(st);
        return HF_ERR_CUDA;
    }
    *out = st;
    return HF_OK;
}

void hf_stepper_destroy(hf_stepper* st) {
    if (!st) return;
    for (auto g : st->exec)
        if (g) cudaGraphExecDestroy(g);
    for (auto g : st->exec_run)
        if (g) cudaGraphExecDestroy(g);
    for (auto e : st->ev)
        if (e) cudaEventDestroy(e);
    for (auto b : st->base)
        if (b) cudaFree(b);
    cudaFree(st->cells);
    cudaFree(st->hist.h);
    cudaFree(st->hist.cost);
    cudaFree(st->phase_flags);
    cudaFree(st->gst);
    cudaFreeHost(st->gst_host);
    cudaFree(st->rec);
    cudaFreeHost(st->rec_host);
    cudaFree(st->ddt);
    cudaFreeHost(st->ddt_host);
    cudaFree(st->trial);
    cudaFree(st->fail);
    cudaFree(st->order);
    cudaFree(st->bins);
    cudaFree(st->d_patch);
    cudaFree(st->fx);
    cudaFree(st->fy);
    delete st;
}

void hf_stepper_graph_info(const hf_stepper* st, uint32_t* last_flags, int32_t* capture_error,
                           uint32_t* phase_flags) {
    if (last_flags) *last_flags = st ? st->last_graph_flags : 0;
    if (capture_error) *capture_error = st ? st->capture_error : 0;
    if (phase_flags)
        for (int k = 0; k < 4; ++k) phase_flags[k] = st ? st->phase_flags_host[k] : 0;
}

hf_status hf_stepper_step(hf_stepper* st, double cfl, double* dt, void* stream) {
    if (!st || !dt) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (!(*dt > 0) && graph_ready(st)) {
        double h = 0.0;
        const hf_status r = graph_step(st, cfl, &h, s);
        if (r == HF_OK) {
            std::swap(st->buf[0], st->buf[3]);
            st->time += h;
            *dt = h;
            ++st->graph_steps;
            return HF_OK;
        }
        if (r == HF_ERR_INADMISSIBLE) {
            *dt = h;  // re-run this step with host control from the untouched start state
            return host_step(st, cfl, dt, s);
        }
        // no graph: host-controlled path from here on
    }
    return host_step(st, cfl, dt, s);
}

hf_status hf_stepper_run(hf_stepper* st, int32_t nsteps, double cfl, int32_t* steps_done, void* stream) {
    if (steps_done) *steps_done = 0;
    if (!st || nsteps < 0 || !(cfl > 0)) return HF_ERR_ARG;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int done = 0;
    while (done < nsteps) {
        int taken = 0;
        hf_status r = HF_OK;
        if (graph_ready(st)) {
            r = run_batch(st, nsteps - done, cfl, s, &taken);
            if (r == HF_ERR_CUDA && taken == 0 && st->use_graph) {
                st->use_graph = 0;  // no run graphs: host-controlled steps from here on
                r = HF_OK;
            }
        } else {
            double h = 0.0;
            r = hf_stepper_step(st, cfl, &h, stream);
            taken = r == HF_OK ? 1 : 0;
        }
        done += taken;
        if (steps_done) *steps_done = done;
        if (r != HF_OK) return r;
    }
    return HF_OK;
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

hf_status hf_stepper_cfl_dt(hf_stepper* st, double cfl, double* dt, void* stream) {
    if (!st || !dt) return HF_ERR_ARG;
    return hf_cfl_dt(st->ctx, &st->L, &st->P, 1, st->buf[0], cfl, dt, stream);
}

void hf_stepper_stats(const hf_stepper* st, int64_t* graph_steps, int64_t* host_steps) {
    if (graph_steps) *graph_steps = st ? st->graph_steps : 0;
    if (host_steps) *host_steps = st ? st->host_steps : 0;
}

void hf_stepper_set_graph(hf_stepper* st, int enable) {
    if (st) st->use_graph = enable != 0;
}

}  // extern "C"
