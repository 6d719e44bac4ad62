// Stiff per-cell chemistry: the reference's constant-(rho, e) ODE
// (HyperFlow_V3/src/chemistry.cpp:36-53: unknowns Y_0..Y_{NS-2}, last species
// dependent, T from the UV inversion at every evaluation) integrated over dt with
// Rodas4 (Hairer & Wanner, Solving ODEs II, Sec. VI.7; KPP coefficient ordering),
// WRMS errors with weights atol + rtol*max(|y_old|, |y_new|), an analytic Jacobian,
// and the KPP step controller.  Cell semantics follow Chemistry::advance
// (chemistry.cpp:55-76): properties() check, clip y >= -1e-13 to 0, dependent
// species closes the mass, final properties() check.  Batch semantics follow
// ChemistryBatch::advance (chemistry_batch.cpp:21-50): all-or-nothing with the
// lowest failing index.
//
// The per-cell pieces (thermo, kinetics, right-hand side, Jacobian, Rodas4 step
// attempt) are in hf_kinetics.cuh; this file holds the chemistry kernels (plain,
// persistent, batched with its cost-ordered queue), the ErrorEst tagging kernel and
// the allocation-free entry point.  Rate data: pre-exponential factors sit in
// __constant__ memory (c_A, c_A0) so they can be scaled for sensitivity checks;
// reaction structure, temperature exponents and activation temperatures are
// compile-time constants of the generated mechanism table, so every species index
// is a register index.
#include <atomic>
#include <cstdlib>
#include "hf_chem_coop.cuh"

namespace hf {

cudaError_t chem_set_rate_scale(const double* scale) { return upload_rate_constants(scale); }

// ---------------------------------------------------------------- kernels
template <int NS>
__device__ __forceinline__ void load_cell(const double* U, int64_t cs, int64_t base, double* u) {
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) u[n] = U[base + n * cs];
}
__device__ __forceinline__ void report(DevStatus* st, int* fail, int64_t i, int code) {
    fail[i] = code;
    atomicOr(&st->flags, code == CELL_MAXSTEPS ? ST_MAXSTEPS : ST_CHEM_FAIL);
    atomicMin(&st->bad_cell, (unsigned long long)i);
}

// Plain form: one thread runs one cell to completion.
template <int NS>
__global__ void __launch_bounds__(64) k_chem_plain(const double* __restrict__ U, int64_t cs,
                                                   const int64_t* __restrict__ cell_index, int64_t count, double dt,
                                                   const double* __restrict__ dt_dev,
                                                   const double* __restrict__ dt_cell, double rtol, double atol,
                                                   double* __restrict__ trial, int* __restrict__ fail, DevStatus* st) {
    if (st->abort_run) return;  // an earlier step of this device-resident run failed
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    if (dt_dev) dt = *dt_dev;  // interval from device memory (graph-captured steps)
    double u[NS + 3];
    load_cell<NS>(U, cs, cell_index ? cell_index[i] : i, u);
    ChemCell<NS> c;
    int r = cell_begin<NS>(c, u, dt_cell ? dt_cell[i] : dt, rtol, atol);
    while (r == CELL_CONTINUE) r = cell_attempt<NS>(c, rtol, atol);
    atomicAdd(&st->steps, (unsigned long long)c.attempts);
    if (r == CELL_DONE && cell_end<NS>(c, u)) {
#pragma unroll
        for (int n = 0; n < NS + 3; ++n) trial[n * count + i] = u[n];
        fail[i] = 0;
    } else {
        report(st, fail, i, r == CELL_MAXSTEPS ? CELL_MAXSTEPS : CELL_FAIL);
    }
}

// Persistent form: each lane holds one cell and the warp advances all its lanes by
// one step attempt per iteration (the same instruction stream for every lane).
// A lane whose cell finishes writes it and takes the next cell index from the
// device work queue (one atomic per warp refill round).  The number of step
// attempts per lane varies freely; lanes stay busy until the queue is empty.
template <int NS>
__global__ void __launch_bounds__(64) k_chem_persistent(const double* __restrict__ U, int64_t cs,
                                                        const int64_t* __restrict__ cell_index, int64_t count,
                                                        double dt, const double* __restrict__ dt_cell, double rtol,
                                                        double atol, double* __restrict__ trial,
                                                        int* __restrict__ fail, DevStatus* st) {
    const unsigned lane = threadIdx.x & 31;
    ChemCell<NS> c;
    int64_t cell = -1;
    bool active = false, drained = false;
    unsigned long long my_attempts = 0;
    for (;;) {
        // refill lanes without a cell: one atomic per warp and round
        if (!drained) {
            const unsigned need = __ballot_sync(0xffffffffu, !active);
            bool none = false;
            if (need) {
                const int leader = __ffs(need) - 1;
                unsigned long long base = 0;
                if ((int)lane == leader) base = atomicAdd(&st->counter, (unsigned long long)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!active) {
                    const int64_t k = (int64_t)(base + __popc(need & ((1u << lane) - 1u)));
                    if (k < count) {
                        cell = k;
                        double u[NS + 3];
                        load_cell<NS>(U, cs, cell_index ? cell_index[k] : k, u);
                        const int r = cell_begin<NS>(c, u, dt_cell ? dt_cell[k] : dt, rtol, atol);
                        if (r == CELL_CONTINUE) active = true;
                        else report(st, fail, k, CELL_FAIL);
                    } else {
                        none = true;
                    }
                }
            }
            drained = __any_sync(0xffffffffu, none);
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (drained) break;
            continue;
        }
        if (active) {
            const int r = cell_attempt<NS>(c, rtol, atol);
            if (r != CELL_CONTINUE) {
                my_attempts += c.attempts;
                double u[NS + 3];
                if (r == CELL_DONE && cell_end<NS>(c, u)) {
#pragma unroll
                    for (int n = 0; n < NS + 3; ++n) trial[n * count + cell] = u[n];
                    fail[cell] = 0;
                } else {
                    report(st, fail, cell, r == CELL_MAXSTEPS ? CELL_MAXSTEPS : CELL_FAIL);
                }
                active = false;
            }
        }
    }
    if (my_attempts) atomicAdd(&st->steps, my_attempts);
}

template <int NS>
__global__ void k_chem_commit(double* __restrict__ U, int64_t cs, const int64_t* __restrict__ cell_index, int64_t count,
                              const double* __restrict__ trial) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int64_t b = cell_index ? cell_index[i] : i;
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) U[b + n * cs] = trial[n * count + i];
}

// Batched form: the persistent lane-refill loop of k_chem_persistent over a work
// queue ordered most-expensive-first (order[]), starting each cell with
// cell_begin_batched, and recording per cell the attempts taken (cost[]) and the
// controller's proposed next step (h_hist[]) for the next call.
// Cooperative phase of the batched kernel: queue positions [0, ncoop) (the costliest
// buckets), one cell per group of 8 lanes (hf_chem_coop.cuh), the refill scheme of the
// per-lane loop with groups in place of lanes.
template <int NS>
__device__ __forceinline__ void coop_phase(const double* __restrict__ U, int64_t cs,
                                           const int64_t* __restrict__ cell_index, const int32_t* __restrict__ order,
                                           int64_t count, int64_t ncoop, double dt, const double* __restrict__ dt_cell,
                                           double rtol, double atol, double* __restrict__ trial,
                                           int* __restrict__ fail, double* __restrict__ h_hist,
                                           int32_t* __restrict__ cost, DevStatus* st, coop::GShared* sh) {
    using namespace coop;
    const Grp g = grp();
    const unsigned lane = threadIdx.x & 31;
    GInt c{};
    double y = 0.0, f0 = 0.0, J[NQ];
#pragma unroll
    for (int j = 0; j < NQ; ++j) J[j] = 0.0;
    int64_t cell = -1;
    bool active = false, drained = false;
    unsigned long long my_attempts = 0;
    auto finish = [&](int64_t k, bool screened) {
        double u[NS + 3];
        const bool ok = gend<NS>(g, c, y, u, sh->T);
        if (g.t == 0) {
            if (ok) {
#pragma unroll
                for (int n = 0; n < NS + 3; ++n) trial[n * count + k] = u[n];
                fail[k] = 0;
                if (!screened && h_hist) h_hist[k] = c.h;
                if (cost) cost[k] = screened ? 0 : c.attempts;
            } else {
                report(st, fail, k, CELL_FAIL);
            }
        }
    };
    for (;;) {
        if (!drained) {
            const unsigned need = __ballot_sync(0xffffffffu, !active) & 0x01010101u;  // first lane of each group
            bool none = false;
            if (need) {
                const int leader = __ffs(need) - 1;
                unsigned long long base = 0;
                if ((int)lane == leader) base = atomicAdd(&st->coop_counter, (unsigned long long)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!active) {
                    const int64_t q = (int64_t)(base + __popc(need & ((1u << g.base) - 1u)));
                    if (q < ncoop) {
                        const int64_t k = (int64_t)order[q];
                        cell = k;
                        double u[NS + 3];
                        const int64_t b = cell_index ? cell_index[k] : k;
#pragma unroll
                        for (int n = 0; n < NS + 3; ++n) u[n] = U[b + n * cs];
                        const int r = gbegin<NS>(g, c, y, f0, J, u, dt_cell ? dt_cell[k] : dt, rtol, atol,
                                                 h_hist ? h_hist[k] : 0.0, sh);
                        if (g.t == 0) atomicAdd(&st->coop_cells, 1ull);
                        if (r == CELL_CONTINUE) active = true;
                        else if (r == CELL_DONE) finish(k, true);
                        else if (g.t == 0) report(st, fail, k, CELL_FAIL);
                    } else {
                        none = true;
                    }
                }
            }
            drained = __any_sync(0xffffffffu, none);
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (drained) break;
            continue;
        }
        if (active) {
            const int r = gattempt<NS>(g, c, y, f0, J, rtol, atol, sh);
            if (r != CELL_CONTINUE) {
                if (g.t == 0) my_attempts += c.attempts;
                if (r == CELL_DONE) finish(cell, false);
                else if (g.t == 0) report(st, fail, cell, r == CELL_MAXSTEPS ? CELL_MAXSTEPS : CELL_FAIL);
                active = false;
            }
        }
    }
    if (my_attempts) atomicAdd(&st->steps, my_attempts);
}

template <int NS, int MINB, bool COOP>
__global__ void __launch_bounds__(64, MINB) k_chem_batched(const double* __restrict__ U, int64_t cs,
                                                     const int64_t* __restrict__ cell_index,
                                                     const int32_t* __restrict__ order, int64_t count, double dt,
                                                     const double* __restrict__ dt_dev,
                                                     const double* __restrict__ dt_cell, double rtol, double atol,
                                                     double* __restrict__ trial, int* __restrict__ fail,
                                                     double* __restrict__ h_hist, int32_t* __restrict__ cost,
                                                     const unsigned long long* __restrict__ coop_n, DevStatus* st) {
    if (st->abort_run) return;  // an earlier step of this device-resident run failed
    const unsigned lane = threadIdx.x & 31;
    if (dt_dev) dt = *dt_dev;  // interval from device memory (graph-captured steps)
    // COOP: the costliest cells first, one cell per group of 8 lanes; the rest one per
    // lane.  Without it the kernel holds no shared memory (the L1 keeps the lanes' stacks).
    int64_t ncoop = 0;
    if constexpr (COOP) {
        ncoop = (order && coop_n) ? (int64_t)*coop_n : 0;
        if (ncoop > 0) {
            __shared__ coop::GShared sh[2][4];  // 64-thread blocks: 2 warps of 4 groups
            coop_phase<NS>(U, cs, cell_index, order, count, ncoop, dt, dt_cell, rtol, atol, trial, fail, h_hist,
                           cost, st, &sh[threadIdx.x >> 5][(threadIdx.x & 31) >> 3]);
        }
    }
    ChemCell<NS> c;
    int64_t cell = -1;
    bool active = false, drained = false;
    unsigned long long my_attempts = 0;
    for (;;) {
        if (!drained) {
            const unsigned need = __ballot_sync(0xffffffffu, !active);
            bool none = false;
            if (need) {
                const int leader = __ffs(need) - 1;
                unsigned long long base = 0;
                if ((int)lane == leader) base = atomicAdd(&st->counter, (unsigned long long)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!active) {
                    const int64_t q = ncoop + (int64_t)(base + __popc(need & ((1u << lane) - 1u)));
                    if (q < count) {
                        const int64_t k = order ? (int64_t)order[q] : q;
                        cell = k;
                        double u[NS + 3];
                        load_cell<NS>(U, cs, cell_index ? cell_index[k] : k, u);
                        const int r = cell_begin_batched<NS>(c, u, dt_cell ? dt_cell[k] : dt, rtol, atol,
                                                             h_hist ? h_hist[k] : 0.0);
                        if (r == CELL_CONTINUE) {
                            active = true;
                        } else if (r == CELL_DONE && cell_end<NS>(c, u)) {
#pragma unroll
                            for (int n = 0; n < NS + 3; ++n) trial[n * count + k] = u[n];
                            fail[k] = 0;
                            if (cost) cost[k] = 0;
                        } else {
                            report(st, fail, k, CELL_FAIL);
                        }
                    } else {
                        none = true;
                    }
                }
            }
            drained = __any_sync(0xffffffffu, none);
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (drained) break;
            continue;
        }
        if (active) {
            const int r = cell_attempt<NS>(c, rtol, atol);
            if (r != CELL_CONTINUE) {
                my_attempts += c.attempts;
                double u[NS + 3];
                if (r == CELL_DONE && cell_end<NS>(c, u)) {
#pragma unroll
                    for (int n = 0; n < NS + 3; ++n) trial[n * count + cell] = u[n];
                    fail[cell] = 0;
                    if (h_hist) h_hist[cell] = c.h;
                    if (cost) cost[cell] = c.attempts;
                } else {
                    report(st, fail, cell, r == CELL_MAXSTEPS ? CELL_MAXSTEPS : CELL_FAIL);
                }
                active = false;
            }
        }
    }
    if (my_attempts) atomicAdd(&st->steps, my_attempts);
}

// Launch settings of the batched form, process-wide (hf_set_chem_tuning; the first use
// reads HF_CHEM_MINB and HF_COOP_MIN_BUCKET / HF_COOP=0):
//  * blocks of 64 lanes per SM the queue kernel's register budget is built for: 4 (255
//    registers) or 5, 6, 8 (fewer registers, more resident lanes); the same per-cell code;
//  * the cooperative queue takes cells that used at least 2^coop_min - 1 attempts in the
//    previous call (coop_min = NBUCKET, the default: no cooperative phase, and the kernel
//    instance without it).
std::atomic<int> g_tune_minb{0}, g_tune_coop{0};
void chem_tuning(int* minb, int* coop_min) {
    if (g_tune_minb.load() == 0) {
        const char* e = getenv("HF_CHEM_MINB");
        const int v = e ? atoi(e) : 4;
        int expect = 0;
        g_tune_minb.compare_exchange_strong(expect, (v == 5 || v == 6 || v == 8) ? v : 4);
    }
    if (g_tune_coop.load() == 0) {
        const char* off = getenv("HF_COOP");
        const char* e = getenv("HF_COOP_MIN_BUCKET");
        int v = e ? atoi(e) : 16;
        v = v < 1 ? 1 : (v > 16 ? 16 : v);
        if (off && atoi(off) == 0) v = 16;
        int expect = 0;
        g_tune_coop.compare_exchange_strong(expect, v);
    }
    *minb = g_tune_minb.load();
    *coop_min = g_tune_coop.load();
}

// Work-queue order: counting sort of cells by bucket = floor(log2(cost + 1)) (16
// buckets), most expensive bucket first.  Cells of one bucket keep no particular
// order; each cell's result does not depend on its position.
constexpr int NBUCKET = 16;
__device__ __forceinline__ int cost_bucket(int32_t c) {
    const int b = 31 - __clz((unsigned)c + 1u);
    return min(b, NBUCKET - 1);
}
__global__ void k_order_hist(const int32_t* __restrict__ cost, int64_t count, unsigned long long* __restrict__ bins) {
    __shared__ unsigned int sb[NBUCKET];
    if (threadIdx.x < NBUCKET) sb[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&sb[cost_bucket(max(cost[i], 0))], 1u);
    __syncthreads();
    if (threadIdx.x < NBUCKET && sb[threadIdx.x]) atomicAdd(&bins[threadIdx.x], (unsigned long long)sb[threadIdx.x]);
}
// bins[b] -> start offset of bucket b, descending buckets first; bins[NBUCKET] = the
// cells of the cooperative queue: whole buckets from the costliest down to min_bucket
// while they fit in cap cells (whole buckets, so the choice does not depend on the
// order within a bucket).
__global__ void k_order_scan(unsigned long long* bins, unsigned long long cap, int min_bucket) {
    unsigned long long off = 0, ncoop = 0;
    bool open = true;
    for (int b = NBUCKET - 1; b >= 0; --b) {
        const unsigned long long n = bins[b];
        if (open && b >= min_bucket && ncoop + n <= cap) ncoop += n;
        else open = false;
        bins[b] = off;
        off += n;
    }
    bins[NBUCKET] = ncoop;
}
__global__ void k_order_scatter(const int32_t* __restrict__ cost, int64_t count, unsigned long long* __restrict__ bins,
                                int32_t* __restrict__ order) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long pos = atomicAdd(&bins[cost_bucket(max(cost[i], 0))], 1ull);
        order[pos] = (int32_t)i;
    }
}

template <int NS>
static cudaError_t chem_batched_impl(double* U, int64_t cs, const int64_t* idx, int64_t count, double dt,
                                     const double* dt_dev, const double* dtc, double rtol, double atol,
                                     double* h_hist, int32_t* cost, int32_t* order, unsigned long long* bins,
                                     double* trial, int* fail, DevStatus* st, int sm_count, cudaStream_t s,
                                     int64_t* launches) {
    int minb, coop_min;
    chem_tuning(&minb, &coop_min);
    const bool coop = coop_min < NBUCKET;
    auto kern = coop ? (minb == 8   ? k_chem_batched<NS, 8, true>
                        : minb == 6 ? k_chem_batched<NS, 6, true>
                        : minb == 5 ? k_chem_batched<NS, 5, true>
                                    : k_chem_batched<NS, 4, true>)
                     : (minb == 8   ? k_chem_batched<NS, 8, false>
                        : minb == 6 ? k_chem_batched<NS, 6, false>
                        : minb == 5 ? k_chem_batched<NS, 5, false>
                                    : k_chem_batched<NS, 4, false>);
    const int bs = 64;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bs, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (int64_t)sm_count * per_sm;
    const int64_t need = (count + bs - 1) / bs;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    const unsigned long long* coop_n = nullptr;
    if (cost && order) {
        cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(unsigned long long) * (NBUCKET + 1), s);
        if (e != cudaSuccess) return e;
        const int g = sm_count * 4;
        const unsigned long long cap = (unsigned long long)blocks * (bs / 32) * 4;  // 4 groups per warp
        k_order_hist<<<g, 256, 0, s>>>(cost, count, bins);
        k_order_scan<<<1, 1, 0, s>>>(bins, cap, coop_min);
        k_order_scatter<<<g, 256, 0, s>>>(cost, count, bins, order);
        *launches += 3;
        coop_n = bins + NBUCKET;
    } else {
        order = nullptr;
    }
    kern<<<(unsigned)blocks, bs, 0, s>>>(U, cs, idx, order, count, dt, dt_dev, dtc, rtol, atol, trial, fail, h_hist,
                                         cost, coop_n, st);
    ++*launches;
    return cudaGetLastError();
}
// The batched kernel instances without the cooperative phase use no shared memory: the
// unified L1 / shared storage goes to L1, which caches the lanes' stack frames.
cudaError_t chem_prefer_l1() {
    const void* kernels[] = {(const void*)k_chem_batched<9, 4, false>,  (const void*)k_chem_batched<9, 5, false>,
                             (const void*)k_chem_batched<9, 6, false>,  (const void*)k_chem_batched<9, 8, false>,
                             (const void*)k_chem_batched<10, 4, false>, (const void*)k_chem_batched<10, 5, false>,
                             (const void*)k_chem_batched<10, 6, false>, (const void*)k_chem_batched<10, 8, false>};
    for (const void* k : kernels) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                   (int)cudaSharedmemCarveoutMaxL1);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
cudaError_t launch_chem_batched(int ns, double* U, int64_t cs, const int64_t* idx, int64_t count, double dt,
                                const double* dt_dev, const double* dtc, double rtol, double atol, double* h_hist,
                                int32_t* cost, int32_t* order, unsigned long long* bins, double* trial, int* fail,
                                DevStatus* st, int sm_count, cudaStream_t s, int64_t* launches) {
    return ns == 9 ? chem_batched_impl<9>(U, cs, idx, count, dt, dt_dev, dtc, rtol, atol, h_hist, cost, order, bins,
                                          trial, fail, st, sm_count, s, launches)
                   : chem_batched_impl<10>(U, cs, idx, count, dt, dt_dev, dtc, rtol, atol, h_hist, cost, order, bins,
                                           trial, fail, st, sm_count, s, launches);
}

template <int NS>
static cudaError_t chem_impl(int form, double* U, int64_t cs, const int64_t* idx, int64_t count, double dt,
                             const double* dtc, double rtol, double atol, double* trial, int* fail, DevStatus* st,
                             int sm_count, cudaStream_t s, int64_t* launches, const double* dt_dev) {
    const int bs = 64;
    if (form == HF_CHEM_PLAIN) {
        k_chem_plain<NS><<<(unsigned)((count + bs - 1) / bs), bs, 0, s>>>(U, cs, idx, count, dt, dt_dev, dtc, rtol, atol,
                                                                          trial, fail, st);
    } else {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chem_persistent<NS>, bs, 0);
        if (per_sm < 1) per_sm = 1;
        int64_t blocks = (int64_t)sm_count * per_sm;
        const int64_t need = (count + bs - 1) / bs;
        if (blocks > need) blocks = need;
        if (blocks < 1) blocks = 1;
        k_chem_persistent<NS><<<(unsigned)blocks, bs, 0, s>>>(U, cs, idx, count, dt, dtc, rtol, atol, trial, fail, st);
    }
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_chem(int ns, int form, double* U, int64_t cs, const int64_t* idx, int64_t count, double dt,
                        const double* dtc, double rtol, double atol, double* trial, int* fail, DevStatus* st,
                        int sm_count, cudaStream_t s, int64_t* launches, const double* dt_dev) {
    return ns == 9 ? chem_impl<9>(form, U, cs, idx, count, dt, dtc, rtol, atol, trial, fail, st, sm_count, s, launches,
                                  dt_dev)
                   : chem_impl<10>(form, U, cs, idx, count, dt, dtc, rtol, atol, trial, fail, st, sm_count, s, launches,
                                   dt_dev);
}
cudaError_t launch_chem_commit(int ns, double* U, int64_t cs, const int64_t* idx, int64_t count, const double* trial,
                               cudaStream_t s, int64_t* launches) {
    const int bs = 128;
    if (ns == 9) k_chem_commit<9><<<(unsigned)((count + bs - 1) / bs), bs, 0, s>>>(U, cs, idx, count, trial);
    else k_chem_commit<10><<<(unsigned)((count + bs - 1) / bs), bs, 0, s>>>(U, cs, idx, count, trial);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- tagging
// BlockAMR::ErrorEst (BlockAMR.cpp:170-200) per valid cell: tag box (optionally moving),
// relative pressure and temperature jumps to the face neighbours, fuel consumption
// rate -w_H2 W_H2 / rho, plus the relative density jump (extension, density_tag > 0).
template <int NS>
__global__ void k_tag(Level L, const hf_patch* __restrict__ patches, const double* __restrict__ U, double t,
                      hf_tag_criteria c, uint8_t* __restrict__ tags, const int64_t* __restrict__ tag_off,
                      DevStatus* st) {
    constexpr int NV = NS + 3;
    const hf_patch P = patches[blockIdx.y];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)P.nx * P.ny) return;
    const int li = (int)(k % P.nx), lj = (int)(k / P.nx);
    const int i = P.ilo + li, j = P.jlo + lj;
    const double x = L.xlo + (i + 0.5) * L.dx - c.velocity[0] * t;
    const double y = L.ylo + (j + 0.5) * L.dy - c.velocity[1] * t;
    bool marked = c.has_box && x >= c.box[0] && x <= c.box[1] && y >= c.box[2] && y <= c.box[3];
    if (!c.box_only) {
        auto load = [&](int a, int b, double* q) {
#pragma unroll
            for (int n = 0; n < NV; ++n)
                q[n] = U[P.offset + (int64_t)n * P.comp_stride + (int64_t)(b + P.ng) * P.pitch + (a + P.ng)];
        };
        double q[NV];
        load(li, lj, q);
        Props p;
        bool ok = properties<NS>(q, p, 1000.0);
        double rho = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) rho += q[s];
        for (int d = 0; d < 2 && ok; ++d) {
            const int di = d == 0, dj = d == 1;
            double ql[NV], qr[NV];
            load(li - di, lj - dj, ql);
            load(li + di, lj + dj, qr);
            Props pl, pr;
            ok = properties<NS>(ql, pl, p.T) && properties<NS>(qr, pr, p.T);
            if (!ok) break;
            const double jump = fmax(fabs(pl.p - p.p) / fmin(pl.p, p.p), fabs(pr.p - p.p) / fmin(pr.p, p.p));
            const double temp = fmax(fabs(pl.T - p.T) / fmin(pl.T, p.T), fabs(pr.T - p.T) / fmin(pr.T, p.T));
            marked = marked || jump > c.pressure_tag || temp > c.temperature_tag;
            if (c.density_tag > 0.0) {
                double rl = 0.0, rr = 0.0;
#pragma unroll
                for (int s = 0; s < NS; ++s) { rl += ql[s]; rr += qr[s]; }
                const double rj = fmax(fabs(rl - rho) / fmin(rl, rho), fabs(rr - rho) / fmin(rr, rho));
                marked = marked || rj > c.density_tag;
            }
        }
        if (!ok) {
            atomicOr(&st->flags, ST_STAGE_BAD);
            atomicMin(&st->bad_cell, (unsigned long long)(tag_off[blockIdx.y] + k));
        } else if (c.chemistry) {
            double C[NS], w[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                C[s] = q[s] * INVW.v[s];
                w[s] = 0.0;
            }
            KinCtx<NS> kc;
            kin_setup<NS>(p.T, C, kc);
            all_rates<NS>(kc, C, w, std::make_index_sequence<NR>{});
            marked = marked || -w[0] * D_MW.v[0] / rho > c.fuel_rate_tag;
        }
    }
    tags[tag_off[blockIdx.y] + k] = marked ? 1 : 0;
}
cudaError_t launch_tag(int ns, const Level& L, const hf_patch* patches_dev, const hf_patch* patches_host, int npatch,
                       const double* U, double time, const hf_tag_criteria& c, uint8_t* tags, const int64_t* tag_off,
                       DevStatus* st, cudaStream_t s, int64_t* launches) {
    int64_t mx = 1;
    for (int p = 0; p < npatch; ++p) mx = max(mx, (int64_t)patches_host[p].nx * patches_host[p].ny);
    dim3 grid((unsigned)((mx + 127) / 128), (unsigned)npatch);
    if (ns == 9) k_tag<9><<<grid, 128, 0, s>>>(L, patches_dev, U, time, c, tags, tag_off, st);
    else k_tag<10><<<grid, 128, 0, s>>>(L, patches_dev, U, time, c, tags, tag_off, st);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- allocation-free entry
// Scratch of hf_chem_advance_noalloc: a file-scope device array of fixed size, so the
// entry point allocates nothing.  Host code reaches it only through the device address
// that cudaGetSymbolAddress returns (the symbol itself is a host-side stand-in).
struct NoAllocScratch {
    DevStatus st;
    int fail[HF_NOALLOC_MAX_CELLS];
    double trial[(NS_MAX + 3) * HF_NOALLOC_MAX_CELLS];
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

}  // namespace hf

namespace hf {
__global__ void k_fastmath(const double* __restrict__ x, int64_t n, double* __restrict__ e, double* __restrict__ ep,
                           double* __restrict__ em, double* __restrict__ l) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    e[i] = fexp(v);
    fexp_pair(v, ep[i], em[i]);
    l[i] = flog(v);
}
}  // namespace hf
extern "C" hf_status hf_fastmath_eval(const double* x, int64_t n, double* exp_out, double* pair_pos, double* pair_neg,
                                      double* log_out, void* stream) {
    if (n < 0 || !x || !exp_out || !pair_pos || !pair_neg || !log_out) return HF_ERR_ARG;
    if (n == 0) return HF_OK;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    hf::k_fastmath<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x, n, exp_out, pair_pos, pair_neg,
                                                                              log_out);
    return cudaGetLastError() == cudaSuccess ? HF_OK : HF_ERR_CUDA;
}
extern "C" hf_status hf_set_chem_tuning(int32_t blocks_per_sm, int32_t coop_min_bucket) {
    if (blocks_per_sm < 0 || coop_min_bucket < 0 || coop_min_bucket > 16 ||
        (blocks_per_sm && blocks_per_sm != 4 && blocks_per_sm != 5 && blocks_per_sm != 6 && blocks_per_sm != 8))
        return HF_ERR_ARG;
    int m = 0, c = 0;
    hf::chem_tuning(&m, &c);  // settle the defaults first
    if (blocks_per_sm) hf::g_tune_minb.store(blocks_per_sm);
    if (coop_min_bucket) hf::g_tune_coop.store(coop_min_bucket);
    return HF_OK;
}
extern "C" void hf_get_chem_tuning(int32_t* blocks_per_sm, int32_t* coop_min_bucket) {
    int m = 0, c = 0;
    hf::chem_tuning(&m, &c);
    if (blocks_per_sm) *blocks_per_sm = m;
    if (coop_min_bucket) *coop_min_bucket = c;
}

#include <mutex>

namespace {
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
hf::NoAllocScratch* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Once per device, with that device current: the array's device address, and the
// rate constants if no context has loaded them on this device yet.
cudaError_t noalloc_setup(int dev, hf::NoAllocScratch** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        hf::NoAllocScratch* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, hf::g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        double a0 = 0.0;
        e = cudaMemcpyFromSymbol(&a0, hf::c_A, sizeof(double));
        if (e != cudaSuccess) return e;
        if (a0 == 0.0) {
            e = hf::chem_set_rate_scale(nullptr);
            if (e != cudaSuccess) return e;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}
}  // namespace

extern "C" hf_status hf_chem_advance_noalloc(int nspecies, double* U, int64_t comp_stride, const int64_t* cell_index,
                                             int64_t count, double dt, const double* dt_cell, double rtol, double atol,
                                             int64_t* first_failed, void* stream) {
    using namespace hf;
    if (first_failed) *first_failed = -1;
    if ((nspecies != 9 && nspecies != 10) || !U || count < 0 || count > HF_NOALLOC_MAX_CELLS ||
        (!cell_index && comp_stride < count) || (!dt_cell && (!(dt > 0) || !isfinite(dt))) || !(rtol > 0) ||
        !(atol > 0))
        return HF_ERR_ARG;
    if (count == 0) return HF_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return HF_ERR_CUDA;
    NoAllocScratch* S = nullptr;
    if (noalloc_setup(dev, &S) != cudaSuccess) return HF_ERR_CUDA;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(&S->st, 0, sizeof(DevStatus), s) != cudaSuccess ||
        cudaMemsetAsync(&S->st.bad_cell, 0xff, sizeof(unsigned long long), s) != cudaSuccess)
        return HF_ERR_CUDA;
    int64_t launches = 0;
    if (launch_chem(nspecies, HF_CHEM_PLAIN, U, comp_stride, cell_index, count, dt, dt_cell, rtol, atol, S->trial,
                    S->fail, &S->st, 1, s, &launches) != cudaSuccess)
        return HF_ERR_CUDA;
    DevStatus h;
    if (cudaMemcpyAsync(&h, &S->st, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return HF_ERR_CUDA;
    if (h.flags & (ST_CHEM_FAIL | ST_MAXSTEPS)) {
        if (first_failed) *first_failed = (int64_t)h.bad_cell;
        return (h.flags & ST_CHEM_FAIL) ? HF_ERR_CHEM_FAIL : HF_ERR_MAXSTEPS;
    }
    if (launch_chem_commit(nspecies, U, comp_stride, cell_index, count, S->trial, s, &launches) != cudaSuccess)
        return HF_ERR_CUDA;
    return HF_OK;
}
