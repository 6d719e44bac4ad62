// Internal declarations shared by the translation units of libhyperflow_gpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/hyperflow_gpu.h"

namespace hf {

// Device-side status of one stage / reduction launch.
struct DevStatus {
    unsigned int flags;
    unsigned int pad;
    unsigned long long bad_cell;   // lowest failing linear index (atomicMin), ~0 = none
    unsigned long long rate_bits;  // CFL: max rate as the bits of a non-negative double
    unsigned long long counter;    // work-queue head / generic counter
    unsigned long long coop_counter;  // head of the batched chemistry's cooperative queue
    unsigned long long steps;      // integrator steps (accepted + rejected)
    unsigned long long repairs;
    unsigned long long coop_cells;  // cells the batched chemistry took in groups of 8 lanes
    // Set when a step of a device-resident multi-step run failed; the step kernels of
    // the later steps of that run return at entry.  Never set outside such runs (the
    // per-step reset of the status block leaves it alone: it is the last member).
    unsigned int abort_run;
    unsigned int pad2;
};
enum : unsigned int {
    ST_STAGE_BAD = 1u,    // a stage output cell is inadmissible
    ST_NEGATIVE = 2u,     // a stage output cell has a negative partial density
    ST_COMBINE_BAD = 4u,  // a Heun-combined cell is inadmissible
    ST_FACE_BAD = 8u,     // a face fell back to an inadmissible cell state
    ST_MATERIAL = 16u,    // negative species beyond roundoff (repairRoundoff throws)
    ST_TIMEOUT = 32u,     // a bounded wait gave up
    ST_CHEM_FAIL = 64u,
    ST_MAXSTEPS = 128u,
    ST_BAD_INPUT = 256u,
};

struct Level {  // device copy of hf_level
    int nx, ny;
    int periodic[2], lo[2], hi[2];
    double dx, dy, xlo, ylo, wedge_start;
    double inlet[13];
};
inline Level make_level(const hf_level& l) {
    Level d{};
    d.nx = l.nx; d.ny = l.ny;
    for (int k = 0; k < 2; ++k) { d.periodic[k] = l.periodic[k]; d.lo[k] = l.bc_lo[k]; d.hi[k] = l.bc_hi[k]; }
    d.dx = l.dx; d.dy = l.dy; d.xlo = l.xlo; d.ylo = l.ylo; d.wedge_start = l.wedge_start;
    for (int n = 0; n < 13; ++n) d.inlet[n] = l.inlet[n];
    return d;
}

// Counter updates from the host stepper (hf_abi.cu)
void ctx_add_counters(hf_ctx* ctx, int64_t first_order_stages, int64_t retries);
void ctx_add_repairs(hf_ctx* ctx, int64_t repairs);
void ctx_add_coop(hf_ctx* ctx, int64_t coop_cells);
// The message hf_last_error returns, for failures found outside hf_abi.cu
void ctx_set_error(hf_ctx* ctx, const char* msg);
// Counters and device time of work run outside the ABI entry points (graph-captured steps)
void ctx_add_launches(hf_ctx* ctx, int64_t kernels, int64_t chem_cells, int64_t chem_steps);
bool ctx_timing_enabled(const hf_ctx* ctx);
void ctx_add_timing(hf_ctx* ctx, double flux_ms, double chem_ms, double other_ms, int64_t flux_launches,
                    int64_t chem_launches, int64_t other_launches);

// Launch wrappers (hf_flux.cu)
cudaError_t launch_fill(int ns, const Level& L, const hf_patch* patches_host, const hf_patch* patches_dev,
                        int npatch, double* U, cudaStream_t s, int64_t* launches);
// hdev (nullable): read the stage length h from device memory instead of the argument
cudaError_t launch_flux_plain(int ns, const Level& L, const hf_patch& P, int pidx, const double* Uin,
                              const double* Uold, double* Uout, double* fx, double* fy, double h,
                              int first_order, int64_t cell_base, DevStatus* st, cudaStream_t s,
                              int64_t* launches, const double* hdev = nullptr);
// The plain form over all patches of a level in 3 launches; off_dev[3p..3p+2] = patch p's
// x-face offset in FX, y-face offset in FY and first cell index (face arrays packed per
// patch, component-major within a patch, as launch_flux_plain writes them).
cudaError_t launch_flux_multi(int ns, const Level& L, const hf_patch* patches_host, const hf_patch* patches_dev,
                              int npatch, const int64_t* off_dev, const double* Uin, const double* Uold, double* Uout,
                              double* FX, double* FY, double h, int first_order, DevStatus* st, cudaStream_t s,
                              int64_t* launches, const double* hdev = nullptr);
// hdev (nullable): read the stage length h from device memory instead of the argument
cudaError_t launch_flux_fused(int ns, const Level& L, const hf_patch& P, const void* tmap, const double* Uin,
                              const double* Uold, double* Uout, double h, const double* hdev, int first_order,
                              int64_t cell_base, DevStatus* st, cudaStream_t s, int64_t* launches);
cudaError_t launch_dt_from_rate(const DevStatus* st, double cfl, double* dt, cudaStream_t s, int64_t* launches);
bool make_tensor_map(void* tmap, const double* base, const hf_patch& P, int nv);
cudaError_t launch_combine(int ns, const hf_patch& P, const double* Uold, double* U, int64_t cell_base,
                           DevStatus* st, cudaStream_t s, int64_t* launches);
// Every patch of a level in one launch; base_dev[p] = patch p's first cell index.
cudaError_t launch_validate_multi(int ns, const hf_patch* patches_host, const hf_patch* patches_dev, int npatch,
                                  const int64_t* base_dev, const double* U, DevStatus* st, cudaStream_t s,
                                  int64_t* launches);
cudaError_t launch_cfl_multi(int ns, const Level& L, const hf_patch* patches_host, const hf_patch* patches_dev,
                             int npatch, const int64_t* base_dev, const double* U, DevStatus* st, cudaStream_t s,
                             int64_t* launches);
cudaError_t launch_validate(int ns, const hf_patch& P, const double* U, int64_t cell_base, DevStatus* st,
                            cudaStream_t s, int64_t* launches);
cudaError_t launch_cfl(int ns, const Level& L, const hf_patch& P, const double* U, DevStatus* st,
                       cudaStream_t s, int64_t* launches);
cudaError_t launch_properties(int ns, const double* q, int64_t stride, int64_t count, double* p, double* a,
                              double* T, int32_t* status, DevStatus* st, cudaStream_t s, int64_t* launches);
cudaError_t launch_hllc(int ns, const double* l, const double* r, const double* pl, const double* pr,
                        int64_t stride, int64_t count, int dir, double* f, cudaStream_t s, int64_t* launches);
// Regions (4 int32 each, fine level indices, in device memory) of one fine patch from one
// coarse patch, one launch; max_coarse_cells bounds each region's coarsened box.
cudaError_t launch_interp_regions(int ns, const hf_patch& C, const double* Uc, const hf_patch& F, double* Uf,
                                  const int32_t* regions_dev, int nregions, int64_t max_coarse_cells, cudaStream_t s,
                                  int64_t* launches);
cudaError_t launch_interp(int ns, const hf_patch& C, const double* Uc, const hf_patch& F, double* Uf,
                          const int32_t* region, cudaStream_t s, int64_t* launches);

// Chemistry (hf_chem.cu)
cudaError_t chem_set_rate_scale(const double* scale);
// L1 preference of the batched chemistry kernels without shared memory (once per context)
cudaError_t chem_prefer_l1();

// Discrete adjoint of 0D chemistry runs (hf_adjoint.cu).  Scratch arrays are
// [slot][component][chunk] with chunk the stride.
struct AdjointArgs {
    const double* U0;
    int64_t cs, count, i0, chunk;  // input stride, total cells, first cell and cells of this launch
    double dt, dT, rtol, atol;
    int ncalls, K, objective, cap, backward;
    double* ckpt;     // [ceil(ncalls/K)][NV][chunk]
    double* seg;      // [K+1][NV][chunk]
    double* tape;     // [cap][NS+1][chunk]
    int32_t* nstep;   // [K][chunk]
    uint32_t* clipm;  // [K][chunk]
    double* J;        // [count]
    double* dJdp;     // [NR][count]
    double* dJdy0;    // [NS-1][count] or null
    int* fail;        // [count]
    DevStatus* st;
};
cudaError_t adjoint_set_rate_scale(const double* scale);
// Adjoint of one chemistry call per cell of a ghosted patch (cells [i0, i0+chunk));
// tape: [cap][NS+1][chunk] scratch; pcell: [NR][nx*ny] accumulators.
cudaError_t launch_chem_call_adjoint(int ns, const hf_patch& P, const double* U, const double* ubar_out,
                                     double* ubar_in, double dt, double rtol, double atol, double* tape, int cap,
                                     int64_t i0, int64_t chunk, double* pcell, DevStatus* st, cudaStream_t s,
                                     int64_t* launches);
// Adjoint of one Euler stage (hf_flux_adjoint.cu): U is the ghost-filled stage input,
// outbar the cotangent of the stage output, ch the stage's weight in the output (1, or
// 1/2 with a Heun combination), h the stage length; inbar receives the interior
// cotangent of U.  FAx / FAy: 4 NV (nx+1) ny and 4 NV nx (ny+1) doubles; UG: a
// ghosted array of the patch's layout.
cudaError_t launch_stage_adjoint(int ns, const Level& L, const hf_patch& P, const double* U, const double* outbar,
                                 double ch, double h, int first_order, double* FAx, double* FAy, double* UG,
                                 double* inbar, DevStatus* st, cudaStream_t s, int64_t* launches);
size_t adjoint_bytes_per_cell(int ns, int ncalls, int K, int cap);
cudaError_t launch_chem_adjoint(int ns, const AdjointArgs& a, cudaStream_t s, int64_t* launches);
// dt_dev (nullable, plain form): read the interval from device memory instead of dt
cudaError_t launch_chem(int ns, int form, double* U, int64_t comp_stride, const int64_t* cell_index,
                        int64_t count, double dt, const double* dt_cell, double rtol, double atol,
                        double* trial, int* fail, DevStatus* st, int sm_count, cudaStream_t s,
                        int64_t* launches, const double* dt_dev = nullptr);
// dt_dev (nullable): read the interval from device memory instead of dt
// bins: CHEM_BINS unsigned long long of device scratch (cost buckets and the size of the
// cooperative queue)
constexpr int CHEM_BINS = 32;
cudaError_t launch_chem_batched(int ns, double* U, int64_t cs, const int64_t* idx, int64_t count, double dt,
                                const double* dt_dev, const double* dtc, double rtol, double atol, double* h_hist,
                                int32_t* cost, int32_t* order, unsigned long long* bins, double* trial, int* fail,
                                DevStatus* st, int sm_count, cudaStream_t s, int64_t* launches);
cudaError_t launch_tag(int ns, const Level& L, const hf_patch* patches_dev, const hf_patch* patches_host, int npatch,
                       const double* U, double time, const hf_tag_criteria& c, uint8_t* tags, const int64_t* tag_off,
                       DevStatus* st, cudaStream_t s, int64_t* launches);

// Block-AMR level operations (hf_amr.cu)
size_t totals_scratch_bytes(int nv);
cudaError_t launch_totals(const hf_patch* patches_dev, int npatch, int64_t total, const double* U, const uint8_t* mask,
                          int nv, double vol, int absolute, void* scratch, double* out_dev, cudaStream_t s,
                          int64_t* launches);
cudaError_t launch_average_down(const hf_patch* fine_dev, const hf_patch* fine_host, int nfine, const double* Uf,
                                const hf_patch* coarse_dev, int ncoarse, double* Uc, int nv, cudaStream_t s,
                                int64_t* launches);
cudaError_t launch_reflux(const Level& L, const hf_patch* coarse_dev, const hf_patch* coarse_host, int ncoarse,
                          const int64_t* cfx_off, const int64_t* cfy_off, const double* fxc, const double* fyc,
                          double* Uc, const hf_patch* fine_dev, const hf_patch* fine_host, int nfine,
                          const int64_t* ffx_off, const int64_t* ffy_off, const double* fxf, const double* fyf,
                          int* cover, double h, int nv, cudaStream_t s, int64_t* launches,
                          const double* hdev = nullptr);
cudaError_t launch_chem_commit(int ns, double* U, int64_t comp_stride, const int64_t* cell_index,
                               int64_t count, const double* trial, cudaStream_t s, int64_t* launches);

// Composite roundoff repair (hf_amr.cu): repairRoundoff over the leaf cells of several
// levels.  Each level gives its patch table and first-cell offsets (device), an
// optional leaf mask over its patch-packed cells (null: every cell is a leaf), its
// state and its cell volume; npatch and max_cells (the largest patch's cell count) are
// host values for the launch shape.
constexpr int REPAIR_CAP = 2048;  // negative entries summed in the reference's order
constexpr int REPAIR_MAX_LEVELS = 8;
struct RepairLevel {
    const hf_patch* patches;
    const int64_t* base;
    const uint8_t* leaf;
    double* U;
    int npatch;
    int64_t max_cells;
    double vol;
};
struct RepairLevels {
    RepairLevel lev[REPAIR_MAX_LEVELS];
    int nlev;
};
struct RepairScratch {  // device memory, cleared by every launch_composite_repair
    unsigned long long peak_bits[16];
    unsigned long long mass_bits[16];
    double deficit[16];          // atomic deficit sums (used past REPAIR_CAP entries)
    unsigned long long count;    // negative entries found
    unsigned long long donor[16];
    unsigned long long key[REPAIR_CAP];  // species << 60 | level << 52 | cell
    double val[REPAIR_CAP];              // deficit of the entry (-value x volume)
};
size_t repair_scratch_bytes();
// Flags ST_MATERIAL in st and adds the number of zeroed values to st->repairs.
cudaError_t launch_composite_repair(int ns, const RepairLevels& R, RepairScratch* rs, DevStatus* st, cudaStream_t s,
                                    int64_t* launches);

}  // namespace hf
