/* hyperflow_gpu.h - C ABI of the GB300 reacting-Euler step (HyperFlow V3 hot path).
 *
 * The reference has no C ABI: its time stepper (BlockAMR, HyperFlow_V3/src/BlockAMR.cpp)
 * calls C++ functions per block.  Each entry point below replaces one of them and
 * keeps its argument meaning and its error behaviour, with return codes in place of
 * exceptions.  Conventions:
 *   - A cell state is NV = NS+3 doubles: rhoY_0..rhoY_{NS-1}, rho*u, rho*v, rho*E
 *     (HyperFlow_V3/src/solver.hpp:17-25).  NS = 9 for H2_Li.yaml; NS = 10 with the
 *     inert AR extension species.
 *   - Grid data is structure-of-arrays FP64 in caller-owned DEVICE memory: component n
 *     of cell (i, j) of a patch lives at base[offset + n*comp_stride + (j+ng)*pitch + (i+ng)],
 *     i in [-ng, nx+ng), j in [-ng, ny+ng) (valid cells plus ng ghost layers).
 *   - Batches of cells (chemistry, properties) are SoA with a component stride.
 *   - Every call is stream-ordered on the caller's cudaStream_t (passed as void*; NULL =
 *     legacy default stream).  Calls that report a status synchronise that stream.
 *   - Device code never traps; failures are flags the host reads after the stream syncs.
 *   - One hf_ctx per host thread; a context is not re-entrant (chemistry_batch.hpp:6-7).
 */
#ifndef HYPERFLOW_GPU_H
#define HYPERFLOW_GPU_H
#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define HF_EXPORT __attribute__((visibility("default")))
#else
#define HF_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hf_status {
    HF_OK = 0,
    HF_ERR_INADMISSIBLE = 1, /* std::domain_error of properties()/validate() (physics.cpp:8,13) */
    HF_ERR_CHEM_FAIL = 2,    /* a chemistry cell failed (chemistry_batch.cpp:40-49); see first_failed */
    HF_ERR_MAXSTEPS = 3,     /* chemistry step limit reached (CVodeSetMaxNumSteps(5000), chemistry.cpp:25) */
    HF_ERR_ARG = 4,          /* std::invalid_argument */
    HF_ERR_CUDA = 5,         /* a CUDA runtime call failed */
    HF_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
    HF_ERR_NEGATIVE = 7,     /* materially negative species after a stage (BlockAMR.cpp:320-321) */
    HF_ERR_FACE = 8,         /* a face fell back to an inadmissible cell state: properties() throws
                                inside the flux loop (BlockAMR.cpp:223), which only run()'s
                                rollback catches */
    HF_ERR_COMBINE = 9       /* the Heun combination is inadmissible (validate, BlockAMR.cpp:269) */
} hf_status;

/* Boundary kinds: the strings of the reference's case JSON (BlockAMR.cpp:38-59). */
enum { HF_BC_REFLECTING = 0, HF_BC_TRANSMISSIVE = 1, HF_BC_INFLOW = 2, HF_BC_WEDGE = 3 };

/* Chemistry forms. */
enum { HF_CHEM_PLAIN = 0,      /* one thread per cell, one launch (the drop-in form) */
       HF_CHEM_PERSISTENT = 1  /* persistent launch pulling cells from a device work queue */ };

/* Flux forms. */
enum { HF_FLUX_PLAIN = 0,      /* face kernels + update kernel, one launch set per patch; needs
                                  filled ghosts (hf_fill_ghosts) */
       HF_FLUX_FUSED = 1       /* one fused kernel per level: TMA tile + halo in shared memory,
                                  domain boundaries resolved while loading (no ghost fill needed
                                  for a level made of one patch that covers the domain) */ };

typedef struct hf_ctx hf_ctx;

/* A level: the domain box at this level and its boundary description
 * (BlockAMR.cpp:48-59; FlowBoundary.hpp:8-11; geometry of BlockAMR.cpp:211,225). */
typedef struct hf_level {
    int32_t nx, ny;            /* domain cells at this level; domain small end is (0,0) */
    double dx, dy;             /* cell size */
    double xlo, ylo;           /* ProbLo */
    int32_t periodic[2];
    int32_t bc_lo[2], bc_hi[2];/* HF_BC_* per direction; WEDGE only for bc_lo[1] */
    double inlet[13];          /* fixed inflow state ("fresh"), first NV entries used */
    double wedge_start;        /* x of the wedge tip (bc_lo[1] == HF_BC_WEDGE) */
} hf_level;

/* A patch (an AMReX box of the level) inside a level buffer. */
typedef struct hf_patch {
    int32_t ilo, jlo;          /* level index of the first valid cell */
    int32_t nx, ny;            /* valid cells */
    int32_t ng;                /* ghost layers stored (>= 2) */
    int32_t pad_;
    int64_t pitch;             /* elements between rows, >= nx + 2 ng (even for HF_FLUX_FUSED) */
    int64_t comp_stride;       /* elements between components, >= pitch*(ny+2 ng) (even for FUSED) */
    int64_t offset;            /* element offset of this patch's storage in the level buffer */
} hf_patch;

/* Counters kept by a context (BlockAMR.cpp:426-438 summary fields). */
typedef struct hf_counters {
    int64_t first_order_stages;   /* positivity_first_order_stages */
    int64_t roundoff_repairs;     /* roundoff_redistributions */
    int64_t retries;              /* retries (host stepper) */
    int64_t chem_cell_calls;      /* chemistry_cell_calls */
    int64_t chem_steps;           /* accepted + rejected integrator steps */
    int64_t kernel_launches;      /* kernels launched by this context */
    int64_t chem_coop_cells;      /* cells the batched chemistry integrated in groups of 8 lanes
                                     (extension: the reference integrates one cell per thread) */
} hf_counters;

/* ---- context (replaces Cantera::newSolution(mechanism) + ChemistryBatch construction,
 *      BlockAMR.cpp:29-30, chemistry_batch.cpp:9-20) ---- */
/* mechanism: NULL, "H2_Li", a path ending in "H2_Li.yaml" (9 species), or "H2_Li+AR"
 * (10 species, inert AR extension).  device: CUDA ordinal. */
HF_EXPORT hf_status hf_init(const char* mechanism, int device, hf_ctx** out);
HF_EXPORT void hf_destroy(hf_ctx* ctx);
HF_EXPORT int hf_nspecies(const hf_ctx* ctx);
HF_EXPORT const char* hf_last_error(const hf_ctx* ctx);
HF_EXPORT void hf_get_counters(const hf_ctx* ctx, hf_counters* out);
/* Device time per kernel class, measured with CUDA events recorded on the caller's stream
 * around each launch while enabled (enable != 0 also resets the sums): ms[0] flux stages
 * (hf_flux_update), ms[1] chemistry (hf_chem_advance), ms[2] ghost fill and reductions.
 * launches[k] counts the launches of each class.  Extension: the reference keeps host wall
 * timers only (flow_seconds / chemistry_seconds, BlockAMR.cpp:267-284,435). */
HF_EXPORT void hf_set_timing(hf_ctx* ctx, int enable);
HF_EXPORT void hf_get_timing(const hf_ctx* ctx, double ms[3], int64_t launches[3]);
/* Multiply each reaction's pre-exponential factor(s) by scale[r] (21 entries; NULL resets).
 * Used for d/d ln A_k sensitivity checks; not in the reference.  The factors live in
 * constant memory, one copy per device and process: the scale applies to every context
 * on the current device and to hf_chem_advance_noalloc until it is reset. */
HF_EXPORT hf_status hf_set_rate_scale(hf_ctx* ctx, const double* scale);
/* Launch settings of the batched chemistry form, process-wide (no counterpart in the
 * reference; set by an autotuner, hyperflow_gb300/tune.py): blocks_per_sm, the resident
 * 64-lane blocks per SM its register budget is built for (4, 5, 6 or 8; fewer registers
 * per lane as it grows; the same per-cell code); coop_min_bucket b (1..16): cells that
 * took at least 2^b - 1 step attempts in the previous call are integrated by groups of 8
 * lanes (16: never).  0 leaves a setting unchanged.  Results are the same to rounding
 * for any setting; with a fixed setting they are reproducible bit for bit.  The first
 * use reads HF_CHEM_MINB and HF_COOP_MIN_BUCKET (HF_COOP=0: 16); defaults 4 and 16. */
HF_EXPORT hf_status hf_set_chem_tuning(int32_t blocks_per_sm, int32_t coop_min_bucket);
HF_EXPORT void hf_get_chem_tuning(int32_t* blocks_per_sm, int32_t* coop_min_bucket);

/* Measured FP64 FMA throughput of the device (GFLOP/s, FMA = 2 flops): the FP64 roofline
 * denominator of the chemistry and flux kernels.  Independent FMA chains on every SM, best
 * of three timed launches after a warm-up.  Measurement utility; no reference counterpart. */
HF_EXPORT hf_status hf_fp64_peak(hf_ctx* ctx, double* gflops, void* stream);

/* The chemistry kernels' table-driven exponential and logarithm on n device values:
 * exp_out = exp(x); pair_pos, pair_neg = exp(x), exp(-x) from the paired form;
 * log_out = log(x).  Check utility (within a few ulp of the correctly rounded values);
 * no reference counterpart. */
HF_EXPORT hf_status hf_fastmath_eval(const double* x, int64_t n, double* exp_out, double* pair_pos, double* pair_neg,
                                     double* log_out, void* stream);

/* ---- EOS / flux primitives on batches (physics.cpp:4-48) ---- */
/* properties(): q is SoA [NV][stride] device memory with count cells; writes p, a, T and
 * status[i] (0 ok, 1 inadmissible).  Returns HF_OK or HF_ERR_INADMISSIBLE if any failed. */
HF_EXPORT hf_status hf_properties(hf_ctx* ctx, const double* q, int64_t stride, int64_t count, double* p,
                        double* a, double* T, int32_t* status, void* stream);
/* hllc(): left/right SoA [NV][stride], dir 0 = x (n = mx), 1 = y (n = my); props_l/r are
 * SoA [3][stride] (p, a, T).  flux SoA [NV][stride]. */
HF_EXPORT hf_status hf_hllc(hf_ctx* ctx, const double* left, const double* right, const double* props_l,
                  const double* props_r, int64_t stride, int64_t count, int dir, double* flux,
                  void* stream);

/* ---- ghost fill (BlockAMR::fill, FlowBoundary::operator(), BlockAMR.cpp:137-146,
 *      FlowBoundary.hpp:12-36) on one level: same-level exchange (incl. periodic images),
 *      then physical boundaries in AMReX order (faces, then corners). ---- */
HF_EXPORT hf_status hf_fill_ghosts(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch,
                         double* U, void* stream);

/* ---- coarse -> fine interpolation (ConservativeInterp::interp, ConservativeInterp.cpp:18-51).
 * For every coarse cell (ci, cj) of the coarse index box [cilo..cihi] x [cjlo..cjhi]
 * (fine box coarsened), reads coarse cell and its 4 neighbours from the coarse patch and
 * writes the children that fall inside the fine target region [filo..fihi] x [fjlo..fjhi]
 * (fine level index) of the fine patch. ---- */
HF_EXPORT hf_status hf_interp_coarse_to_fine(hf_ctx* ctx, const hf_patch* coarse, const double* Uc,
                                   const hf_patch* fine, double* Uf, const int32_t region[4],
                                   void* stream);

/* ---- one Euler stage of one level (BlockAMR::euler body, BlockAMR.cpp:210-243) plus the
 * Heun combine of BlockAMR::flow (BlockAMR.cpp:268-269) when U_old is non-NULL:
 *   U_out = [U_old + E(U_in)]/2  (U_old given)   or   U_out = E(U_in),
 *   E(q) = q - h/dx (Fx(i+1)-Fx(i)) - h/dy (Fy(j+1)-Fy(j)).
 * U_in must have filled ghosts for HF_FLUX_PLAIN.  fx/fy (nullable) receive face fluxes
 * (x faces: [NV][ny][nx+1] per patch, y faces [NV][ny+1][nx]) for reflux.
 * first_order: face states qb/qc (BlockAMR.cpp:220).  Each updated cell is validated
 * (BlockAMR.cpp:257); returns HF_ERR_INADMISSIBLE (-> first-order redo) when a stage
 * output is inadmissible, HF_ERR_NEGATIVE when a species went negative by more than
 * roundoff (also -> first-order redo), HF_ERR_FACE or HF_ERR_COMBINE (-> rollback), and
 * repairs roundoff-negative species like repairRoundoff (BlockAMR.cpp:299-334).
 * HF_FLUX_FUSED requires npatch == 1, a patch covering the level domain, ng even, and
 * fx == fy == NULL.
 * bad_cell (nullable) receives the lowest failing linear cell index or -1. ---- */
HF_EXPORT hf_status hf_flux_update(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch,
                         const double* U_in, const double* U_old, double* U_out, double* fx,
                         double* fy, double h, int first_order, int form, int64_t* bad_cell,
                         void* stream);

/* ---- chemistry (ChemistryBatch::advance, chemistry_batch.cpp:21-50 over
 * Chemistry::advance, chemistry.cpp:55-76).  U is SoA [NV][stride] device memory holding
 * count cells (or a level buffer when cell_index is given: cell_index[i] is the element
 * index of cell i's component 0, components comp_stride apart).  dt: one interval for all,
 * or dt_cell[i] per cell when dt_cell is non-NULL (extension).  rtol/atol: 1e-8/1e-15 in
 * the reference.  All-or-nothing: on failure U is unchanged and *first_failed is the lowest
 * failing cell index.  form: HF_CHEM_PLAIN or HF_CHEM_PERSISTENT.  count 0 is a no-op
 * (U may then be NULL); a negative count, count > comp_stride without cell_index, dt <= 0
 * without dt_cell, or non-positive tolerances return HF_ERR_ARG before any device work. ---- */
HF_EXPORT hf_status hf_chem_advance(hf_ctx* ctx, double* U, int64_t comp_stride, const int64_t* cell_index,
                          int64_t count, double dt, const double* dt_cell, double rtol, double atol,
                          int form, int64_t* first_failed, void* stream);

/* Per-cell integrator history of the batched chemistry form (extension: the reference's
 * CVODE restarts every cell from scratch on each call).  Caller-owned device arrays of
 * count entries, zero-initialised before the first call.  h: the step size the controller
 * proposed after the cell's last interval (warm start of the next call); cost: the cell's
 * step attempts in the last call (orders the work queue most-expensive-first). */
typedef struct hf_chem_history {
    double* h;
    int32_t* cost;
} hf_chem_history;

/* Batched chemistry: the persistent work-queue kernel plus a frozen-cell screen (a cell whose
 * scaled derivative and Jacobian norms over dt are tiny takes one second-order Taylor step,
 * truncation error below 2e-5 tolerance units), warm-started step sizes and a cost-ordered
 * queue.  Same arguments, semantics and errors as hf_chem_advance (ChemistryBatch::advance,
 * chemistry_batch.cpp:21-50); history may be NULL. */
HF_EXPORT hf_status hf_chem_advance_batched(hf_ctx* ctx, double* U, int64_t comp_stride, const int64_t* cell_index,
                                            int64_t count, double dt, const double* dt_cell, double rtol,
                                            double atol, const hf_chem_history* history, int64_t* first_failed,
                                            void* stream);

/* Sensitivities of 0D chemistry runs (build-defined extension: the reference has no
 * sensitivity code).  A cell at rest at constant (rho, e) is advanced by ncalls chemistry
 * calls of dt each, every call as hf_chem_advance's plain form (Chemistry::advance,
 * chemistry.cpp:55-76).  The objective is read at the call boundaries t_n = n dt:
 *   HF_OBJ_IGNITION_DELAY: the time T first reaches T_0 + ignition_dT, interpolated
 *                          linearly between the boundaries around the crossing (NaN, and
 *                          zero gradients, when it never does);
 *   HF_OBJ_PEAK_PRESSURE:  max_n p_n;   HF_OBJ_FINAL_T: T at t = ncalls dt. */
enum { HF_OBJ_IGNITION_DELAY = 0, HF_OBJ_PEAK_PRESSURE = 1, HF_OBJ_FINAL_T = 2 };

typedef struct hf_adjoint_opts {
    int32_t objective;         /* HF_OBJ_* */
    int32_t checkpoint_every;  /* chemistry calls between stored checkpoints (>= 1) */
    double ignition_dT;        /* temperature rise that defines ignition (K) */
    double rtol, atol;         /* integrator tolerances (the reference's: 1e-8, 1e-15) */
} hf_adjoint_opts;

/* Objective of count cells (SoA, component stride comp_stride, device memory; not
 * modified) into objective[count] (device).  Chemistry failures: HF_ERR_CHEM_FAIL or
 * HF_ERR_MAXSTEPS with the lowest failing cell in *first_failed, objective NaN there. */
HF_EXPORT hf_status hf_chem_objective(hf_ctx* ctx, const double* U0, int64_t comp_stride, int64_t count, double dt,
                                      int32_t ncalls, const hf_adjoint_opts* opts, double* objective,
                                      int64_t* first_failed, void* stream);

/* Objective and its discrete adjoint: dJ_dlnA[r*count + i] = dJ_i / d ln(multiplier_r)
 * for the NR = 21 reactions of H2_Li.yaml in file order (duplicates separately; the
 * multiplier scales the forward and reverse rate constants, both falloff limits), and
 * (optional, may be NULL) dJ_dY0[k*count + i] = dJ_i / dY_k(0), k < NS-1, at fixed rho
 * and e with the last species closing the mass.  The derivative is that of the run with
 * its accepted step sequence frozen.  State is checkpointed every checkpoint_every calls
 * and recomputed in the reverse sweep; the scratch (about 0.4 MB per cell for 2000 calls,
 * 50 per checkpoint) is processed in chunks of cells.  Errors as hf_chem_objective. */
HF_EXPORT hf_status hf_chem_adjoint(hf_ctx* ctx, const double* U0, int64_t comp_stride, int64_t count, double dt,
                                    int32_t ncalls, const hf_adjoint_opts* opts, double* objective, double* dJ_dlnA,
                                    double* dJ_dY0, int64_t* first_failed, void* stream);

/* ---- Discrete adjoint of a run of Strang steps (build-defined extension) ----
 * hf_flow_record replays nsteps steps of BlockAMR::run (BlockAMR.cpp:409-419) on a one-patch
 * level from U0 (SoA [NV][ny][nx], device) with the plain forms (ghost fill + face/update
 * kernels, one thread per cell chemistry), each stage redone first order when its output is
 * inadmissible (:257-263).  dts (host, nsteps) gives the step sizes; NULL: the CFL dt of
 * each step with cfl.  It records the step sizes (dts_out, host, may be NULL), the stages'
 * first-order flags and the state every checkpoint_every steps, and writes the final state
 * to U_final (device SoA, may be NULL).  No wedge boundary.  Errors as the ABI calls it
 * makes (a stage inadmissible even first order: HF_ERR_INADMISSIBLE; no dt halving). */
typedef struct hf_flow_tape hf_flow_tape;
HF_EXPORT hf_status hf_flow_record(hf_ctx* ctx, const hf_level* level, const double* U0, int32_t nsteps,
                                   const double* dts, double cfl, int32_t checkpoint_every, int chemistry,
                                   double rtol, double atol, double* U_final, double* dts_out, hf_flow_tape** out,
                                   void* stream);
/* Reverse sweep of a recorded run from seed = dJ/dU_final (device SoA): U0_bar = dJ/dU0
 * (device SoA, may be NULL) and dJ_dlnA[21] (host, may be NULL) = dJ/d ln A_r (rate
 * multipliers as hf_chem_adjoint).  The derivative of the frozen map: the recorded step
 * sizes and every branch of the forward (minmod selections, first-order fallbacks, HLLC wave
 * cases, wall overrides, chemistry step sequences and clips) are held fixed; roundoff
 * repairs count as the identity.  Segments of checkpoint_every steps are recomputed from
 * their checkpoint. */
HF_EXPORT hf_status hf_flow_adjoint(hf_flow_tape* tape, const double* seed, double* U0_bar, double* dJ_dlnA,
                                    void* stream);
HF_EXPORT void hf_flow_tape_destroy(hf_flow_tape* tape);
/* Adjoint of one Euler stage (the discrete transpose used by hf_flow_adjoint): for the map
 * from a one-patch level's interior state U (ghosts filled from it by the boundary
 * conditions) to the stage output U - h div F of hf_flux_update (no Heun combination;
 * first_order as the forward stage took it), Ubar_in = J^T Ubar_out on the interior cells.
 * U must hold the filled ghosts of the forward stage; U, Ubar_out and Ubar_in share the
 * patch layout (one domain-covering patch, ng = 2).  No wedge boundary.  HF_ERR_FACE if a
 * face state is inadmissible. */
HF_EXPORT hf_status hf_flux_adjoint(hf_ctx* ctx, const hf_level* level, const hf_patch* patch, const double* U,
                                    const double* Ubar_out, double h, int first_order, double* Ubar_in,
                                    void* stream);

/* Chemistry without any device allocation.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: an embedding application whose device memory
 * budget is fixed up front and handed to its own pool (so a library allocation fails or
 * breaks the budget), or host code that must not take the device-wide synchronisation
 * that cudaMalloc and cudaFree can imply.  It needs no hf_ctx (hf_init allocates).  It
 * runs the plain form of hf_chem_advance (one thread per cell, same results, same
 * all-or-nothing semantics and error codes) with its scratch (trial states, failure
 * codes, status word) in one statically sized device array that every GPU loading this
 * library holds until the process exits: HF_NOALLOC_MAX_CELLS cells, about 1.8 MB.
 *   - nspecies: 9 (H2_Li) or 10 (H2_Li+AR); count > HF_NOALLOC_MAX_CELLS -> HF_ERR_ARG.
 *   - The call reads its status word back to the host and synchronises the stream before
 *     it commits the batch (all-or-nothing).
 *   - The first call on a device (the current device) looks up the array's device address
 *     and, if no hf_ctx has loaded the rate constants on that device, loads them.
 *   - The rate constants are the device's current ones: hf_set_rate_scale on any context
 *     in the process rescales them for this call too (they are one per device).
 *   - Every call uses the same array: calls that overlap on the GPU (other streams or
 *     threads) race.  Each call clears the status word it needs before launching.
 * Arguments as hf_chem_advance without ctx and form. */
#define HF_NOALLOC_MAX_CELLS 16384
HF_EXPORT hf_status hf_chem_advance_noalloc(int nspecies, double* U, int64_t comp_stride, const int64_t* cell_index,
                                            int64_t count, double dt, const double* dt_cell, double rtol,
                                            double atol, int64_t* first_failed, void* stream);

/* ---- block-AMR level operations ---- */
/* BlockAMR::totals (BlockAMR.cpp:347-355): out[n] = sum over the valid cells of the patches
 * (those whose leaf_mask byte is non-zero when leaf_mask is given; leaf_mask packs the
 * patches' cells in order, row-major) of U[n] (or |U[n]| if absolute) * cell_volume.
 * Deterministic double-double reduction (the reference sums in long double).  out: host
 * array of NV doubles. */
HF_EXPORT hf_status hf_totals(hf_ctx* ctx, const hf_patch* patches, int npatch, const double* U,
                              const uint8_t* leaf_mask, double cell_volume, int absolute, double* out,
                              void* stream);
/* average_down (BlockAMR.cpp:157-159, AMReX average_down at ratio 2): every coarse cell
 * under a fine patch becomes the mean of its four children.  Fine patches have even ilo,
 * jlo, nx, ny (level index of the fine level); their coarsened boxes lie in the coarse
 * patches. */
HF_EXPORT hf_status hf_average_down(hf_ctx* ctx, const hf_patch* fine, int nfine, const double* Uf,
                                    const hf_patch* coarse, int ncoarse, double* Uc, void* stream);
/* Reflux (BlockAMR.cpp:247-255: FluxRegister CrseInit(-h dA_c), FineAdd(+h dA_f),
 * ClearInternalBorders, Reflux(scale 1)): every uncovered coarse cell next to a fine patch
 * has the coarse flux of the shared face replaced by the sum of the fine fluxes.
 * coarse_level describes the coarse level (domain, dx, periodicity); fxc/fyc and fxf/fyf
 * are the face fluxes written by hf_flux_update for the coarse and fine patches (packed
 * per patch in patch order); h is the stage length. */
HF_EXPORT hf_status hf_reflux(hf_ctx* ctx, const hf_level* coarse_level, const hf_patch* coarse, int ncoarse,
                              double* Uc, const double* fxc, const double* fyc, const hf_patch* fine, int nfine,
                              const double* fxf, const double* fyf, double h, void* stream);
/* Tagging criteria of BlockAMR::ErrorEst (BlockAMR.cpp:170-200) and its case keys, plus a
 * relative density-jump criterion (extension; off when density_tag <= 0). */
typedef struct hf_tag_criteria {
    double pressure_tag;     /* "pressure_tag" (0.08) */
    double temperature_tag;  /* "temperature_tag" (0.08) */
    double fuel_rate_tag;    /* "fuel_rate_tag" (50), used when chemistry != 0 */
    double density_tag;      /* extension: max relative density jump to a neighbour */
    int32_t chemistry;       /* "chemistry" */
    int32_t box_only;        /* "tag_mode" == "box" */
    int32_t has_box;         /* "tag_box" given */
    int32_t pad_;
    double box[4];           /* "tag_box": x0, x1, y0, y1 */
    double velocity[2];      /* "tag_velocity" */
} hf_tag_criteria;
/* ErrorEst on the valid cells of the patches (ghost layers filled): tags packs the
 * patches' cells in order (1 = tagged).  HF_ERR_INADMISSIBLE if a cell of a stencil is
 * inadmissible (properties() throws there in the reference). */
HF_EXPORT hf_status hf_tag_cells(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch,
                                 const double* U, double time, const hf_tag_criteria* criteria, uint8_t* tags,
                                 void* stream);

/* ---- Multi-level block AMR (BlockAMR::run with max_level > 0, BlockAMR.cpp:400-439) ----
 * Levels 0..max_level at ratio 2 with no time subcycling; each level a dense ghosted array
 * over its domain whose active blocks (block x block cells) are the patches.  Per stage:
 * ghosts (physical, in-place neighbours, ConservativeInterp from the coarser level at
 * coarse-fine boundaries), the Euler update of every level, reflux and average_down
 * finest to coarsest, a first-order redo of the composite stage when needed; Heun
 * combination; react() on the leaf cells; rollback and dt halving.  Regrid every
 * regrid_interval steps (and max_level times at creation): ErrorEst tags (tags) on level l
 * make a level-(l+1) block active when a tagged cell lies in its footprint grown by
 * tag_buffer cells and its footprint grown by 2 cells lies in active level-l blocks (both
 * wrap across periodic edges); new blocks are filled by ConservativeInterp; the conserved totals are checked to 1e-8 of the
 * totals of magnitudes (regridChecked).  base: level 0 (nx, ny multiples of block/2). */
typedef struct hf_amr_opts {
    int32_t max_level;        /* "max_level" */
    int32_t block;            /* block size ("max_grid_size"), even, >= 8 */
    int32_t tag_buffer;       /* "tag_buffer" (cells of the tagged level) */
    int32_t regrid_interval;  /* "regrid_interval" (steps; <= 0: no regrid after creation) */
    int32_t chemistry;        /* "chemistry" */
    int32_t chem_form;        /* HF_CHEM_PLAIN or HF_CHEM_PERSISTENT (batched) */
    double rtol, atol;
    hf_tag_criteria tags;
} hf_amr_opts;
typedef struct hf_amr hf_amr;
/* U0: level-0 state, SoA [NV][ny][nx] device memory (copied). */
HF_EXPORT hf_status hf_amr_create(hf_ctx* ctx, const hf_level* base, const double* U0, const hf_amr_opts* opts,
                                  hf_amr** out, void* stream);
/* As hf_amr_create, with the initial state of levels 0..nlevels-1 (host array of device
 * pointers to SoA [NV][ny_l][nx_l] dense level states; entries after the first may be
 * NULL): while the initial hierarchy is built, a block of level l that becomes active
 * takes U_levels[l] instead of the interpolation of level l-1 (the reference's
 * MakeNewLevelFromScratch, BlockAMR.cpp:124-131, evaluates the initial condition on
 * every level), the remap check is skipped, and the levels are then averaged down and
 * validated (run(), :401).  nlevels <= max_level + 1. */
HF_EXPORT hf_status hf_amr_create_levels(hf_ctx* ctx, const hf_level* base, const double* const* U_levels,
                                         int nlevels, const hf_amr_opts* opts, hf_amr** out, void* stream);
HF_EXPORT void hf_amr_destroy(hf_amr* amr);
/* One Strang step of every level; *dt as hf_stepper_step (<= 0: stableDt over all levels). */
HF_EXPORT hf_status hf_amr_step(hf_amr* amr, double cfl, double* dt, void* stream);
/* BlockAMR::stableDt (BlockAMR.cpp:335-346) over the active cells of every level: the
 * step hf_amr_step takes when given *dt <= 0 on its host-driven path. */
HF_EXPORT hf_status hf_amr_cfl_dt(hf_amr* amr, double cfl, double* dt, void* stream);
HF_EXPORT hf_status hf_amr_regrid(hf_amr* amr, void* stream);
/* Level sizes, block grid, finest level and the level's leaf cells. */
HF_EXPORT hf_status hf_amr_info(const hf_amr* amr, int lev, int32_t* nx, int32_t* ny, int32_t* nbx, int32_t* nby,
                                int32_t* finest, int64_t* leaf_cells);
/* Level lev's dense state (SoA [NV][ny_l][nx_l], device; cells of inactive blocks are
 * stale) and its block activity map ([nby][nbx], host, may be NULL). */
HF_EXPORT hf_status hf_amr_get_level(hf_amr* amr, int lev, double* U, uint8_t* active, void* stream);
/* Composite totals over the leaf cells of all levels (host, NV doubles). */
HF_EXPORT hf_status hf_amr_totals(hf_amr* amr, double* out, void* stream);
HF_EXPORT double hf_amr_time(const hf_amr* amr);
/* Graph-captured steps (default on; CFL steps with the batched chemistry form): the whole
 * multi-level Strang step is one CUDA graph (device dt, one status read per step),
 * recaptured after every regrid; a step whose graph raises a flag is re-run by the
 * host-driven path from the untouched start state.  Extension: the reference has no
 * device graph. */
HF_EXPORT void hf_amr_set_graph(hf_amr* amr, int enable);
HF_EXPORT void hf_amr_stats(const hf_amr* amr, int64_t* graph_steps, int64_t* host_steps);


/* ---- reductions ---- */
/* BlockAMR::stableDt (BlockAMR.cpp:335-346) over the valid cells of the patches:
 * *dt = cfl / max((|u|+a)/dx + (|v|+a)/dy).  HF_ERR_INADMISSIBLE if a cell is not. */
HF_EXPORT hf_status hf_cfl_dt(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch,
                    const double* U, double cfl, double* dt, void* stream);
/* BlockAMR::validate (BlockAMR.cpp:286-298): HF_ERR_INADMISSIBLE and the lowest failing
 * linear cell index if any valid cell is inadmissible. */
HF_EXPORT hf_status hf_validate(hf_ctx* ctx, const hf_level* level, const hf_patch* patches, int npatch,
                      const double* U, int64_t* bad_cell, void* stream);
/* BlockAMR::repairRoundoff (BlockAMR.cpp:299-334) over the leaf cells of nlev levels, in
 * place: per species the peak partial density and the donor (the first cell, levels in
 * order, patches in order, cells row by row, holding the largest mass = value x cell
 * volume) over all leaf cells; a value below zero by at most 64 ulp of the peak is set
 * to zero and its deficit (-value x volume) taken from the donor, the deficits added in
 * that cell order.  HF_ERR_NEGATIVE if a value is further below zero or not finite, or a
 * donor holds no more mass than its deficit (the reference throws); the state may then
 * be partly repaired.  Level l: levels[l] (its dx, dy give the cell volume),
 * patches[l][0..npatch[l]-1], state U[l], and leaf[l] (nullable: every cell is a leaf), a
 * device byte mask over the patches' cells packed in order, row-major.  *repairs (may be
 * NULL): the number of values set to zero.  The stepper calls the same kernels after
 * every stage (one level: hf_flux_update; every level after reflux: hf_amr_step). */
HF_EXPORT hf_status hf_repair_roundoff(hf_ctx* ctx, int nlev, const hf_level* levels, const hf_patch* const* patches,
                                       const int* npatch, double* const* U, const uint8_t* const* leaf,
                                       int64_t* repairs, void* stream);

/* ---- host stepper over a single-patch uniform level (BlockAMR::run loop body,
 * BlockAMR.cpp:409-419): Strang flow(dt/2), react(dt), flow(dt/2), each flow a Heun pair
 * of Euler stages; rollback and dt halving up to 18 attempts. ---- */
typedef struct hf_stepper hf_stepper;
/* U0: initial valid cells, SoA [NV][ny][nx] in DEVICE memory (copied in); NULL starts
 * from zeros, for a host that loads the state with hf_stepper_set_host. */
HF_EXPORT hf_status hf_stepper_create(hf_ctx* ctx, const hf_level* level, const double* U0, int chemistry,
                            double rtol, double atol, int flux_form, int chem_form,
                            hf_stepper** out);
HF_EXPORT void hf_stepper_destroy(hf_stepper* st);
/* One Strang step.  *dt in: requested interval (<= 0: CFL dt with the given cfl);
 * out: the accepted interval. */
HF_EXPORT hf_status hf_stepper_step(hf_stepper* st, double cfl, double* dt, void* stream);
/* nsteps CFL Strang steps with no host round trip between them (the loop of BlockAMR::run,
 * BlockAMR.cpp:409-419, for nsteps iterations): the captured step graphs are launched back
 * to back, up to 256 per batch, and the host reads one device record per batch.  A step
 * whose graph raises a flag stops the batch on the device (the steps after it do nothing)
 * and is re-run with host control (first-order redo, rollback, dt halving) exactly as
 * hf_stepper_step would.  Same results as nsteps calls of hf_stepper_step with *dt = 0.
 * *steps_done (may be NULL) receives the steps completed, also on error.  Either
 * chemistry form (batched, or plain: one thread per cell) runs inside the graphs. */
HF_EXPORT hf_status hf_stepper_run(hf_stepper* st, int32_t nsteps, double cfl, int32_t* steps_done, void* stream);
/* Copy the valid cells out, SoA [NV][ny][nx], to DEVICE memory. */
HF_EXPORT hf_status hf_stepper_get(hf_stepper* st, double* U, void* stream);
/* Copy valid cells in from / out to HOST memory (pinned or pageable), SoA [NV][ny][nx]. */
HF_EXPORT hf_status hf_stepper_set_host(hf_stepper* st, const double* U, void* stream);
HF_EXPORT hf_status hf_stepper_get_host(hf_stepper* st, double* U, void* stream);
HF_EXPORT double hf_stepper_time(const hf_stepper* st);
/* stableDt of the current state (BlockAMR.cpp:335-346). */
HF_EXPORT hf_status hf_stepper_cfl_dt(hf_stepper* st, double cfl, double* dt, void* stream);
/* Steps taken through the captured CUDA graph (either flux form + either chemistry form +
 * CFL dt: one graph launch and one status read per step) and through the host-controlled path
 * (every other case, and any graph step whose status reported a failure, re-run from the
 * untouched start state).  Extension: the reference has no device graph. */
HF_EXPORT void hf_stepper_stats(const hf_stepper* st, int64_t* graph_steps, int64_t* host_steps);
/* Why graph steps fall back to the host-controlled path: the status flags of the last
 * graph step (0 when it was accepted; a failed cell or stage sets them), the CUDA error of
 * a capture that failed (0 when none did; the graph path is then off), and (phase_flags,
 * 4 entries, nullable) the last single graph step's flags at its start, after the CFL
 * reduction and the first flow, after the chemistry and its validation, and after the
 * second flow. */
HF_EXPORT void hf_stepper_graph_info(const hf_stepper* st, uint32_t* last_flags, int32_t* capture_error,
                                     uint32_t* phase_flags);
/* Enable (default) or disable the graph path. */
HF_EXPORT void hf_stepper_set_graph(hf_stepper* st, int enable);

#ifdef __cplusplus
}
#endif
#endif
