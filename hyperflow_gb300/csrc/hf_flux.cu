// Flux path kernels: ghost fill, Euler-stage flux + update (plain and fused
// forms), Heun combine, validation, CFL reduction, and the coarse->fine
// conservative interpolation (the roundoff repair is in hf_amr.cu).  Reference
// semantics:
//   ghost fill      HyperFlow_V3/src/BlockAMR.cpp:48-59,137-146; src/FlowBoundary.hpp:12-36
//                   (AMReX FillPatchSingleLevel: FillBoundary, then filcc per cell and the
//                   FlowBoundary functor, faces before corners)
//   Euler stage     BlockAMR.cpp:210-243 (MUSCL on conserved variables, admissibility
//                   fallback per face side, HLLC, wall-flux override, flux divergence)
//   Heun combine    BlockAMR.cpp:266-269
//   validate        BlockAMR.cpp:286-298
//   stableDt        BlockAMR.cpp:335-346
//   interpolation   src/ConservativeInterp.cpp:18-51
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstring>
#include "hf_device.cuh"
#include "hf_internal.h"

namespace hf {

// ---------------------------------------------------------------- helpers
struct PView {
    const double* U;
    hf_patch P;
    __device__ __forceinline__ int64_t idx(int li, int lj, int n) const {
        return P.offset + (int64_t)n * P.comp_stride + (int64_t)(lj + P.ng) * P.pitch + (li + P.ng);
    }
    __device__ __forceinline__ double get(int li, int lj, int n) const { return U[idx(li, lj, n)]; }
};

// AMReX BCType equivalents of the reference's boundary kinds (BlockAMR.cpp:52-58)
enum : int { BCT_INT = 0, BCT_FOEXTRAP = 1, BCT_EVEN = 2, BCT_ODD = 3, BCT_EXT = 4 };

__device__ __forceinline__ int bct(const Level& L, int d, int hi, int n, int NS) {
    if (L.periodic[d]) return BCT_INT;
    const int kind = hi ? L.hi[d] : L.lo[d];
    if (kind == HF_BC_INFLOW || kind == HF_BC_WEDGE) return BCT_EXT;
    if (kind == HF_BC_REFLECTING) return n == NS + d ? BCT_ODD : BCT_EVEN;
    return BCT_FOEXTRAP;
}

__device__ __forceinline__ void flag(DevStatus* st, unsigned f, unsigned long long cell) {
    atomicOr(&st->flags, f);
    atomicMin(&st->bad_cell, cell);
}

// ---------------------------------------------------------------- ghost fill
// Cell accessor in level coordinates for patch P (which must hold the cell in its
// ghosted box).
struct GView {
    double* U;
    hf_patch P;
    __device__ __forceinline__ double& at(int gi, int gj, int n) const {
        return U[P.offset + (int64_t)n * P.comp_stride + (int64_t)(gj - P.jlo + P.ng) * P.pitch + (gi - P.ilo + P.ng)];
    }
};

template <int NS>
__device__ void filcc_cell(const Level& L, const GView& v, int gi, int gj) {
    const int ihi = L.nx - 1, jhi = L.ny - 1;
#pragma unroll 1
    for (int n = 0; n < NS + 3; ++n) {
        if (gi < 0 || gi > ihi) {
            const int t = bct(L, 0, gi > ihi, n, NS);
            const int src = gi < 0 ? -gi - 1 : 2 * ihi - gi + 1;
            if (t == BCT_FOEXTRAP) v.at(gi, gj, n) = v.at(gi < 0 ? 0 : ihi, gj, n);
            else if (t == BCT_EVEN) v.at(gi, gj, n) = v.at(src, gj, n);
            else if (t == BCT_ODD) v.at(gi, gj, n) = -v.at(src, gj, n);
        }
        if (gj < 0 || gj > jhi) {
            const int t = bct(L, 1, gj > jhi, n, NS);
            const int src = gj < 0 ? -gj - 1 : 2 * jhi - gj + 1;
            if (t == BCT_FOEXTRAP) v.at(gi, gj, n) = v.at(gi, gj < 0 ? 0 : jhi, n);
            else if (t == BCT_EVEN) v.at(gi, gj, n) = v.at(gi, src, n);
            else if (t == BCT_ODD) v.at(gi, gj, n) = -v.at(gi, src, n);
        }
    }
}

template <int NS>
__device__ void flow_boundary_cell(const Level& L, const GView& v, int gi, int gj) {
    const bool mixedBottom = !L.periodic[1] && L.lo[1] == HF_BC_WEDGE;
    const bool below = gj < 0;
    const int iv[2] = {gi, gj}, hiE[2] = {L.nx - 1, L.ny - 1};
#pragma unroll 1
    for (int n = 0; n < NS + 3; ++n) {
        bool fixed = false;
        for (int d = 0; d < 2; ++d) {
            const bool mixed = mixedBottom && d == 1 && below;
            fixed = fixed || (iv[d] < 0 && bct(L, d, 0, n, NS) == BCT_EXT && !mixed);
            fixed = fixed || (iv[d] > hiE[d] && bct(L, d, 1, n, NS) == BCT_EXT);
        }
        if (fixed) { v.at(gi, gj, n) = L.inlet[n]; continue; }
        if (mixedBottom && below) {
            const double x = L.xlo + (gi + 0.5) * L.dx;
            const bool wall = x >= L.wedge_start;
            const int jj = wall ? -gj - 1 : 0;
            const int ii = min(max(gi, 0), L.nx - 1);
            double val = v.at(ii, jj, n);
            if (wall && n == NS + 1) val = -val;
            v.at(gi, gj, n) = val;
        }
    }
}

__device__ __forceinline__ bool ghost_coord(const hf_patch& P, int64_t k, int& li, int& lj) {
    const int ng = P.ng, W = P.nx + 2 * ng;
    const int64_t strip = (int64_t)ng * W;
    if (k < strip) { lj = -ng + (int)(k / W); li = -ng + (int)(k % W); return true; }
    k -= strip;
    if (k < strip) { lj = P.ny + (int)(k / W); li = -ng + (int)(k % W); return true; }
    k -= strip;
    const int64_t side = (int64_t)ng * P.ny;
    if (k < side) { lj = (int)(k / ng); li = -ng + (int)(k % ng); return true; }
    k -= side;
    if (k < side) { lj = (int)(k / ng); li = P.nx + (int)(k % ng); return true; }
    return false;
}

// phase 0: same-level exchange (periodic images included); 1: faces; 2: corners.
template <int NS>
__global__ void k_fill(Level L, const hf_patch* __restrict__ patches, int npatch, double* U, int phase) {
    const hf_patch P = patches[blockIdx.y];
    int li, lj;
    if (!ghost_coord(P, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, li, lj)) return;
    const int gi = P.ilo + li, gj = P.jlo + lj;
    const bool gx = L.periodic[0] || (gi >= 0 && gi < L.nx);
    const bool gy = L.periodic[1] || (gj >= 0 && gj < L.ny);
    const int out = (!gx) + (!gy);
    GView v{U, P};
    if (phase == 0) {
        if (out) return;
        const int wi = ((gi % L.nx) + L.nx) % L.nx, wj = ((gj % L.ny) + L.ny) % L.ny;
        for (int q = 0; q < npatch; ++q) {
            const hf_patch& Q = patches[q];
            if (wi >= Q.ilo && wi < Q.ilo + Q.nx && wj >= Q.jlo && wj < Q.jlo + Q.ny) {
                GView s{U, Q};
                for (int n = 0; n < NS + 3; ++n) v.at(gi, gj, n) = s.at(wi, wj, n);
                return;
            }
        }
        return;
    }
    if (out != phase) return;
    filcc_cell<NS>(L, v, gi, gj);
    flow_boundary_cell<NS>(L, v, gi, gj);
}

template <int NS>
static cudaError_t fill_impl(const Level& L, const hf_patch* ph, const hf_patch* pd, int npatch, double* U,
                             cudaStream_t s, int64_t* launches) {
    int64_t gmax = 0;
    for (int p = 0; p < npatch; ++p) {
        const int64_t W = ph[p].nx + 2 * ph[p].ng;
        gmax = max(gmax, (int64_t)2 * ph[p].ng * W + (int64_t)2 * ph[p].ng * ph[p].ny);
    }
    const int bs = 128;
    dim3 grid((unsigned)((gmax + bs - 1) / bs), (unsigned)npatch);
    for (int phase = 0; phase < 3; ++phase) {
        k_fill<NS><<<grid, bs, 0, s>>>(L, pd, npatch, U, phase);
        ++*launches;
    }
    return cudaGetLastError();
}
cudaError_t launch_fill(int ns, const Level& L, const hf_patch* ph, const hf_patch* pd, int npatch, double* U,
                        cudaStream_t s, int64_t* launches) {
    return ns == 9 ? fill_impl<9>(L, ph, pd, npatch, U, s, launches) : fill_impl<10>(L, ph, pd, npatch, U, s, launches);
}

// ---------------------------------------------------------------- face flux (shared)
// One face: 4-cell stencil values are fetched by get(k, n), k = 0..3 for qa..qd.
template <int NS, int D, class Get>
__device__ __forceinline__ bool face_flux(const Level& L, int gi, int gj, int first_order, Get get, double* f) {
    constexpr int NV = NS + 3;
    double lq[NV], rq[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        const double qa = get(0, n), qb = get(1, n), qc = get(2, n), qd = get(3, n);
        if (first_order) {
            lq[n] = qb;
            rq[n] = qc;
        } else {
            lq[n] = qb + 0.5 * minmod(qb - qa, qc - qb);
            rq[n] = qc - 0.5 * minmod(qc - qb, qd - qc);
        }
    }
    Props pl, pr;
    if (!properties<NS>(lq, pl, 1000.0)) {
#pragma unroll
        for (int n = 0; n < NV; ++n) lq[n] = get(1, n);
        if (!properties<NS>(lq, pl, 1000.0)) return false;
    }
    if (!properties<NS>(rq, pr, 1000.0)) {
#pragma unroll
        for (int n = 0; n < NV; ++n) rq[n] = get(2, n);
        if (!properties<NS>(rq, pr, 1000.0)) return false;
    }
    hllc<NS, NS + D>(lq, rq, pl, pr, f);
    // wall-flux override, BlockAMR.cpp:224-229
    const bool loWall = !L.periodic[D] && (L.lo[D] == HF_BC_REFLECTING || L.lo[D] == HF_BC_WEDGE);
    const bool hiWall = !L.periodic[D] && L.hi[D] == HF_BC_REFLECTING;
    const bool mixedBottom = !L.periodic[1] && L.lo[1] == HF_BC_WEDGE;
    const int coord = D == 0 ? gi : gj;
    const double x = L.xlo + (gi + 0.5) * L.dx;
    const bool lowWall = loWall && !(D == 1 && mixedBottom && x < L.wedge_start);
    if ((coord == 0 && lowWall) || (coord == (D == 0 ? L.nx : L.ny) && hiWall)) {
#pragma unroll
        for (int k = 0; k < NS; ++k) f[k] = 0.0;
        f[D == 0 ? NS + 1 : NS] = 0.0;
        f[NS + 2] = 0.0;
    }
    return true;
}

// ---------------------------------------------------------------- plain form
// Face idx of direction D of patch P into F (component stride = the patch's face count).
template <int NS, int D>
__device__ __forceinline__ void face_one(const Level& L, const hf_patch& P, const double* __restrict__ U,
                                         double* __restrict__ F, int first_order, int64_t cell_base, DevStatus* st,
                                         int64_t idx) {
    const int fnx = P.nx + (D == 0), fny = P.ny + (D == 1);
    if (idx >= (int64_t)fnx * fny) return;
    const int fi = (int)(idx % fnx), fj = (int)(idx / fnx);
    PView v{U, P};
    auto get = [&](int k, int n) {
        return D == 0 ? v.get(fi - 2 + k, fj, n) : v.get(fi, fj - 2 + k, n);
    };
    double f[NS + 3];
    if (!face_flux<NS, D>(L, P.ilo + fi, P.jlo + fj, first_order, get, f)) {
        flag(st, ST_FACE_BAD, cell_base + (int64_t)min(fj, P.ny - 1) * P.nx + min(fi, P.nx - 1));
#pragma unroll
        for (int n = 0; n < NS + 3; ++n) f[n] = 0.0;
    }
    const int64_t nf = (int64_t)fnx * fny;
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) F[n * nf + idx] = f[n];
}

template <int NS, int D>
__global__ void __launch_bounds__(128) k_face_plain(Level L, hf_patch P, const double* __restrict__ U,
                                                    double* __restrict__ F, int first_order, int64_t cell_base,
                                                    DevStatus* st) {
    if (st->abort_run) return;  // an earlier step of this device-resident run failed
    face_one<NS, D>(L, P, U, F, first_order, cell_base, st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// All patches of a level in one launch: patch blockIdx.y, its x/y face arrays at
// off[3p], off[3p+1] of FX/FY and its first cell's index at off[3p+2].
template <int NS, int D>
__global__ void __launch_bounds__(128) k_face_multi(Level L, const hf_patch* __restrict__ patches,
                                                    const int64_t* __restrict__ off, const double* __restrict__ U,
                                                    double* __restrict__ F, int first_order, DevStatus* st) {
    if (st->abort_run) return;
    const int p = blockIdx.y;
    const hf_patch P = patches[p];
    face_one<NS, D>(L, P, U, F + off[3 * p + D], first_order, off[3 * p + 2], st,
                    (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Validation of an updated cell, then optional Heun combine.  Negative partial
// densities are reported (ST_NEGATIVE) instead of validated: the host then runs
// the roundoff repair (which may zero them) before validating.
template <int NS>
__device__ __forceinline__ void finish_cell(double* q, const double* __restrict__ Uold, int64_t gidx,
                                            int64_t cstride, double* __restrict__ Uout, int64_t cell,
                                            DevStatus* st) {
    constexpr int NV = NS + 3;
    bool neg = false;
#pragma unroll
    for (int k = 0; k < NS; ++k) neg = neg || (q[k] < 0.0);
    Props p;
    if (neg) {
        flag(st, ST_NEGATIVE, cell);
    } else if (!properties<NS>(q, p, 1000.0)) {
        flag(st, ST_STAGE_BAD, cell);
    }
    if (Uold) {
#pragma unroll
        for (int n = 0; n < NV; ++n) q[n] = 0.5 * Uold[gidx + n * cstride] + 0.5 * q[n];
        if (!neg && !properties<NS>(q, p, 1000.0)) flag(st, ST_COMBINE_BAD, cell);
    }
#pragma unroll
    for (int n = 0; n < NV; ++n) Uout[gidx + n * cstride] = q[n];
}

// Update, validation and optional Heun combine of cell idx of patch P.
template <int NS>
__device__ __forceinline__ void update_one(const hf_patch& P, const double* __restrict__ Uin,
                                           const double* __restrict__ Uold, double* __restrict__ Uout,
                                           const double* __restrict__ Fx, const double* __restrict__ Fy, double cx,
                                           double cy, int64_t cell_base, DevStatus* st, int64_t idx) {
    constexpr int NV = NS + 3;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t nfx = (int64_t)(P.nx + 1) * P.ny, nfy = (int64_t)P.nx * (P.ny + 1);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
    double q[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        const double fl = Fx[n * nfx + (int64_t)j * (P.nx + 1) + i], fr = Fx[n * nfx + (int64_t)j * (P.nx + 1) + i + 1];
        const double fb = Fy[n * nfy + (int64_t)j * P.nx + i], ft = Fy[n * nfy + (int64_t)(j + 1) * P.nx + i];
        q[n] = Uin[g + n * P.comp_stride] - cx * (fr - fl) - cy * (ft - fb);
    }
    finish_cell<NS>(q, Uold, g, P.comp_stride, Uout, cell_base + idx, st);
}

template <int NS>
__global__ void __launch_bounds__(128) k_update_plain(hf_patch P, const double* __restrict__ Uin,
                                                      const double* __restrict__ Uold, double* __restrict__ Uout,
                                                      const double* __restrict__ Fx, const double* __restrict__ Fy,
                                                      double cx, double cy, const double* __restrict__ hdev,
                                                      double dx, double dy, int64_t cell_base, DevStatus* st) {
    if (st->abort_run) return;
    if (hdev) {  // stage step from device memory (graph-captured steps): h/dx as on the host
        const double h = *hdev;
        cx = h / dx;
        cy = h / dy;
    }
    update_one<NS>(P, Uin, Uold, Uout, Fx, Fy, cx, cy, cell_base, st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int NS>
__global__ void __launch_bounds__(128) k_update_multi(const hf_patch* __restrict__ patches,
                                                      const int64_t* __restrict__ off, const double* __restrict__ Uin,
                                                      const double* __restrict__ Uold, double* __restrict__ Uout,
                                                      const double* __restrict__ FX, const double* __restrict__ FY,
                                                      double cx, double cy, const double* __restrict__ hdev,
                                                      double dx, double dy, DevStatus* st) {
    if (st->abort_run) return;
    if (hdev) {  // stage step from device memory (graph-captured steps): h/dx as on the host
        const double h = *hdev;
        cx = h / dx;
        cy = h / dy;
    }
    const int p = blockIdx.y;
    const hf_patch P = patches[p];
    update_one<NS>(P, Uin, Uold, Uout, FX + off[3 * p], FY + off[3 * p + 1], cx, cy, off[3 * p + 2], st,
                   (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int NS>
static cudaError_t flux_plain_impl(const Level& L, const hf_patch& P, const double* Uin, const double* Uold,
                                   double* Uout, double* fx, double* fy, double h, int first_order,
                                   int64_t cell_base, DevStatus* st, cudaStream_t s, int64_t* launches,
                                   const double* hdev) {
    const int bs = 128;
    const int64_t nfx = (int64_t)(P.nx + 1) * P.ny, nfy = (int64_t)P.nx * (P.ny + 1);
    k_face_plain<NS, 0><<<(unsigned)((nfx + bs - 1) / bs), bs, 0, s>>>(L, P, Uin, fx, first_order, cell_base, st);
    k_face_plain<NS, 1><<<(unsigned)((nfy + bs - 1) / bs), bs, 0, s>>>(L, P, Uin, fy, first_order, cell_base, st);
    const int64_t nc = (int64_t)P.nx * P.ny;
    k_update_plain<NS><<<(unsigned)((nc + bs - 1) / bs), bs, 0, s>>>(P, Uin, Uold, Uout, fx, fy, h / L.dx, h / L.dy,
                                                                     hdev, L.dx, L.dy, cell_base, st);
    *launches += 3;
    return cudaGetLastError();
}
template <int NS>
static cudaError_t flux_multi_impl(const Level& L, const hf_patch* ph, const hf_patch* pd, int npatch,
                                   const int64_t* offd, const double* Uin, const double* Uold, double* Uout,
                                   double* FX, double* FY, double h, int first_order, DevStatus* st, cudaStream_t s,
                                   int64_t* launches, const double* hdev) {
    const int bs = 128;
    int64_t mfx = 1, mfy = 1, mc = 1;
    for (int p = 0; p < npatch; ++p) {
        mfx = max(mfx, (int64_t)(ph[p].nx + 1) * ph[p].ny);
        mfy = max(mfy, (int64_t)ph[p].nx * (ph[p].ny + 1));
        mc = max(mc, (int64_t)ph[p].nx * ph[p].ny);
    }
    k_face_multi<NS, 0><<<dim3((unsigned)((mfx + bs - 1) / bs), (unsigned)npatch), bs, 0, s>>>(L, pd, offd, Uin, FX,
                                                                                             first_order, st);
    k_face_multi<NS, 1><<<dim3((unsigned)((mfy + bs - 1) / bs), (unsigned)npatch), bs, 0, s>>>(L, pd, offd, Uin, FY,
                                                                                             first_order, st);
    k_update_multi<NS><<<dim3((unsigned)((mc + bs - 1) / bs), (unsigned)npatch), bs, 0, s>>>(
        pd, offd, Uin, Uold, Uout, FX, FY, h / L.dx, h / L.dy, hdev, L.dx, L.dy, st);
    *launches += 3;
    return cudaGetLastError();
}
cudaError_t launch_flux_multi(int ns, const Level& L, const hf_patch* patches_host, const hf_patch* patches_dev,
                              int npatch, const int64_t* off_dev, const double* Uin, const double* Uold, double* Uout,
                              double* FX, double* FY, double h, int first_order, DevStatus* st, cudaStream_t s,
                              int64_t* launches, const double* hdev) {
    return ns == 9 ? flux_multi_impl<9>(L, patches_host, patches_dev, npatch, off_dev, Uin, Uold, Uout, FX, FY, h,
                                        first_order, st, s, launches, hdev)
                   : flux_multi_impl<10>(L, patches_host, patches_dev, npatch, off_dev, Uin, Uold, Uout, FX, FY, h,
                                         first_order, st, s, launches, hdev);
}
cudaError_t launch_flux_plain(int ns, const Level& L, const hf_patch& P, int, const double* Uin, const double* Uold,
                              double* Uout, double* fx, double* fy, double h, int first_order, int64_t cell_base,
                              DevStatus* st, cudaStream_t s, int64_t* launches, const double* hdev) {
    return ns == 9 ? flux_plain_impl<9>(L, P, Uin, Uold, Uout, fx, fy, h, first_order, cell_base, st, s, launches, hdev)
                   : flux_plain_impl<10>(L, P, Uin, Uold, Uout, fx, fy, h, first_order, cell_base, st, s, launches,
                                         hdev);
}

// ---------------------------------------------------------------- fused form
// One CTA per TX x TY tile.  The tile plus its 2-cell halo, all NV components, is
// copied from the ghosted SoA array into shared memory with one TMA tensor load
// (box HX x HY x NV doubles).  Halo cells outside the domain are then overwritten
// with their boundary values computed from the tile (periodic images from global
// memory), in AMReX order.  Faces are evaluated into shared memory, then each
// thread updates, validates and (optionally) Heun-combines one cell.
// A 32 x 7 tile has (TX+1) TY + TX (TY+1) = 487 faces, which 8 warps take in two
// passes (a 32 x 8 tile has 552: a third, nearly empty pass that the other warps wait
// for at the barrier); the first TX x TY threads then update one cell each.  Nine
// warps would cap registers at 168 (three warps on one scheduler) and spill.
constexpr int TX = 32, TY = 7, HX = TX + 4, HY = TY + 4, NTHR = 256;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

template <int NS>
struct FusedSmem {
    static constexpr int NV = NS + 3;
    static constexpr int TILE = NV * HY * HX;
    static constexpr int FXN = NV * TY * (TX + 1);
    static constexpr int FYN = NV * (TY + 1) * TX;
    static constexpr size_t bytes = (size_t)(TILE + FXN + FYN) * sizeof(double) + 128;
};

template <int NS>
__global__ void __launch_bounds__(NTHR) k_flux_fused(const __grid_constant__ CUtensorMap tmap, Level L, hf_patch P,
                                                     const double* __restrict__ Uin, const double* __restrict__ Uold,
                                                     double* __restrict__ Uout, double cx, double cy,
                                                     const double* __restrict__ hdev, int first_order,
                                                     int64_t cell_base, DevStatus* st) {
    constexpr int NV = NS + 3;
    if (st->abort_run) return;  // an earlier step of this device-resident run failed
    if (hdev) {  // stage length from device memory (graph-captured steps)
        const double h = *hdev;
        cx = h / L.dx;
        cy = h / L.dy;
    }
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ int s_fail;
    double* tile = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    double* sfx = tile + FusedSmem<NS>::TILE;
    double* sfy = sfx + FusedSmem<NS>::FXN;
    const int tid = threadIdx.x;
    const int ti0 = blockIdx.x * TX, tj0 = blockIdx.y * TY;
    auto T = [&](int hi, int hj, int n) -> double& { return tile[(n * HY + hj) * HX + hi]; };

    // 1. TMA load of the box starting at ghosted-array coordinates (ti0-2+ng, tj0-2+ng, 0)
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        constexpr unsigned bytes = (unsigned)(FusedSmem<NS>::TILE * sizeof(double));
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(bytes)
                     : "memory");
        const int x = ti0 - 2 + P.ng, y = tj0 - 2 + P.ng, z = 0;
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                smem_u32(tile)),
            "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(&mbar))
            : "memory");
    }
    {
        // bounded, non-blocking wait on phase 0 of the barrier (at most ~2^20 polls
        // spaced by __nanosleep, well under a second), then an error flag
        unsigned done = 0;
        for (int it = 0; it < (1 << 20) && !done; ++it) {
            asm volatile(
                "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                : "=r"(done)
                : "r"(smem_u32(&mbar))
                : "memory");
            if (!done) __nanosleep(64);
        }
        if (!done) atomicOr(&s_fail, 1);
    }
    __syncthreads();
    if (s_fail) {
        if (tid == 0) flag(st, ST_TIMEOUT, cell_base + (int64_t)tj0 * P.nx + ti0);
        return;
    }

    // 2. boundary values for halo cells outside the domain (edge tiles only)
    const int gi0 = P.ilo + ti0 - 2, gj0 = P.jlo + tj0 - 2;
    const bool edge = gi0 < 0 || gj0 < 0 || gi0 + HX > L.nx || gj0 + HY > L.ny;
    if (edge) {
        auto in_g = [&](int g, int d) { return L.periodic[d] || (g >= 0 && g < (d == 0 ? L.nx : L.ny)); };
        for (int phase = 0; phase < 3; ++phase) {
            for (int c = tid; c < HX * HY; c += NTHR) {
                const int hi = c % HX, hj = c / HX;
                const int gi = gi0 + hi, gj = gj0 + hj;
                const bool inside = gi >= 0 && gi < L.nx && gj >= 0 && gj < L.ny;
                if (inside) continue;
                const bool gx = in_g(gi, 0), gy = in_g(gj, 1);
                const int out = (!gx) + (!gy);
                if (phase == 0) {
                    if (out) continue;
                    // periodic image: the patch covers the domain, read its valid cell
                    const int wi = ((gi % L.nx) + L.nx) % L.nx - P.ilo, wj = ((gj % L.ny) + L.ny) % L.ny - P.jlo;
                    for (int n = 0; n < NV; ++n)
                        T(hi, hj, n) = Uin[P.offset + (int64_t)n * P.comp_stride + (int64_t)(wj + P.ng) * P.pitch + (wi + P.ng)];
                    continue;
                }
                if (out != phase) continue;
                auto S = [&](int ggi, int ggj, int n) -> double& { return T(ggi - gi0, ggj - gj0, n); };
                const int ihi = L.nx - 1, jhi = L.ny - 1;
                for (int n = 0; n < NV; ++n) {
                    if (gi < 0 || gi > ihi) {
                        const int t = bct(L, 0, gi > ihi, n, NS);
                        const int src = gi < 0 ? -gi - 1 : 2 * ihi - gi + 1;
                        if (t == BCT_FOEXTRAP) S(gi, gj, n) = S(gi < 0 ? 0 : ihi, gj, n);
                        else if (t == BCT_EVEN) S(gi, gj, n) = S(src, gj, n);
                        else if (t == BCT_ODD) S(gi, gj, n) = -S(src, gj, n);
                    }
                    if (gj < 0 || gj > jhi) {
                        const int t = bct(L, 1, gj > jhi, n, NS);
                        const int src = gj < 0 ? -gj - 1 : 2 * jhi - gj + 1;
                        if (t == BCT_FOEXTRAP) S(gi, gj, n) = S(gi, gj < 0 ? 0 : jhi, n);
                        else if (t == BCT_EVEN) S(gi, gj, n) = S(gi, src, n);
                        else if (t == BCT_ODD) S(gi, gj, n) = -S(gi, src, n);
                    }
                }
                const bool mixedBottom = !L.periodic[1] && L.lo[1] == HF_BC_WEDGE;
                const bool below = gj < 0;
                for (int n = 0; n < NV; ++n) {
                    bool fixed = false;
                    fixed = fixed || (gi < 0 && bct(L, 0, 0, n, NS) == BCT_EXT);
                    fixed = fixed || (gi > ihi && bct(L, 0, 1, n, NS) == BCT_EXT);
                    fixed = fixed || (gj < 0 && bct(L, 1, 0, n, NS) == BCT_EXT && !(mixedBottom && below));
                    fixed = fixed || (gj > jhi && bct(L, 1, 1, n, NS) == BCT_EXT);
                    if (fixed) { S(gi, gj, n) = L.inlet[n]; continue; }
                    if (mixedBottom && below) {
                        const double x = L.xlo + (gi + 0.5) * L.dx;
                        const bool wall = x >= L.wedge_start;
                        const int jj = wall ? -gj - 1 : 0;
                        const int ii = min(max(gi, 0), L.nx - 1);
                        double val = S(ii, jj, n);
                        if (wall && n == NS + 1) val = -val;
                        S(gi, gj, n) = val;
                    }
                }
            }
            __syncthreads();
        }
    }

    // 3. faces: x faces (TX+1) x TY, y faces TX x (TY+1)
    constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1);
    for (int f = tid; f < NFX + NFY; f += NTHR) {
        double fl[NV];
        bool ok;
        int ci, cj;
        if (f < NFX) {
            const int fi = f % (TX + 1), fj = f / (TX + 1);
            ci = ti0 + fi; cj = tj0 + fj;
            auto get = [&](int k, int n) { return T(fi + k, fj + 2, n); };
            ok = (ci <= P.nx && cj < P.ny) ? face_flux<NS, 0>(L, P.ilo + ci, P.jlo + cj, first_order, get, fl) : true;
            if (!ok) { for (int n = 0; n < NV; ++n) fl[n] = 0.0; }
            for (int n = 0; n < NV; ++n) sfx[(n * TY + fj) * (TX + 1) + fi] = fl[n];
        } else {
            const int g = f - NFX;
            const int fi = g % TX, fj = g / TX;
            ci = ti0 + fi; cj = tj0 + fj;
            auto get = [&](int k, int n) { return T(fi + 2, fj + k, n); };
            ok = (ci < P.nx && cj <= P.ny) ? face_flux<NS, 1>(L, P.ilo + ci, P.jlo + cj, first_order, get, fl) : true;
            if (!ok) { for (int n = 0; n < NV; ++n) fl[n] = 0.0; }
            for (int n = 0; n < NV; ++n) sfy[(n * (TY + 1) + fj) * TX + fi] = fl[n];
        }
        if (!ok) flag(st, ST_FACE_BAD, cell_base + (int64_t)min(cj, P.ny - 1) * P.nx + min(ci, P.nx - 1));
    }
    __syncthreads();

    // 4. update, validate, combine
    if (tid >= TX * TY) return;
    const int i = tid % TX, j = tid / TX;
    const int ci = ti0 + i, cj = tj0 + j;
    if (ci >= P.nx || cj >= P.ny) return;
    double q[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        const double fL = sfx[(n * TY + j) * (TX + 1) + i], fR = sfx[(n * TY + j) * (TX + 1) + i + 1];
        const double fB = sfy[(n * (TY + 1) + j) * TX + i], fT = sfy[(n * (TY + 1) + j + 1) * TX + i];
        q[n] = T(i + 2, j + 2, n) - cx * (fR - fL) - cy * (fT - fB);
    }
    const int64_t g = P.offset + (int64_t)(cj + P.ng) * P.pitch + (ci + P.ng);
    finish_cell<NS>(q, Uold, g, P.comp_stride, Uout, cell_base + (int64_t)cj * P.nx + ci, st);
}

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

bool make_tensor_map(void* tmap, const double* base, const hf_patch& P, int nv) {
    auto enc = get_encode();
    if (!enc) return false;
    const double* b = base + P.offset;
    if ((reinterpret_cast<uintptr_t>(b) & 15) || (P.pitch & 1) || (P.comp_stride & 1) || (P.ng & 1)) return false;
    cuuint64_t dims[3] = {(cuuint64_t)P.pitch, (cuuint64_t)(P.ny + 2 * P.ng), (cuuint64_t)nv};
    cuuint64_t strides[2] = {(cuuint64_t)P.pitch * 8, (cuuint64_t)P.comp_stride * 8};
    cuuint32_t box[3] = {HX, HY, (cuuint32_t)nv};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(reinterpret_cast<CUtensorMap*>(tmap), CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(b),
                     dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int NS>
static cudaError_t flux_fused_impl(const Level& L, const hf_patch& P, const void* tmap, const double* Uin,
                                   const double* Uold, double* Uout, double h, const double* hdev, int first_order,
                                   int64_t cell_base, DevStatus* st, cudaStream_t s, int64_t* launches) {
    static bool attr = false;
    const size_t smem = FusedSmem<NS>::bytes;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_flux_fused<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    dim3 grid((unsigned)((P.nx + TX - 1) / TX), (unsigned)((P.ny + TY - 1) / TY));
    k_flux_fused<NS><<<grid, NTHR, smem, s>>>(*reinterpret_cast<const CUtensorMap*>(tmap), L, P, Uin, Uold, Uout,
                                              h / L.dx, h / L.dy, hdev, first_order, cell_base, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_flux_fused(int ns, const Level& L, const hf_patch& P, const void* tmap, const double* Uin,
                              const double* Uold, double* Uout, double h, const double* hdev, int first_order,
                              int64_t cell_base, DevStatus* st, cudaStream_t s, int64_t* launches) {
    return ns == 9 ? flux_fused_impl<9>(L, P, tmap, Uin, Uold, Uout, h, hdev, first_order, cell_base, st, s, launches)
                   : flux_fused_impl<10>(L, P, tmap, Uin, Uold, Uout, h, hdev, first_order, cell_base, st, s, launches);
}

// dt = cfl / (max rate of the CFL reduction); dt[1] = dt / 2 (the flow half step)
__global__ void k_dt_from_rate(const DevStatus* __restrict__ st, double cfl, double* __restrict__ dt) {
    if (st->abort_run) return;
    double rate;
    const unsigned long long b = st->rate_bits;
    memcpy(&rate, &b, sizeof rate);
    const double d = cfl / rate;
    dt[0] = d;
    dt[1] = 0.5 * d;
}
cudaError_t launch_dt_from_rate(const DevStatus* st, double cfl, double* dt, cudaStream_t s, int64_t* launches) {
    k_dt_from_rate<<<1, 1, 0, s>>>(st, cfl, dt);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- combine / validate / cfl
template <int NS>
__global__ void k_combine(hf_patch P, const double* __restrict__ Uold, double* __restrict__ U, int64_t cell_base,
                          DevStatus* st) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
    double q[NS + 3];
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) {
        q[n] = 0.5 * Uold[g + n * P.comp_stride] + 0.5 * U[g + n * P.comp_stride];
        U[g + n * P.comp_stride] = q[n];
    }
    Props p;
    if (!properties<NS>(q, p, 1000.0)) flag(st, ST_COMBINE_BAD, cell_base + idx);
}
template <int NS>
__device__ __forceinline__ void validate_one(const hf_patch& P, const double* __restrict__ U, int64_t cell_base,
                                             DevStatus* st, int64_t idx) {
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
    double q[NS + 3];
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) q[n] = U[g + n * P.comp_stride];
    Props p;
    if (!properties<NS>(q, p, 1000.0)) flag(st, ST_STAGE_BAD, cell_base + idx);
}
template <int NS>
__global__ void k_validate(hf_patch P, const double* __restrict__ U, int64_t cell_base, DevStatus* st) {
    if (st->abort_run) return;
    validate_one<NS>(P, U, cell_base, st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
// every patch of a level in one launch: patch blockIdx.y, its first cell index base[p]
template <int NS>
__global__ void k_validate_multi(const hf_patch* __restrict__ patches, const int64_t* __restrict__ base,
                                 const double* __restrict__ U, DevStatus* st) {
    if (st->abort_run) return;
    const hf_patch P = patches[blockIdx.y];
    validate_one<NS>(P, U, base[blockIdx.y], st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// CFL rate of cell idx of patch P (0 outside it or when inadmissible, which is flagged
// with bad index cell_base + idx); the block's warps fold it into st->rate_bits.
template <int NS>
__device__ __forceinline__ void cfl_one(const Level& L, const hf_patch& P, const double* __restrict__ U,
                                        int64_t cell_base, DevStatus* st, int64_t idx) {
    double rate = 0.0;
    if (idx < (int64_t)P.nx * P.ny) {
        const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
        const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
        double q[NS + 3];
#pragma unroll
        for (int n = 0; n < NS + 3; ++n) q[n] = U[g + n * P.comp_stride];
        Props p;
        if (!properties<NS>(q, p, 1000.0)) {
            flag(st, ST_STAGE_BAD, cell_base + idx);
        } else {
            double rho = 0.0;
#pragma unroll
            for (int k = 0; k < NS; ++k) rho += q[k];
            rate = (fabs(q[NS] / rho) + p.a) / L.dx + (fabs(q[NS + 1] / rho) + p.a) / L.dy;
        }
    }
    // warp max then one atomic per warp (max is order independent: deterministic)
    for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
    if ((threadIdx.x & 31) == 0 && rate > 0.0) atomicMax(&st->rate_bits, (unsigned long long)__double_as_longlong(rate));
}
template <int NS>
__global__ void k_cfl(Level L, hf_patch P, const double* __restrict__ U, DevStatus* st) {
    if (st->abort_run) return;
    cfl_one<NS>(L, P, U, 0, st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int NS>
__global__ void k_cfl_multi(Level L, const hf_patch* __restrict__ patches, const int64_t* __restrict__ base,
                            const double* __restrict__ U, DevStatus* st) {
    if (st->abort_run) return;
    const hf_patch P = patches[blockIdx.y];
    cfl_one<NS>(L, P, U, base[blockIdx.y], st, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

#define HF_DISPATCH(ns, call) ((ns) == 9 ? call<9> : call<10>)
cudaError_t launch_combine(int ns, const hf_patch& P, const double* Uold, double* U, int64_t cell_base, DevStatus* st,
                           cudaStream_t s, int64_t* launches) {
    const int64_t n = (int64_t)P.nx * P.ny;
    HF_DISPATCH(ns, k_combine)<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, Uold, U, cell_base, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_validate(int ns, const hf_patch& P, const double* U, int64_t cell_base, DevStatus* st,
                            cudaStream_t s, int64_t* launches) {
    const int64_t n = (int64_t)P.nx * P.ny;
    HF_DISPATCH(ns, k_validate)<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, U, cell_base, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_validate_multi(int ns, const hf_patch* ph, const hf_patch* pd, int npatch, const int64_t* base_dev,
                                  const double* U, DevStatus* st, cudaStream_t s, int64_t* launches) {
    int64_t mc = 1;
    for (int p = 0; p < npatch; ++p) mc = max(mc, (int64_t)ph[p].nx * ph[p].ny);
    HF_DISPATCH(ns, k_validate_multi)<<<dim3((unsigned)((mc + 127) / 128), (unsigned)npatch), 128, 0, s>>>(
        pd, base_dev, U, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_cfl_multi(int ns, const Level& L, const hf_patch* ph, const hf_patch* pd, int npatch,
                             const int64_t* base_dev, const double* U, DevStatus* st, cudaStream_t s,
                             int64_t* launches) {
    int64_t mc = 1;
    for (int p = 0; p < npatch; ++p) mc = max(mc, (int64_t)ph[p].nx * ph[p].ny);
    HF_DISPATCH(ns, k_cfl_multi)<<<dim3((unsigned)((mc + 127) / 128), (unsigned)npatch), 128, 0, s>>>(L, pd, base_dev,
                                                                                                     U, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_cfl(int ns, const Level& L, const hf_patch& P, const double* U, DevStatus* st, cudaStream_t s,
                       int64_t* launches) {
    const int64_t n = (int64_t)P.nx * P.ny;
    HF_DISPATCH(ns, k_cfl)<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(L, P, U, st);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- batch primitives
template <int NS>
__global__ void k_properties(const double* __restrict__ q, int64_t stride, int64_t count, double* p, double* a,
                             double* T, int32_t* status, DevStatus* st) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double s[NS + 3];
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) s[n] = q[n * stride + i];
    Props pr{0.0, 0.0, 0.0};
    const bool ok = properties<NS>(s, pr, 1000.0);
    p[i] = pr.p;
    a[i] = pr.a;
    T[i] = pr.T;
    status[i] = ok ? 0 : 1;
    if (!ok) flag(st, ST_STAGE_BAD, i);
}
template <int NS>
__global__ void k_hllc(const double* __restrict__ l, const double* __restrict__ r, const double* __restrict__ pl,
                       const double* __restrict__ pr, int64_t stride, int64_t count, int dir, double* f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double a[NS + 3], b[NS + 3], o[NS + 3];
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) { a[n] = l[n * stride + i]; b[n] = r[n * stride + i]; }
    const Props A{pl[i], pl[stride + i], pl[2 * stride + i]}, B{pr[i], pr[stride + i], pr[2 * stride + i]};
    if (dir == 0) hllc<NS, NS>(a, b, A, B, o);
    else hllc<NS, NS + 1>(a, b, A, B, o);
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) f[n * stride + i] = o[n];
}
cudaError_t launch_properties(int ns, const double* q, int64_t stride, int64_t count, double* p, double* a, double* T,
                              int32_t* status, DevStatus* st, cudaStream_t s, int64_t* launches) {
    HF_DISPATCH(ns, k_properties)<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(q, stride, count, p, a, T, status, st);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_hllc(int ns, const double* l, const double* r, const double* pl, const double* pr, int64_t stride,
                        int64_t count, int dir, double* f, cudaStream_t s, int64_t* launches) {
    HF_DISPATCH(ns, k_hllc)<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(l, r, pl, pr, stride, count, dir, f);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- interpolation
// ConservativeInterp.cpp:18-51: one thread per coarse cell of the coarsened target
// region; one common minmod slope pair for all components, theta halved (<= 48
// times) until all four children are admissible, theta = 0 otherwise.
template <int NS>
__device__ __forceinline__ void interp_one(const hf_patch& C, const double* __restrict__ Uc, const hf_patch& F,
                                           double* __restrict__ Uf, int rfi0, int rfj0, int rfi1, int rfj1,
                                           int64_t idx) {
    constexpr int NV = NS + 3;
    // coarse index box of the region
    const int ci0 = rfi0 >> 1, cj0 = rfj0 >> 1, ci1 = rfi1 >> 1, cj1 = rfj1 >> 1;
    const int cnx = ci1 - ci0 + 1, cny = cj1 - cj0 + 1;
    if (idx >= (int64_t)cnx * cny) return;
    const int ci = ci0 + (int)(idx % cnx), cj = cj0 + (int)(idx / cnx);
    auto rd = [&](int gi, int gj, int n) {
        return Uc[C.offset + (int64_t)n * C.comp_stride + (int64_t)(gj - C.jlo + C.ng) * C.pitch + (gi - C.ilo + C.ng)];
    };
    double q[NV], sx[NV], sy[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        q[n] = rd(ci, cj, n);
        sx[n] = minmod(q[n] - rd(ci - 1, cj, n), rd(ci + 1, cj, n) - q[n]);
        sy[n] = minmod(q[n] - rd(ci, cj - 1, n), rd(ci, cj + 1, n) - q[n]);
    }
    double theta = 1.0;
    bool accepted = false;
    for (int attempt = 0; attempt < 48; ++attempt) {
        bool good = true;
        for (int b = 0; b < 2 && good; ++b)
            for (int a = 0; a < 2 && good; ++a) {
                double child[NV];
#pragma unroll
                for (int n = 0; n < NV; ++n) child[n] = q[n] + theta * ((a ? 0.25 : -0.25) * sx[n] + (b ? 0.25 : -0.25) * sy[n]);
                Props p;
                good = properties<NS>(child, p, 1000.0);
            }
        if (good) { accepted = true; break; }
        theta *= 0.5;
    }
    if (!accepted) theta = 0.0;
    for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) {
            const int fi = 2 * ci + a, fj = 2 * cj + b;
            if (fi < rfi0 || fi > rfi1 || fj < rfj0 || fj > rfj1) continue;
#pragma unroll
            for (int n = 0; n < NV; ++n)
                Uf[F.offset + (int64_t)n * F.comp_stride + (int64_t)(fj - F.jlo + F.ng) * F.pitch + (fi - F.ilo + F.ng)] =
                    q[n] + theta * ((a ? 0.25 : -0.25) * sx[n] + (b ? 0.25 : -0.25) * sy[n]);
        }
}
template <int NS>
__global__ void k_interp(hf_patch C, const double* __restrict__ Uc, hf_patch F, double* __restrict__ Uf, int rfi0,
                         int rfj0, int rfi1, int rfj1) {
    interp_one<NS>(C, Uc, F, Uf, rfi0, rfj0, rfi1, rfj1, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
// Many regions of one fine patch from one coarse patch: region blockIdx.y is
// regions[4r .. 4r+3] = (i0, j0, i1, j1) in fine level indices.
template <int NS>
__global__ void k_interp_regions(hf_patch C, const double* __restrict__ Uc, hf_patch F, double* __restrict__ Uf,
                                 const int32_t* __restrict__ regions) {
    const int32_t* r = regions + 4 * (int64_t)blockIdx.y;
    interp_one<NS>(C, Uc, F, Uf, r[0], r[1], r[2], r[3], (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
cudaError_t launch_interp_regions(int ns, const hf_patch& C, const double* Uc, const hf_patch& F, double* Uf,
                                  const int32_t* regions_dev, int nregions, int64_t max_coarse_cells, cudaStream_t s,
                                  int64_t* launches) {
    if (nregions <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((max_coarse_cells + 127) / 128), (unsigned)nregions);
    HF_DISPATCH(ns, k_interp_regions)<<<grid, 128, 0, s>>>(C, Uc, F, Uf, regions_dev);
    ++*launches;
    return cudaGetLastError();
}
cudaError_t launch_interp(int ns, const hf_patch& C, const double* Uc, const hf_patch& F, double* Uf,
                          const int32_t* r, cudaStream_t s, int64_t* launches) {
    const int64_t n = (int64_t)((r[2] >> 1) - (r[0] >> 1) + 1) * ((r[3] >> 1) - (r[1] >> 1) + 1);
    HF_DISPATCH(ns, k_interp)<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(C, Uc, F, Uf, r[0], r[1], r[2], r[3]);
    ++*launches;
    return cudaGetLastError();
}

}  // namespace hf
