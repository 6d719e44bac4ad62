// Block-AMR level operations: conserved totals, average_down and reflux.
//   totals        HyperFlow_V3/src/BlockAMR.cpp:347-355 (long double sums over leaf cells)
//   average_down  BlockAMR.cpp:157-159 (AMReX average_down, ratio 2)
//   reflux        BlockAMR.cpp:247-255 (FluxRegister CrseInit / FineAdd /
//                 ClearInternalBorders / Reflux at scale 1)
//   repair        BlockAMR.cpp:299-334 (repairRoundoff over the leaf cells of every level)
// All reductions are deterministic: fixed partitions and fixed combination orders,
// no floating-point atomics in a result (the repair's atomic deficit sum is only the
// fallback past REPAIR_CAP negative entries).
#include <cstddef>
#include <cstring>
#include "hf_internal.h"

namespace hf {

// ---------------------------------------------------------------- totals
// Double-double accumulation (Knuth TwoSum): the sum of many doubles to ~2^-104
// relative, i.e. as good as the reference's long double before rounding to double.
struct DD { double hi, lo; };
__device__ __forceinline__ DD dd_add(DD a, double b) {
    const double s = a.hi + b;
    const double bb = s - a.hi;
    const double err = (a.hi - (s - bb)) + (b - bb);
    const double lo = a.lo + err;
    const double hi = s + lo;
    return DD{hi, lo - (hi - s)};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    DD r = dd_add(a, b.hi);
    const double lo = r.lo + b.lo;
    const double hi = r.hi + lo;
    return DD{hi, lo - (hi - r.hi)};
}

constexpr int TOT_BLOCK = 256;
constexpr int TOT_GRID = 304;  // fixed partition: results independent of the device

// Pass 1: block b sums the cells of a fixed contiguous range (all patches' cells in
// order) into partial[b][n] (double-double, tree order fixed).
__global__ void __launch_bounds__(TOT_BLOCK) k_totals(const hf_patch* __restrict__ patches, int npatch,
                                                      const double* __restrict__ U,
                                                      const uint8_t* __restrict__ mask, int64_t total, int nv,
                                                      double vol, int absolute, DD* __restrict__ partial) {
    __shared__ DD sh[TOT_BLOCK];
    const int64_t per_block = (total + gridDim.x - 1) / gridDim.x;
    const int64_t c0 = (int64_t)blockIdx.x * per_block, c1 = min(total, c0 + per_block);
    for (int n = 0; n < nv; ++n) {
        DD acc{0.0, 0.0};
        int p = 0;
        int64_t base = 0;
        for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            while (p < npatch && c >= base + (int64_t)patches[p].nx * patches[p].ny) {
                base += (int64_t)patches[p].nx * patches[p].ny;
                ++p;
            }
            if (mask && !mask[c]) continue;
            const hf_patch& P = patches[p];
            const int64_t k = c - base;
            const int i = (int)(k % P.nx), j = (int)(k / P.nx);
            const double v = U[P.offset + (int64_t)n * P.comp_stride + (int64_t)(j + P.ng) * P.pitch + (i + P.ng)];
            acc = dd_add(acc, (absolute ? fabs(v) : v) * vol);
        }
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int s = TOT_BLOCK / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] = dd_add(sh[threadIdx.x], sh[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[(int64_t)blockIdx.x * nv + n] = sh[0];
        __syncthreads();
    }
}
// Pass 2: one thread per component adds the block partials in block order.
__global__ void k_totals_final(const DD* __restrict__ partial, int nblocks, int nv, double* __restrict__ out) {
    const int n = threadIdx.x;
    if (n >= nv) return;
    DD acc{0.0, 0.0};
    for (int b = 0; b < nblocks; ++b) acc = dd_add(acc, partial[(int64_t)b * nv + n]);
    out[n] = acc.hi + acc.lo;
}

cudaError_t launch_totals(const hf_patch* patches_dev, int npatch, int64_t total, const double* U, const uint8_t* mask,
                          int nv, double vol, int absolute, void* scratch, double* out_dev, cudaStream_t s,
                          int64_t* launches) {
    DD* partial = static_cast<DD*>(scratch);
    k_totals<<<TOT_GRID, TOT_BLOCK, 0, s>>>(patches_dev, npatch, U, mask, total, nv, vol, absolute, partial);
    k_totals_final<<<1, 32, 0, s>>>(partial, TOT_GRID, nv, out_dev);
    *launches += 2;
    return cudaGetLastError();
}
size_t totals_scratch_bytes(int nv) { return sizeof(DD) * TOT_GRID * nv; }

// ---------------------------------------------------------------- average_down
// One thread per coarse cell under fine patch blockIdx.y: the mean of its four
// children (sum in jref-major, iref-minor order, times 1/4) written into the coarse
// patch that holds the cell.
__global__ void k_average_down(const hf_patch* __restrict__ fine, const double* __restrict__ Uf,
                               const hf_patch* __restrict__ coarse, int ncoarse, double* __restrict__ Uc, int nv) {
    const hf_patch F = fine[blockIdx.y];
    const int cnx = F.nx / 2, cny = F.ny / 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)cnx * cny) return;
    const int ci = F.ilo / 2 + (int)(t % cnx), cj = F.jlo / 2 + (int)(t / cnx);
    for (int q = 0; q < ncoarse; ++q) {
        const hf_patch& C = coarse[q];
        if (ci < C.ilo || ci >= C.ilo + C.nx || cj < C.jlo || cj >= C.jlo + C.ny) continue;
        const int fi = 2 * ci - F.ilo, fj = 2 * cj - F.jlo;
        for (int n = 0; n < nv; ++n) {
            const double* f = Uf + F.offset + (int64_t)n * F.comp_stride;
            double c = 0.0;
            for (int jr = 0; jr < 2; ++jr)
                for (int ir = 0; ir < 2; ++ir) c += f[(int64_t)(fj + jr + F.ng) * F.pitch + (fi + ir + F.ng)];
            Uc[C.offset + (int64_t)n * C.comp_stride + (int64_t)(cj - C.jlo + C.ng) * C.pitch + (ci - C.ilo + C.ng)] =
                0.25 * c;
        }
        return;
    }
}
cudaError_t launch_average_down(const hf_patch* fine_dev, const hf_patch* fine_host, int nfine, const double* Uf,
                                const hf_patch* coarse_dev, int ncoarse, double* Uc, int nv, cudaStream_t s,
                                int64_t* launches) {
    int64_t mx = 1;
    for (int p = 0; p < nfine; ++p) mx = max(mx, (int64_t)(fine_host[p].nx / 2) * (fine_host[p].ny / 2));
    dim3 grid((unsigned)((mx + 127) / 128), (unsigned)nfine);
    k_average_down<<<grid, 128, 0, s>>>(fine_dev, Uf, coarse_dev, ncoarse, Uc, nv);
    ++*launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- reflux
// cover[cj*nxc + ci] = index of the fine patch whose coarsened box holds coarse cell
// (ci, cj), or -1.
__global__ void k_cover_clear(int* cover, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) cover[t] = -1;
}
__global__ void k_cover_mark(const hf_patch* __restrict__ fine, int nxc, int* __restrict__ cover) {
    const hf_patch F = fine[blockIdx.y];
    const int cnx = F.nx / 2, cny = F.ny / 2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)cnx * cny) return;
    const int ci = F.ilo / 2 + (int)(t % cnx), cj = F.jlo / 2 + (int)(t / cnx);
    cover[(int64_t)cj * nxc + ci] = blockIdx.y;
}

// One thread per cell of coarse patch blockIdx.y.  An uncovered cell gathers the
// register h (dA_f (F_f1 + F_f2) - dA_c F_c) of each of its faces (x-lo, x-hi, y-lo,
// y-hi, in that order) whose neighbour is covered, and adds it (low face) or
// subtracts it (high face), divided by the cell volume.
__global__ void k_reflux(Level L, const hf_patch* __restrict__ coarse, const int64_t* __restrict__ cfx_off,
                         const int64_t* __restrict__ cfy_off, const double* __restrict__ fxc,
                         const double* __restrict__ fyc, double* __restrict__ Uc, const hf_patch* __restrict__ fine,
                         const int64_t* __restrict__ ffx_off, const int64_t* __restrict__ ffy_off,
                         const double* __restrict__ fxf, const double* __restrict__ fyf,
                         const int* __restrict__ cover, double h, const double* __restrict__ hdev, int nv) {
    if (hdev) h = *hdev;  // stage length from device memory (graph-captured steps)
    const hf_patch C = coarse[blockIdx.y];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)C.nx * C.ny) return;
    const int li = (int)(t % C.nx), lj = (int)(t / C.nx);
    const int i = C.ilo + li, j = C.jlo + lj;
    if (cover[(int64_t)j * L.nx + i] >= 0) return;
    const double dxc = L.dx, dyc = L.dy, dxf = 0.5 * dxc, dyf = 0.5 * dyc, vol = dxc * dyc;
    const int64_t nfxc = (int64_t)(C.nx + 1) * C.ny, nfyc = (int64_t)C.nx * (C.ny + 1);
    for (int side = 0; side < 4; ++side) {
        const int d = side >> 1, hi = side & 1;
        int ni = i + (d == 0 ? (hi ? 1 : -1) : 0), nj = j + (d == 1 ? (hi ? 1 : -1) : 0);
        if (ni < 0 || ni >= L.nx) {
            if (!L.periodic[0]) continue;
            ni = (ni + L.nx) % L.nx;
        }
        if (nj < 0 || nj >= L.ny) {
            if (!L.periodic[1]) continue;
            nj = (nj + L.ny) % L.ny;
        }
        const int b = cover[(int64_t)nj * L.nx + ni];
        if (b < 0) continue;
        const hf_patch F = fine[b];
        const int64_t nfxf = (int64_t)(F.nx + 1) * F.ny, nfyf = (int64_t)F.nx * (F.ny + 1);
        for (int n = 0; n < nv; ++n) {
            double Fc, F1, F2, dAc, dAf;
            if (d == 0) {
                const int cface = hi ? li + 1 : li;
                Fc = fxc[cfx_off[blockIdx.y] + n * nfxc + (int64_t)lj * (C.nx + 1) + cface];
                const int fi = hi ? 0 : F.nx;
                const int fj0 = 2 * nj - F.jlo;
                const double* fb = fxf + ffx_off[b] + n * nfxf;
                F1 = fb[(int64_t)fj0 * (F.nx + 1) + fi];
                F2 = fb[(int64_t)(fj0 + 1) * (F.nx + 1) + fi];
                dAc = dyc;
                dAf = dyf;
            } else {
                const int cface = hi ? lj + 1 : lj;
                Fc = fyc[cfy_off[blockIdx.y] + n * nfyc + (int64_t)cface * C.nx + li];
                const int fj = hi ? 0 : F.ny;
                const int fi0 = 2 * ni - F.ilo;
                const double* fb = fyf + ffy_off[b] + n * nfyf;
                F1 = fb[(int64_t)fj * F.nx + fi0];
                F2 = fb[(int64_t)fj * F.nx + fi0 + 1];
                dAc = dxc;
                dAf = dxf;
            }
            const double reg = -h * dAc * Fc + h * dAf * (F1 + F2);
            double& u = Uc[C.offset + (int64_t)n * C.comp_stride + (int64_t)(lj + C.ng) * C.pitch + (li + C.ng)];
            u += (hi ? -reg : reg) / vol;
        }
    }
}

cudaError_t launch_reflux(const Level& L, const hf_patch* coarse_dev, const hf_patch* coarse_host, int ncoarse,
                          const int64_t* cfx_off, const int64_t* cfy_off, const double* fxc, const double* fyc,
                          double* Uc, const hf_patch* fine_dev, const hf_patch* fine_host, int nfine,
                          const int64_t* ffx_off, const int64_t* ffy_off, const double* fxf, const double* fyf,
                          int* cover, double h, int nv, cudaStream_t s, int64_t* launches, const double* hdev) {
    const int64_t nc = (int64_t)L.nx * L.ny;
    k_cover_clear<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(cover, nc);
    int64_t mf = 1;
    for (int p = 0; p < nfine; ++p) mf = max(mf, (int64_t)(fine_host[p].nx / 2) * (fine_host[p].ny / 2));
    k_cover_mark<<<dim3((unsigned)((mf + 127) / 128), (unsigned)nfine), 128, 0, s>>>(fine_dev, L.nx, cover);
    int64_t mc = 1;
    for (int p = 0; p < ncoarse; ++p) mc = max(mc, (int64_t)coarse_host[p].nx * coarse_host[p].ny);
    k_reflux<<<dim3((unsigned)((mc + 127) / 128), (unsigned)ncoarse), 128, 0, s>>>(
        L, coarse_dev, cfx_off, cfy_off, fxc, fyc, Uc, fine_dev, ffx_off, ffy_off, fxf, fyf, cover, h, hdev, nv);
    *launches += 3;
    return cudaGetLastError();
}

// ---------------------------------------------------------------- composite roundoff repair
// repairRoundoff (BlockAMR.cpp:299-334) over the leaf cells of levels 0..nlev-1, in the
// reference's order: levels in turn, the patches of a level in table order, the cells
// of a patch row by row.  A cell is identified by its level and its patch-packed index
// (base[p] + row-major index in patch p).
//   scan pass 0: per species the peak partial density and the largest mass
//                (value x cell volume) over all leaf cells;
//   scan pass 1: donor = the first cell (lowest level, then lowest index) holding that
//                mass (the reference keeps the first strictly larger mass);
//   apply:       a negative value beyond 64 ulp of the peak, or a non-finite one, is
//                material (the reference throws); smaller ones are zeroed and their
//                deficits (-value x volume) recorded with the cell's key;
//   fix:         one block sorts the recorded entries by (species, level, cell) and adds
//                each species' deficits in that order, as the reference's loop does,
//                then takes each deficit from its donor (material when the donor's mass
//                does not exceed it).
// Non-negative doubles order like their bit patterns, so maxima are integer atomics.
__device__ __forceinline__ unsigned long long repair_key(int l, int64_t c) {
    return ((unsigned long long)l << 52) | (unsigned long long)c;
}

template <int NS>
__global__ void k_crep_scan(RepairLevel R, int l, int pass, RepairScratch* rs) {
    const hf_patch P = R.patches[blockIdx.y];
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int64_t c = R.base[blockIdx.y] + idx;
    if (R.leaf && !R.leaf[c]) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        const double v = R.U[g + n * P.comp_stride];
        if (!(v > 0.0)) continue;
        const double m = v * R.vol;
        if (pass == 0) {
            atomicMax(&rs->peak_bits[n], (unsigned long long)__double_as_longlong(v));
            if (m > 0.0) atomicMax(&rs->mass_bits[n], (unsigned long long)__double_as_longlong(m));
        } else if (m > 0.0 && (unsigned long long)__double_as_longlong(m) == rs->mass_bits[n]) {
            atomicMin(&rs->donor[n], repair_key(l, c));
        }
    }
}

template <int NS>
__global__ void k_crep_apply(RepairLevel R, int l, RepairScratch* rs, DevStatus* st) {
    const hf_patch P = R.patches[blockIdx.y];
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int64_t c = R.base[blockIdx.y] + idx;
    if (R.leaf && !R.leaf[c]) return;
    const int i = (int)(idx % P.nx), j = (int)(idx / P.nx);
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        double& u = R.U[g + n * P.comp_stride];
        const double v = u;
        if (v >= 0.0) continue;
        const double peak = __longlong_as_double((long long)rs->peak_bits[n]);
        if (!isfinite(v) || -v > 64.0 * 2.220446049250313e-16 * peak) {
            atomicOr(&st->flags, ST_MATERIAL);
            atomicMin(&st->bad_cell, (unsigned long long)c);
            continue;
        }
        const double d = -v * R.vol;
        atomicAdd(&rs->deficit[n], d);
        const unsigned long long k = atomicAdd(&rs->count, 1ull);
        if (k < (unsigned long long)REPAIR_CAP) {
            rs->key[k] = ((unsigned long long)n << 60) | repair_key(l, c);
            rs->val[k] = d;
        }
        atomicAdd(&st->repairs, 1ull);
        u = 0.0;
    }
}

constexpr int REPAIR_FIX_THREADS = 1024;
__global__ void __launch_bounds__(REPAIR_FIX_THREADS) k_crep_fix(RepairLevels R, int ns, RepairScratch* rs,
                                                                  DevStatus* st) {
    __shared__ unsigned long long sk[REPAIR_CAP];
    __shared__ double sv[REPAIR_CAP];
    __shared__ double def[16];
    const unsigned long long cnt = rs->count;
    if (cnt == 0) return;
    const int t = threadIdx.x;
    if (cnt <= (unsigned long long)REPAIR_CAP) {
        int n2 = 2;
        while ((unsigned long long)n2 < cnt) n2 <<= 1;
        for (int i = t; i < n2; i += blockDim.x) {
            const bool in = (unsigned long long)i < cnt;
            sk[i] = in ? rs->key[i] : ~0ull;
            sv[i] = in ? rs->val[i] : 0.0;
        }
        __syncthreads();
        for (int k = 2; k <= n2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = t; i < n2; i += blockDim.x) {
                    const int o = i ^ j;
                    if (o > i && ((sk[i] > sk[o]) == ((i & k) == 0))) {
                        const unsigned long long a = sk[i];
                        sk[i] = sk[o];
                        sk[o] = a;
                        const double b = sv[i];
                        sv[i] = sv[o];
                        sv[o] = b;
                    }
                }
                __syncthreads();
            }
        if (t < ns) {
            double sum = 0.0;
            for (unsigned long long i = 0; i < cnt; ++i)
                if ((int)(sk[i] >> 60) == t) sum += sv[i];
            def[t] = sum;
        }
    } else if (t < ns) {
        def[t] = rs->deficit[t];  // more entries than the sort holds: atomic order
    }
    __syncthreads();
    if (t >= ns) return;
    const double d = def[t];
    if (!(d > 0.0)) return;
    const unsigned long long key = rs->donor[t];
    const double mass = __longlong_as_double((long long)rs->mass_bits[t]);
    if (key == ~0ull || !(mass > d)) {
        atomicOr(&st->flags, ST_MATERIAL);
        return;
    }
    const int l = (int)((key >> 52) & 0xffull);
    const int64_t c = (int64_t)(key & ((1ull << 52) - 1));
    const RepairLevel& L = R.lev[l];
    for (int p = 0; p < L.npatch; ++p) {
        const hf_patch& P = L.patches[p];
        const int64_t b = L.base[p];
        if (c >= b && c < b + (int64_t)P.nx * P.ny) {
            const int64_t k = c - b;
            const int i = (int)(k % P.nx), j = (int)(k / P.nx);
            L.U[P.offset + (int64_t)t * P.comp_stride + (int64_t)(j + P.ng) * P.pitch + (i + P.ng)] -= d / L.vol;
            return;
        }
    }
    atomicOr(&st->flags, ST_MATERIAL);  // unreachable for keys the scan wrote
}

size_t repair_scratch_bytes() { return sizeof(RepairScratch); }

cudaError_t launch_composite_repair(int ns, const RepairLevels& R, RepairScratch* rs, DevStatus* st, cudaStream_t s,
                                    int64_t* launches) {
    cudaError_t e = cudaMemsetAsync(rs, 0, offsetof(RepairScratch, key), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(rs->donor, 0xff, sizeof(rs->donor), s);
    if (e != cudaSuccess) return e;
    for (int pass = 0; pass < 3; ++pass)
        for (int l = 0; l < R.nlev; ++l) {
            const RepairLevel& L = R.lev[l];
            if (L.npatch <= 0) continue;
            const dim3 grid((unsigned)((L.max_cells + 127) / 128), (unsigned)L.npatch);
            if (pass < 2) {
                if (ns == 9) k_crep_scan<9><<<grid, 128, 0, s>>>(L, l, pass, rs);
                else k_crep_scan<10><<<grid, 128, 0, s>>>(L, l, pass, rs);
            } else {
                if (ns == 9) k_crep_apply<9><<<grid, 128, 0, s>>>(L, l, rs, st);
                else k_crep_apply<10><<<grid, 128, 0, s>>>(L, l, rs, st);
            }
            ++*launches;
        }
    k_crep_fix<<<1, REPAIR_FIX_THREADS, 0, s>>>(R, ns, rs, st);
    ++*launches;
    return cudaGetLastError();
}

}  // namespace hf
