// Discrete adjoint of one Euler stage (a build-defined extension: the reference has
// no sensitivity code).  The stage (HyperFlow_V3/src/BlockAMR.cpp:210-243, with the
// Heun combination of :266-269) maps the ghost-filled input U to
//     out = c_old U_old + c_h (U - h/dx (Fx[i+1] - Fx[i]) - h/dy (Fy[j+1] - Fy[j])),
// each face flux F = HLLC(MUSCL states of its 4-cell stencil) with the EOS inside.
// Its transpose, with every branch of the forward (minmod selections, per-side
// first-order fallbacks, HLLC wave cases, wall overrides) held fixed:
//   Qbar = c_h outbar;  Fbar(face) = h/dx (Qbar(right cell) - Qbar(left cell));
//   face reverse sweep -> cotangents of the 4 stencil cells (face buffers);
//   gather per ghosted cell;  transpose of the ghost fill -> interior cotangents.
// The roundoff repair of the forward (BlockAMR.cpp:299-334) is taken as the
// identity, and validation has no derivative.
#include "hf_device.cuh"
#include "hf_internal.h"

namespace hf {
namespace {

// Per-species e_k W_k / R (R units), cv_k W_k / R and d(cv_k W_k / R)/dT of one range.
template <int RG>
__device__ __forceinline__ void species_e_cv(int k, double T, double& e, double& cv, double& dcv) {
    const double* c = D_ECOEF.c[RG][k];
    e = fma(T, fma(T, fma(T, fma(T, fma(T, c[4], c[3]), c[2]), c[1]), c[0]), c[5]);
    cv = fma(T, fma(T, fma(T, fma(T, 5.0 * c[4], 4.0 * c[3]), 3.0 * c[2]), 2.0 * c[1]), c[0]);
    dcv = fma(T, fma(T, fma(T, 20.0 * c[4], 12.0 * c[3]), 6.0 * c[2]), 2.0 * c[1]);
}

// properties() of a state with the intermediates its reverse sweep needs.
template <int NS>
struct Eos {
    double rho, ir, zs, u, v, T, cv, gam, p, a;
    double z[NS];
};
template <int NS>
__device__ __forceinline__ bool eos_fwd(const double* q, Eos<NS>& t) {
    Props pr;
    if (!properties<NS>(q, pr, 1000.0)) return false;
    double rho = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) rho += q[k];
    t.rho = rho;
    t.ir = 1.0 / rho;
    t.zs = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        t.z[k] = q[k] * t.ir * INVW.v[k];
        t.zs += t.z[k];
    }
    t.u = q[NS] * t.ir;
    t.v = q[NS + 1] * t.ir;
    t.T = pr.T;
    t.p = pr.p;
    t.a = pr.a;
    double cv = 0.0;
    const int rg = t.T <= TMID ? 0 : 1;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        double e, c, d;
        if (rg == 0) species_e_cv<0>(k, t.T, e, c, d);
        else species_e_cv<1>(k, t.T, e, c, d);
        cv = fma(t.z[k], c, cv);
    }
    t.cv = cv;
    t.gam = 1.0 + t.zs / cv;
    return true;
}
// qb += d(p, a)/dq^T (pb, ab):  p = rho R T zs,  a^2 = gam R T zs,  gam = 1 + zs/cv,
// T from e(T, z) = e_target (e = E/rho - (u^2 + v^2)/2).
template <int NS>
__device__ __forceinline__ void eos_rev(const double* q, const Eos<NS>& t, double pb, double ab, double* qb) {
    const double a2b = t.a > 0.0 ? ab / (2.0 * t.a) : 0.0;
    double Tb = pb * t.rho * RU * t.zs + a2b * t.gam * RU * t.zs;
    double zsb = pb * t.rho * RU * t.T + a2b * t.gam * RU * t.T;
    double rhob = pb * RU * t.T * t.zs;
    const double gamb = a2b * RU * t.T * t.zs;
    zsb += gamb / t.cv;
    const double cvb = -gamb * t.zs / (t.cv * t.cv);
    const int rg = t.T <= TMID ? 0 : 1;
    double ek[NS], cvk[NS], dcvT = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        double d;
        if (rg == 0) species_e_cv<0>(k, t.T, ek[k], cvk[k], d);
        else species_e_cv<1>(k, t.T, ek[k], cvk[k], d);
        dcvT = fma(t.z[k], d, dcvT);
    }
    Tb += cvb * dcvT;
    // T(e_R, z): dT = (de_R - sum_k e_k dz_k) / cv.  Inside the small jump of e(T) at
    // T_mid (no root) the inversion returns T_mid itself, which then does not move
    // with the state: no derivative through T there.
    if (t.T == TMID) Tb = 0.0;
    const double eRb = Tb / t.cv;
    double irb = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const double zb = zsb + cvb * cvk[k] - Tb * ek[k] / t.cv;
        qb[k] += zb * t.ir * INVW.v[k];
        irb = fma(zb, q[k] * INVW.v[k], irb);
    }
    const double eb = eRb / RU;
    qb[NS + 2] += eb * t.ir;
    irb = fma(eb, q[NS + 2], irb);
    const double ub = -eb * t.u, vb = -eb * t.v;
    qb[NS] += ub * t.ir;
    qb[NS + 1] += vb * t.ir;
    irb += ub * q[NS] + vb * q[NS + 1];
    rhob -= irb * t.ir * t.ir;
#pragma unroll
    for (int k = 0; k < NS; ++k) qb[k] += rhob;
}

// Reverse sweep of hllc<NS, N>: lb, rb += dF/dl^T fb, dF/dr^T fb; (plb, alb), (prb, arb)
// += the cotangents of the two sides' p and a.
template <int NS, int N>
__device__ __forceinline__ void hllc_rev(const double* l, const double* r, const Eos<NS>& el, const Eos<NS>& er,
                                         const double* fb, double* lb, double* rb, double& plb, double& alb,
                                         double& prb, double& arb) {
    constexpr int E = NS + 2, NV = NS + 3;
    double rl = 0.0, rr = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) { rl += l[k]; rr += r[k]; }
    const double ul = l[N] / rl, ur = r[N] / rr;
    const double sl1 = ul - el.a, sl2 = ur - er.a, sr1 = ul + el.a, sr2 = ur + er.a;
    const double sl = fmin(sl1, sl2), sr = fmax(sr1, sr2);
    const bool slL = sl1 <= sl2, srL = sr1 >= sr2;
    double rlb = 0.0, rrb = 0.0, ulb = 0.0, urb = 0.0, slb = 0.0, srb = 0.0;
    if (sl >= 0.0 || sr <= 0.0) {
        const bool useL = sl >= 0.0;
        const double* q = useL ? l : r;
        double* qb = useL ? lb : rb;
        const double v = useL ? ul : ur, p = useL ? el.p : er.p, rq = useL ? rl : rr;
        double vb = fb[E] * p, pb = fb[N] + fb[E] * v;
#pragma unroll
        for (int m = 0; m < NV; ++m) {
            qb[m] += fb[m] * v;
            vb = fma(fb[m], q[m], vb);
        }
        // v = q_N / rho_q
        qb[N] += vb / rq;
        const double rqb = -vb * v / rq;
#pragma unroll
        for (int k = 0; k < NS; ++k) qb[k] += rqb;
        if (useL) plb += pb;
        else prb += pb;
        return;
    }
    const double dl = rl * (sl - ul), dr = rr * (sr - ur);
    const double num = er.p - el.p + dl * ul - dr * ur, den = dl - dr;
    const double sm = num / den;
    const bool left = sm >= 0.0;
    const double* q = left ? l : r;
    double* qb = left ? lb : rb;
    const double v = left ? ul : ur, s = left ? sl : sr, p = left ? el.p : er.p, rq = left ? rl : rr;
    const double scale = (s - v) / (s - sm);
    double rs = 0.0, qs = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        rs += q[k] * scale;
        qs += q[k];
    }
    const double Wt = sm + p / (rq * (s - v));
    // f_m = v q_m + [m==N] p + [m==E] p v + s (st_m - q_m)
    double vb = fb[E] * p, pb = fb[N] + fb[E] * v, sb = 0.0, scaleb = 0.0, rsb = 0.0, smb = 0.0;
    double stb[NV];
#pragma unroll
    for (int m = 0; m < NV; ++m) {
        double st = q[m] * scale;
        if (m == N) st = rs * sm;
        if (m == E) st = q[E] * scale + rs * (sm - v) * Wt;
        qb[m] += fb[m] * (v - s);
        vb = fma(fb[m], q[m], vb);
        sb = fma(fb[m], st - q[m], sb);
        stb[m] = fb[m] * s;
    }
#pragma unroll
    for (int m = 0; m < NV; ++m)
        if (m != N && m != E) {
            qb[m] += stb[m] * scale;
            scaleb = fma(stb[m], q[m], scaleb);
        }
    rsb += stb[N] * sm;
    smb += stb[N] * rs;
    {   // estar = q_E scale + rs (sm - v) Wt,  Wt = sm + p / (rq (s - v))
        const double eb = stb[E];
        const double sv = s - v, g = rs * (sm - v);
        qb[E] += eb * scale;
        scaleb = fma(eb, q[E], scaleb);
        rsb += eb * (sm - v) * Wt;
        smb += eb * (rs * Wt + g);
        vb += eb * (-rs * Wt + g * p / (rq * sv * sv));
        pb += eb * g / (rq * sv);
        const double rqb = -eb * g * p / (rq * rq * sv);
        sb -= eb * g * p / (rq * sv * sv);
#pragma unroll
        for (int k = 0; k < NS; ++k) qb[k] += rqb;
    }
    // rs = sum_k q_k scale
#pragma unroll
    for (int k = 0; k < NS; ++k) qb[k] += rsb * scale;
    scaleb = fma(rsb, qs, scaleb);
    // scale = (s - v) / (s - sm)
    {
        const double d = s - sm;
        sb += scaleb * (1.0 / d - (s - v) / (d * d));
        vb -= scaleb / d;
        smb += scaleb * (s - v) / (d * d);
    }
    // sm = num / den
    const double numb = smb / den, denb = -smb * sm / den;
    prb += numb;
    plb -= numb;
    const double dlb = numb * ul + denb, drb = -numb * ur - denb;
    ulb += numb * dl;
    urb -= numb * dr;
    rlb += dlb * (sl - ul);
    slb += dlb * rl;
    ulb -= dlb * rl;
    rrb += drb * (sr - ur);
    srb += drb * rr;
    urb -= drb * rr;
    // the side's (v, s, p, rho_q)
    if (left) {
        ulb += vb;
        slb += sb;
        plb += pb;
    } else {
        urb += vb;
        srb += sb;
        prb += pb;
    }
    // sl = min(ul - al, ur - ar), sr = max(ul + al, ur + ar)
    if (slL) { ulb += slb; alb -= slb; } else { urb += slb; arb -= slb; }
    if (srL) { ulb += srb; alb += srb; } else { urb += srb; arb += srb; }
    // ul = l_N / rl, ur = r_N / rr; rl = sum l_k, rr = sum r_k
    lb[N] += ulb / rl;
    rlb -= ulb * ul / rl;
    rb[N] += urb / rr;
    rrb -= urb * ur / rr;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        lb[k] += rlb;
        rb[k] += rrb;
    }
}

// Reverse sweep of face_flux<NS, D> (hf_flux.cu): stencil cotangents qbar[4][NV].
// Returns false if the forward face failed (then nothing is added).
template <int NS, int D, class Get>
__device__ __forceinline__ bool face_rev(const Level& L, int gi, int gj, int first_order, Get get, const double* fbar_in,
                                         double (*qbar)[NS + 3]) {
    constexpr int NV = NS + 3, N = NS + D;
    double q[4][NV], lq[NV], rq[NV];
    unsigned selL = 0, selR = 0, zeroL = 0, zeroR = 0;  // minmod branch per component
#pragma unroll
    for (int n = 0; n < NV; ++n) {
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k][n] = get(k, n);
        if (first_order) {
            lq[n] = q[1][n];
            rq[n] = q[2][n];
        } else {
            const double x1 = q[1][n] - q[0][n], y1 = q[2][n] - q[1][n];
            const double x2 = q[2][n] - q[1][n], y2 = q[3][n] - q[2][n];
            lq[n] = q[1][n] + 0.5 * minmod(x1, y1);
            rq[n] = q[2][n] - 0.5 * minmod(x2, y2);
            if (!(x1 * y1 > 0.0)) zeroL |= 1u << n;
            else if (fabs(x1) <= fabs(y1)) selL |= 1u << n;
            if (!(x2 * y2 > 0.0)) zeroR |= 1u << n;
            else if (fabs(x2) <= fabs(y2)) selR |= 1u << n;
        }
    }
    Eos<NS> el, er;
    bool fl = false, fr = false;
    if (!eos_fwd<NS>(lq, el)) {
        fl = true;
#pragma unroll
        for (int n = 0; n < NV; ++n) lq[n] = q[1][n];
        if (!eos_fwd<NS>(lq, el)) return false;
    }
    if (!eos_fwd<NS>(rq, er)) {
        fr = true;
#pragma unroll
        for (int n = 0; n < NV; ++n) rq[n] = q[2][n];
        if (!eos_fwd<NS>(rq, er)) return false;
    }
    double fb[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) fb[n] = fbar_in[n];
    // wall-flux override (BlockAMR.cpp:224-229): the overridden components are constants
    const bool loWall = !L.periodic[D] && (L.lo[D] == HF_BC_REFLECTING || L.lo[D] == HF_BC_WEDGE);
    const bool hiWall = !L.periodic[D] && L.hi[D] == HF_BC_REFLECTING;
    const bool mixedBottom = !L.periodic[1] && L.lo[1] == HF_BC_WEDGE;
    const int coord = D == 0 ? gi : gj;
    const double x = L.xlo + (gi + 0.5) * L.dx;
    const bool lowWall = loWall && !(D == 1 && mixedBottom && x < L.wedge_start);
    if ((coord == 0 && lowWall) || (coord == (D == 0 ? L.nx : L.ny) && hiWall)) {
#pragma unroll
        for (int k = 0; k < NS; ++k) fb[k] = 0.0;
        fb[D == 0 ? NS + 1 : NS] = 0.0;
        fb[NS + 2] = 0.0;
    }
    double lb[NV], rb[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) lb[n] = rb[n] = 0.0;
    double plb = 0.0, alb = 0.0, prb = 0.0, arb = 0.0;
    hllc_rev<NS, N>(lq, rq, el, er, fb, lb, rb, plb, alb, prb, arb);
    eos_rev<NS>(lq, el, plb, alb, lb);
    eos_rev<NS>(rq, er, prb, arb, rb);
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        qbar[0][n] = qbar[1][n] = qbar[2][n] = qbar[3][n] = 0.0;
        const double l = lb[n], r = rb[n];
        // lq = qb + mm(qb - qa, qc - qb)/2  (or qb after a fallback / first order)
        qbar[1][n] += l;
        if (!fl && !first_order && !(zeroL >> n & 1u)) {
            if (selL >> n & 1u) { qbar[1][n] += 0.5 * l; qbar[0][n] -= 0.5 * l; }
            else { qbar[2][n] += 0.5 * l; qbar[1][n] -= 0.5 * l; }
        }
        // rq = qc - mm(qc - qb, qd - qc)/2
        qbar[2][n] += r;
        if (!fr && !first_order && !(zeroR >> n & 1u)) {
            if (selR >> n & 1u) { qbar[2][n] -= 0.5 * r; qbar[1][n] += 0.5 * r; }
            else { qbar[3][n] -= 0.5 * r; qbar[2][n] += 0.5 * r; }
        }
    }
    return true;
}

struct GView {  // ghosted patch array
    const double* U;
    hf_patch P;
    __device__ double get(int i, int j, int n) const {
        return U[P.offset + n * P.comp_stride + (int64_t)(j + P.ng) * P.pitch + (i + P.ng)];
    }
};

// One thread per face: Fbar = c (Qbar(right) - Qbar(left)) with Qbar = ch * outbar on
// the interior, then the face's reverse sweep into FA[k][n][face].
template <int NS, int D>
__global__ void __launch_bounds__(64) k_face_adj(Level L, hf_patch P, const double* __restrict__ U,
                                                 const double* __restrict__ outbar, double ch, double c,
                                                 int first_order, double* __restrict__ FA, DevStatus* st) {
    constexpr int NV = NS + 3;
    const int fnx = P.nx + (D == 0), fny = P.ny + (D == 1);
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)fnx * fny) return;
    const int fi = (int)(idx % fnx), fj = (int)(idx / fnx);
    GView v{U, P}, b{outbar, P};
    const int li = D == 0 ? fi - 1 : fi, lj = D == 0 ? fj : fj - 1;  // cell on the low side
    const bool lin = D == 0 ? li >= 0 : lj >= 0;
    const bool rin = D == 0 ? fi < P.nx : fj < P.ny;
    double fb[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        const double qr = rin ? b.get(fi, fj, n) : 0.0, ql = lin ? b.get(li, lj, n) : 0.0;
        fb[n] = c * ch * (qr - ql);
    }
    auto get = [&](int k, int n) { return D == 0 ? v.get(fi - 2 + k, fj, n) : v.get(fi, fj - 2 + k, n); };
    double qb[4][NV];
    if (!face_rev<NS, D>(L, P.ilo + fi, P.jlo + fj, first_order, get, fb, qb)) {
        atomicOr(&st->flags, ST_FACE_BAD);
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int n = 0; n < NV; ++n) qb[k][n] = 0.0;
    }
    const int64_t nf = (int64_t)fnx * fny;
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int n = 0; n < NV; ++n) FA[((int64_t)k * NV + n) * nf + idx] = qb[k][n];
}

// Cotangent of every ghosted cell (the 2-layer frame included, corners unused):
// direct term ch * outbar on the interior plus the face contributions.
template <int NS>
__global__ void k_gather_adj(hf_patch P, const double* __restrict__ outbar, double ch, const double* __restrict__ FAx,
                             const double* __restrict__ FAy, double* __restrict__ UG) {
    constexpr int NV = NS + 3;
    const int W = P.nx + 4, H = P.ny + 4;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)W * H) return;
    const int i = (int)(idx % W) - 2, j = (int)(idx / W) - 2;
    const bool ix = i >= 0 && i < P.nx, jy = j >= 0 && j < P.ny;
    const int64_t g = P.offset + (int64_t)(j + P.ng) * P.pitch + (i + P.ng);
    const int64_t nfx = (int64_t)(P.nx + 1) * P.ny, nfy = (int64_t)P.nx * (P.ny + 1);
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        double s = (ix && jy) ? ch * outbar[g + n * P.comp_stride] : 0.0;
        if (jy)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int fi = i + 2 - k;
                if (fi >= 0 && fi <= P.nx) s += FAx[((int64_t)k * NV + n) * nfx + (int64_t)j * (P.nx + 1) + fi];
            }
        if (ix)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int fj = j + 2 - k;
                if (fj >= 0 && fj <= P.ny) s += FAy[((int64_t)k * NV + n) * nfy + (int64_t)fj * P.nx + i];
            }
        UG[g + n * P.comp_stride] = s;
    }
}

// Source interior cell of a non-corner ghost cell (i, j) under the level's boundary
// conditions (the fill of k_fill / FlowBoundary.hpp:12-36), and the component whose
// sign flips (-1: none).  Returns false for an inflow ghost (a constant).
__device__ __forceinline__ bool ghost_source(const Level& L, int NS, int i, int j, int& si, int& sj, int& flip) {
    flip = -1;
    si = i;
    sj = j;
    if (i < 0 || i >= L.nx) {
        const bool lo = i < 0;
        if (L.periodic[0]) { si = lo ? i + L.nx : i - L.nx; return true; }
        const int bc = lo ? L.lo[0] : L.hi[0];
        if (bc == HF_BC_INFLOW) return false;
        if (bc == HF_BC_TRANSMISSIVE) { si = lo ? 0 : L.nx - 1; return true; }
        si = lo ? -1 - i : 2 * L.nx - 1 - i;  // reflecting
        flip = NS;
        return true;
    }
    const bool lo = j < 0;
    if (L.periodic[1]) { sj = lo ? j + L.ny : j - L.ny; return true; }
    const int bc = lo ? L.lo[1] : L.hi[1];
    if (bc == HF_BC_INFLOW) return false;
    if (bc == HF_BC_TRANSMISSIVE) { sj = lo ? 0 : L.ny - 1; return true; }
    if (bc == HF_BC_WEDGE && L.xlo + (i + 0.5) * L.dx < L.wedge_start) { sj = 0; return true; }
    sj = lo ? -1 - j : 2 * L.ny - 1 - j;  // reflecting (and the wedge surface)
    flip = NS + 1;
    return true;
}

// Transpose of the ghost fill: inbar(cell) = UG(cell) + sum of the ghost cotangents
// whose source is the cell (with the reflected momentum's sign).
template <int NS>
__global__ void k_fill_adj(Level L, hf_patch P, const double* __restrict__ UG, double* __restrict__ inbar) {
    constexpr int NV = NS + 3;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)P.nx * P.ny) return;
    const int ci = (int)(idx % P.nx), cj = (int)(idx / P.nx);
    GView v{UG, P};
    double s[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) s[n] = v.get(ci, cj, n);
    const int gx[4] = {-2, -1, P.nx, P.nx + 1};
    for (int a = 0; a < 8; ++a) {
        const int gi = a < 4 ? gx[a] : ci, gj = a < 4 ? cj : (a - 4 < 2 ? a - 6 : P.ny + (a - 6));
        int si, sj, flip;
        if (!ghost_source(L, NS, gi, gj, si, sj, flip) || si != ci || sj != cj) continue;
#pragma unroll
        for (int n = 0; n < NV; ++n) s[n] += (n == flip ? -1.0 : 1.0) * v.get(gi, gj, n);
    }
    const int64_t g = P.offset + (int64_t)(cj + P.ng) * P.pitch + (ci + P.ng);
#pragma unroll
    for (int n = 0; n < NV; ++n) inbar[g + n * P.comp_stride] = s[n];
}

template <int NS>
cudaError_t stage_adjoint_impl(const Level& L, const hf_patch& P, const double* U, const double* outbar, double ch,
                               double h, int first_order, double* FAx, double* FAy, double* UG, double* inbar,
                               DevStatus* st, cudaStream_t s, int64_t* launches) {
    const int bs = 64;
    const int64_t nfx = (int64_t)(P.nx + 1) * P.ny, nfy = (int64_t)P.nx * (P.ny + 1);
    k_face_adj<NS, 0><<<(unsigned)((nfx + bs - 1) / bs), bs, 0, s>>>(L, P, U, outbar, ch, h / L.dx, first_order, FAx,
                                                                     st);
    k_face_adj<NS, 1><<<(unsigned)((nfy + bs - 1) / bs), bs, 0, s>>>(L, P, U, outbar, ch, h / L.dy, first_order, FAy,
                                                                     st);
    const int64_t ng = (int64_t)(P.nx + 4) * (P.ny + 4), nc = (int64_t)P.nx * P.ny;
    k_gather_adj<NS><<<(unsigned)((ng + 127) / 128), 128, 0, s>>>(P, outbar, ch, FAx, FAy, UG);
    k_fill_adj<NS><<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(L, P, UG, inbar);
    *launches += 4;
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_stage_adjoint(int ns, const Level& L, const hf_patch& P, const double* U, const double* outbar,
                                 double ch, double h, int first_order, double* FAx, double* FAy, double* UG,
                                 double* inbar, DevStatus* st, cudaStream_t s, int64_t* launches) {
    return ns == 9 ? stage_adjoint_impl<9>(L, P, U, outbar, ch, h, first_order, FAx, FAy, UG, inbar, st, s, launches)
                   : stage_adjoint_impl<10>(L, P, U, outbar, ch, h, first_order, FAx, FAy, UG, inbar, st, s, launches);
}

}  // namespace hf
