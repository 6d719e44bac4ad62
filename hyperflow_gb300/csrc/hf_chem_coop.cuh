// Cooperative Rodas4: one cell per group of 8 lanes (4 cells per warp), for the cells
// whose integration is long (the batched form's costliest cells).  One cell per lane
// leaves such a cell's step chain on a single lane; here the 8 reacting species of the
// H2_Li table (H2, O2, H2O, H, O, OH, HO2, H2O2: the unknowns) are spread over the lanes
// of a group, so one step attempt takes a fraction of the sequential FP64 work.
//
// The ODE, the integrator (Rodas4 tableau, WRMS error, KPP controller, step limits) and
// the cell semantics (clip, closing species, final admissibility) are those of the
// per-lane cell code (hf_kinetics.cuh); results agree with it to rounding (sums are
// taken in another order), not bit for bit.
//
// Lane t of a group holds: y_t, f0_t, the stage vectors' component t, row t of J and of
// the LU factors, and evaluates reactions t, t+8, t+16 of the table (data-driven: the
// same instructions on every lane, reaction parameters from a device table).  Group
// sums and maxima use an xor butterfly over the 8 lanes, which leaves bitwise equal
// results in every lane, so all lanes of a group take the same branches.  Lanes of
// other groups may diverge; every shuffle names only its group's lanes.
//
// N2 never reacts in the table.  With the inert AR extension (NS = 10) the reference's
// unknowns Y_0..Y_8 include N2, whose rate, Jacobian row and stage components are exact
// zeros: it is held constant here and the WRMS norm keeps its divisor NS - 1, which
// gives the reference formulation's error norm.
#pragma once
#include "hf_kinetics.cuh"

namespace hf {
namespace coop {

constexpr int G = 8;   // lanes per cell
constexpr int NQ = 8;  // reacting species (the unknowns of the group integrator)
constexpr int NROUND = (NR + G - 1) / G;
constexpr int NLIST = 24;  // capacity of a species' production list

// Reaction parameters per slot r (r >= NR: an empty slot, A = 0).
struct RxnSlot {
    double b, EaR, b0, Ea0R;
    double lfc;          // log10 F_cent (the table's Troe reactions have constant F_cent)
    int type, effset;    // effset: index of the third-body efficiency set, -1 none
    int r0, r1, p0, p1;  // reactant / product species (-1 none)
    int dn;              // products - reactants
};
constexpr int MAX_EFFSETS = 4;
struct CoopTable {
    RxnSlot s[NROUND * G];
    int neff;
    double eff[MAX_EFFSETS][NS_MAX];
    // production list of species t: entries (slot, sign), one per occurrence, in
    // reaction order; padded with sign 0
    int nlist;
    int lr[NQ][NLIST];
    double ls[NQ][NLIST];
};
constexpr double troe_lfc(const Reaction& rx) {
    return (rx.troeT3 < 1e-20 && rx.troeT1 > 1e20 && !rx.hasT2 && rx.troeA >= 0.5 && rx.troeA <= 2.0)
               ? const_log10(rx.troeA)
               : 0.0;
}
constexpr bool same_eff(const double* a, const double* b) {
    for (int k = 0; k < NS_MAX; ++k)
        if (a[k] != b[k]) return false;
    return true;
}
constexpr CoopTable make_coop_table() {
    CoopTable t{};
    t.neff = 0;
    for (int r = 0; r < NROUND * G; ++r) {
        RxnSlot& s = t.s[r];
        s.r0 = s.r1 = s.p0 = s.p1 = -1;
        s.effset = -1;
        if (r >= NR) continue;
        const Reaction& rx = RXN[r];
        s.b = rx.b;
        s.EaR = rx.EaR;
        s.b0 = rx.b0;
        s.Ea0R = rx.Ea0R;
        s.lfc = troe_lfc(rx);
        s.type = rx.type;
        s.r0 = rx.nreac > 0 ? rx.reac[0] : -1;
        s.r1 = rx.nreac > 1 ? rx.reac[1] : -1;
        s.p0 = rx.nprod > 0 ? rx.prod[0] : -1;
        s.p1 = rx.nprod > 1 ? rx.prod[1] : -1;
        s.dn = rx.nprod - rx.nreac;
        if (rx.type != RXN_ELEMENTARY) {
            int q = -1;
            for (int e = 0; e < t.neff; ++e)
                if (same_eff(t.eff[e], rx.eff)) q = e;
            if (q < 0) {
                q = t.neff++;
                for (int k = 0; k < NS_MAX; ++k) t.eff[q][k] = rx.eff[k];
            }
            s.effset = q;
        }
    }
    int mx = 0;
    for (int k = 0; k < NQ; ++k) {
        int n = 0;
        for (int r = 0; r < NR; ++r) {
            const Reaction& rx = RXN[r];
            for (int i = 0; i < rx.nreac; ++i)
                if (rx.reac[i] == k && n < NLIST) { t.lr[k][n] = r; t.ls[k][n] = -1.0; ++n; }
            for (int i = 0; i < rx.nprod; ++i)
                if (rx.prod[i] == k && n < NLIST) { t.lr[k][n] = r; t.ls[k][n] = 1.0; ++n; }
        }
        for (int e = n; e < NLIST; ++e) { t.lr[k][e] = 0; t.ls[k][e] = 0.0; }
        mx = n > mx ? n : mx;
    }
    t.nlist = mx;
    return t;
}
constexpr CoopTable COOP_TABLE = make_coop_table();
constexpr int list_len_max() {
    int mx = 0;
    for (int k = 0; k < NQ; ++k) {
        int n = 0;
        for (int r = 0; r < NR; ++r) n += (RXN[r].nreac > 0 && RXN[r].reac[0] == k) + (RXN[r].nreac > 1 && RXN[r].reac[1] == k) +
                                         (RXN[r].nprod > 0 && RXN[r].prod[0] == k) + (RXN[r].nprod > 1 && RXN[r].prod[1] == k);
        mx = n > mx ? n : mx;
    }
    return mx;
}
static_assert(list_len_max() <= NLIST, "a species' production list is longer than its table");
static_assert(COOP_TABLE.neff <= MAX_EFFSETS, "too many third-body efficiency sets");
__device__ constexpr CoopTable D_COOP = COOP_TABLE;

// The mechanism facts the group integrator relies on
constexpr bool coop_table_ok() {
    for (int r = 0; r < NR; ++r) {
        const Reaction& rx = RXN[r];
        if (rx.nreac > 2 || rx.nprod > 2) return false;
        for (int i = 0; i < rx.nreac; ++i)
            if (rx.reac[i] >= NQ) return false;
        for (int i = 0; i < rx.nprod; ++i)
            if (rx.prod[i] >= NQ) return false;
        if (rx.type == RXN_FALLOFF && troe_lfc(rx) == 0.0) return false;
    }
    return true;
}
static_assert(coop_table_ok(), "the group integrator needs reactions of <= 2 reacting species on each side, "
                               "among the first 8 species, and constant Troe F_cent");

// ---------------------------------------------------------------- group primitives
struct Grp {
    unsigned mask;  // the group's 8 lanes
    int base;       // first lane of the group
    int t;          // lane within the group
};
__device__ __forceinline__ Grp grp() {
    const int lane = threadIdx.x & 31;
    Grp g;
    g.t = lane & (G - 1);
    g.base = lane & ~(G - 1);
    g.mask = 0xffu << g.base;
    return g;
}
__device__ __forceinline__ double gsum(const Grp& g, double v) {
    v += __shfl_xor_sync(g.mask, v, 1);
    v += __shfl_xor_sync(g.mask, v, 2);
    v += __shfl_xor_sync(g.mask, v, 4);
    return v;
}
__device__ __forceinline__ double gmax(const Grp& g, double v) {
    v = fmax(v, __shfl_xor_sync(g.mask, v, 1));
    v = fmax(v, __shfl_xor_sync(g.mask, v, 2));
    v = fmax(v, __shfl_xor_sync(g.mask, v, 4));
    return v;
}
__device__ __forceinline__ double gget(const Grp& g, double v, int src) {
    return __shfl_sync(g.mask, v, g.base + src);
}

// Composition: z_t = y_t / W_t, C_t = rho z_t for the lane's species; zi[0], zi[1]: z of
// N2 and (NS = 10) AR, from the closing of the mass.
template <int NS>
__device__ __forceinline__ void gcomp(const Grp& g, double rho, double yN2, double y, double& z, double& C,
                                      double* zi) {
    const double s = gsum(g, y);
    z = y * INVW.v[g.t];
    C = rho * z;
    if constexpr (NS == 9) {
        zi[0] = (1.0 - s) * INVW.v[8];
        zi[1] = 0.0;
    } else {
        zi[0] = yN2 * INVW.v[8];
        zi[1] = (1.0 - s - yN2) * INVW.v[9];
    }
}

// Mixture polynomial coefficients of one NASA range over all species of the cell.
template <int NS>
__device__ __forceinline__ void gmix(const Grp& g, double z, const double* zi, int range, double* m) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double v = gsum(g, z * D_ECOEF.c[range][g.t][j]);
        v = fma(zi[0], D_ECOEF.c[range][8][j], v);
        if constexpr (NS == 10) v = fma(zi[1], D_ECOEF.c[range][9][j], v);
        m[j] = v;
    }
}

// UV inversion (the FP64 phase of solve_T, from the warm guess T): Newton until the
// applied correction is below 1e-10 T; T_mid flips as solve_T.  m: the FP64 mixture
// coefficients of the range T ends in.
template <int NS>
__device__ __forceinline__ bool gsolve_T(const Grp& g, double z, const double* zi, double e_target, double& T,
                                         double* m) {
    if (!(T > 0.0) || !(T < 1e5)) T = 1000.0;
    const double et = e_target * (1.0 / RU);
    int range = T <= TMID ? 0 : 1;
    gmix<NS>(g, z, zi, range, m);
    int flips = 0;
    for (int it = 0; it < 60; ++it) {
        const int r = T <= TMID ? 0 : 1;
        if (r != range) {
            range = r;
            gmix<NS>(g, z, zi, range, m);
        }
        double dT = (et - poly_e(m, T)) / poly_cv(m, T);
        if (!isfinite(dT)) return false;
        dT = fmin(1000.0, fmax(-1000.0, dT));
        double Tn = T + dT;
        if (!(Tn > 0.0)) Tn = 0.5 * T;
        const double step = fabs(Tn - T);
        if (step <= 1e-10 * Tn) {
            T = Tn;
            const int rf = T <= TMID ? 0 : 1;
            if (rf != range) gmix<NS>(g, z, zi, rf, m);
            return true;
        }
        flips = ((T <= TMID) != (Tn <= TMID) && step < 0.5) ? flips + 1 : 0;
        if (flips >= 2) {
            T = TMID;
            gmix<NS>(g, z, zi, 0, m);
            return true;
        }
        T = Tn;
    }
    return false;
}

// h/RT of species k at T (NASA7).
__device__ __forceinline__ double species_hRT(int k, double T, double invT) {
    const double* a = D_NASA.c[T <= TMID ? 0 : 1][k];
    return fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25), a[2] * (1.0 / 3.0)), a[1] * 0.5), a[0]) + a[5] * invT;
}

// Species thermo of the lane's species: exp(g), exp(-g) with g = g0/RT, and h/RT.
__device__ __forceinline__ void gthermo(int t, double T, double lnT, double invT, double& eg, double& ieg,
                                        double& hRT) {
    const double* a = D_NASA.c[T <= TMID ? 0 : 1][t];
    hRT = species_hRT(t, T, invT);
    const double sR =
        fma(a[0], lnT, fma(T, fma(T, fma(T, fma(T, a[4] * 0.25, a[3] * (1.0 / 3.0)), a[2] * 0.5), a[1]), a[6]));
    fexp_pair(hRT - sR, eg, ieg);
}

// Third-body concentration of efficiency set q: sum_k eff_qk C_k.
template <int NS>
__device__ __forceinline__ double gthird(const Grp& g, int q, double C, const double* Ci) {
    double v = gsum(g, D_COOP.eff[q][g.t] * C);
    v = fma(D_COOP.eff[q][8], Ci[0], v);
    if constexpr (NS == 10) v = fma(D_COOP.eff[q][9], Ci[1], v);
    return v;
}

// Rate constant of slot s (third-body factor included) and, with D, dk/dT and dk/dM.
// kA, kA0: the slot's pre-exponential factors as loaded (c_A, c_A0: rate scaling applied).
template <bool D>
__device__ __forceinline__ double slot_k(const RxnSlot& s, double lnT, double invT, double M, double* dkdT,
                                         double* dkdM, double kA, double kA0) {
    const double kinf = kA * fexp(fma(s.b, lnT, -s.EaR * invT));
    const double dlnkinf = s.b * invT + s.EaR * invT * invT;
    double k = kinf;
    if (s.type == RXN_THREE_BODY) {
        k = kinf * M;
        if (D) {
            *dkdT = k * dlnkinf;
            *dkdM = kinf;
        }
    } else if (s.type == RXN_FALLOFF) {
        const double k0 = kA0 * fexp(fma(s.b0, lnT, -s.Ea0R * invT));
        const double Pr = k0 * M / kinf;
        const double lFc = s.lfc;
        const double lPr = flog(fmax(Pr, 1e-300)) * fm::INV_LN10;
        const double c = -0.4 - 0.67 * lFc, nn = 0.75 - 1.27 * lFc;
        const double x = lPr + c, den = nn - 0.14 * x;
        const double f1 = x / den;
        const double gg = 1.0 / (1.0 + f1 * f1);
        const double F = fexp(lFc * gg * fm::LN10);
        k = kinf * (Pr / (1.0 + Pr)) * F;
        if (D) {
            const double dPr = !(Pr > 1e-300) ? 0.0 : lFc * (-2.0 * f1 * gg * gg) * (nn / (den * den));
            const double dlnk_dlnPr = 1.0 - Pr / (1.0 + Pr) + dPr;
            const double dlnk0 = s.b0 * invT + s.Ea0R * invT * invT;
            *dkdT = k * (dlnkinf + dlnk_dlnPr * (dlnk0 - dlnkinf));
            *dkdM = M > 0.0 ? k * dlnk_dlnPr / M : k0 * F;
        }
    } else if (D) {
        *dkdT = kinf * dlnkinf;
        *dkdM = 0.0;
    }
    return k;
}

// Shared scratch of one group (one cell being integrated).
struct GShared {
    double T;                      // warm start of the next UV solve (the last evaluation's T)
    double q[NROUND * G];          // rates of progress of one evaluation, by slot
    double v[NROUND * G][NQ + 1];  // per-slot rows of d q / d y_j divided by W_j (column NQ: N2)
    double dTdy[NQ];               // dT/dy_j / rho of the unknowns
    double J[NQ][NQ + 1];          // the Jacobian rows of the last evaluation (column NQ: N2)
};

__device__ __forceinline__ double slot_A(int r) { return r < NR ? c_A[r] : 0.0; }
__device__ __forceinline__ double slot_A0(int r) { return r < NR ? c_A0[r] : 0.0; }

// Rates of progress of the lane's slots into sh->q; with D, also each slot's row of
// d q / d y (scaled by 1/W_j) into sh->v.  The participants' C, exp(+-g) and h/RT come
// by shuffle from the lanes holding those species.
template <int NS, bool D>
__device__ __forceinline__ void grates(const Grp& g, double T, double lnT, double invT, double C, const double* Ci,
                                       double eg, double ieg, double hRT, double dTdy_n2, GShared* sh) {
    constexpr int L = NS - 1;  // the species that closes the mass
    const double rt_p0 = RU * T * (1.0 / ONE_ATM);
    double M[MAX_EFFSETS];
#pragma unroll
    for (int q = 0; q < MAX_EFFSETS; ++q) M[q] = q < COOP_TABLE.neff ? gthird<NS>(g, q, C, Ci) : 0.0;
#pragma unroll
    for (int round = 0; round < NROUND; ++round) {
        const int r = round * G + g.t;
        const RxnSlot& s = D_COOP.s[r];
        double Mr = 0.0;
#pragma unroll
        for (int q = 0; q < MAX_EFFSETS; ++q)
            if (s.effset == q) Mr = M[q];
        double dkdT = 0.0, dkdM = 0.0;
        const double k = slot_k<D>(s, lnT, invT, Mr, &dkdT, &dkdM, slot_A(r), slot_A0(r));
        const bool h0 = s.r0 >= 0, h1 = s.r1 >= 0, h2 = s.p0 >= 0, h3 = s.p1 >= 0;
        const int a0 = h0 ? s.r0 : 0, a1 = h1 ? s.r1 : 0, b0 = h2 ? s.p0 : 0, b1 = h3 ? s.p1 : 0;
        const double Ca = gget(g, C, a0), Cb = gget(g, C, a1), Cc = gget(g, C, b0), Cd = gget(g, C, b1);
        const double ia = gget(g, ieg, a0), ib = gget(g, ieg, a1), ec = gget(g, eg, b0), ed = gget(g, eg, b1);
        // 1/Kc = prod_reac exp(-g) prod_prod exp(g) (RT/p0)^dn, in inv_kc's order
        double ikc = 1.0;
        if (h0) ikc *= ia;
        if (h1) ikc *= ib;
        if (h2) ikc *= ec;
        if (h3) ikc *= ed;
        if (s.dn == 1) ikc *= rt_p0;
        else if (s.dn == -1) ikc /= rt_p0;
        double pf = k, pr = k * ikc, Pf = 1.0, Pb = 1.0;
        if (h0) { pf *= Ca; Pf *= Ca; }
        if (h1) { pf *= Cb; Pf *= Cb; }
        if (h2) { pr *= Cc; Pb *= Cc; }
        if (h3) { pr *= Cd; Pb *= Cd; }
        sh->q[r] = pf - pr;
        if constexpr (D) {
            const double ha = gget(g, hRT, a0), hb = gget(g, hRT, a1), hc = gget(g, hRT, b0), hd = gget(g, hRT, b1);
            double dh = 0.0;
            if (h2) dh += hc;
            if (h3) dh += hd;
            if (h0) dh -= ha;
            if (h1) dh -= hb;
            const double net = Pf - ikc * Pb;
            const double dlnKc = (dh - (double)s.dn) * invT;
            const double dqdT = dkdT * net + k * ikc * dlnKc * Pb;
            const double kr = k * ikc;
            const double dr0 = k * (h1 ? Cb : 1.0), dr1 = k * Ca;
            const double dp0 = -kr * (h3 ? Cd : 1.0), dp1 = -kr * Cc;
            const bool tb_on = s.effset >= 0;
            const int es = tb_on ? s.effset : 0;
            const double tb = tb_on ? dkdM * net : 0.0;
            const double dL = tb * D_COOP.eff[es][L] * INVW.v[L];
#pragma unroll
            for (int j = 0; j <= NQ; ++j) {
                if (j == NQ && NS == 9) break;
                double d = tb * D_COOP.eff[es][j];
                if (h0 && s.r0 == j) d += dr0;
                if (h1 && s.r1 == j) d += dr1;
                if (h2 && s.p0 == j) d += dp0;
                if (h3 && s.p1 == j) d += dp1;
                const double dT = j < NQ ? sh->dTdy[j] : dTdy_n2;
                sh->v[r][j] = fma(dqdT, dT, d * INVW.v[j] - dL);
            }
        }
    }
}

// Production rate of the lane's species from sh->q (one signed entry per occurrence,
// in reaction order, as add_rate accumulates it).
__device__ __forceinline__ double gprod(const Grp& g, const GShared* sh) {
    double w = 0.0;
#pragma unroll
    for (int e = 0; e < COOP_TABLE.nlist; ++e) w = fma(D_COOP.ls[g.t][e], sh->q[D_COOP.lr[g.t][e]], w);
    return w;
}

constexpr unsigned long long QNAN_BITS = 0x7ff8000000000000ull;

// chemistry.cpp:36-53 for the group's cell: dy of the lane's species at y (the lane's
// component), the UV inversion warm-started from sh->T, which it updates.  NaN in every
// lane of the group when the inversion fails or any rate is not finite.
template <int NS>
__device__ __noinline__ double grhs(double rho, double e, double yN2, double y, GShared* sh) {
    const Grp g = grp();
    double z, C, zi[2], m[6];
    gcomp<NS>(g, rho, yN2, y, z, C, zi);
    const double Ci[2] = {rho * zi[0], rho * zi[1]};
    double T = sh->T;
    __syncwarp(g.mask);
    if (!gsolve_T<NS>(g, z, zi, e, T, m)) return __longlong_as_double((long long)QNAN_BITS);
    const double lnT = flog(T), invT = 1.0 / T;
    double eg, ieg, hRT;
    gthermo(g.t, T, lnT, invT, eg, ieg, hRT);
    grates<NS, false>(g, T, lnT, invT, C, Ci, eg, ieg, hRT, 0.0, sh);
    __syncwarp(g.mask);
    const double w = gprod(g, sh);
    const double dy = w * D_MW.v[g.t] * (1.0 / rho);
    __syncwarp(g.mask);
    sh->T = T;
    const double bad = gmax(g, isfinite(dy) ? 0.0 : 1.0);
    return bad > 0.0 ? __longlong_as_double((long long)QNAN_BITS) : dy;
}

// chem_rhs_jac for the group's cell: dy as grhs, and the lane's Jacobian row
// d(dy_t)/dy_j left in sh->J[t][0..NQ-1] (column NQ: d/dy_N2 with the AR extension,
// used only by the frozen-cell screen).
template <int NS>
__device__ __noinline__ double grhs_jac(double rho, double e, double yN2, double y, GShared* sh) {
    const Grp g = grp();
    constexpr int L = NS - 1;
    double z, C, zi[2], m[6];
    gcomp<NS>(g, rho, yN2, y, z, C, zi);
    const double Ci[2] = {rho * zi[0], rho * zi[1]};
    double T = sh->T;
    __syncwarp(g.mask);
    if (!gsolve_T<NS>(g, z, zi, e, T, m)) return __longlong_as_double((long long)QNAN_BITS);
    const double lnT = flog(T), invT = 1.0 / T;
    double eg, ieg, hRT;
    gthermo(g.t, T, lnT, invT, eg, ieg, hRT);
    // dT/dy_j = -(e_j - e_L)/cv with e_k = R T / W_k (h_k/RT - 1), kept divided by rho
    const double cv = poly_cv(m, T);
    const double eL = (species_hRT(L, T, invT) - 1.0) * INVW.v[L];
    const double ir = 1.0 / rho;
    sh->dTdy[g.t] = -T * ((hRT - 1.0) * INVW.v[g.t] - eL) / cv * ir;
    double dTdy_n2 = 0.0;
    if constexpr (NS == 10) dTdy_n2 = -T * ((species_hRT(8, T, invT) - 1.0) * INVW.v[8] - eL) / cv * ir;
    __syncwarp(g.mask);
    grates<NS, true>(g, T, lnT, invT, C, Ci, eg, ieg, hRT, dTdy_n2, sh);
    __syncwarp(g.mask);
    const double w = gprod(g, sh);
    const double dy = w * D_MW.v[g.t] * ir;
    double row[NQ + 1];
#pragma unroll
    for (int j = 0; j <= NQ; ++j) row[j] = 0.0;
#pragma unroll
    for (int e2 = 0; e2 < COOP_TABLE.nlist; ++e2) {
        const double sg = D_COOP.ls[g.t][e2];
        const int r = D_COOP.lr[g.t][e2];
#pragma unroll
        for (int j = 0; j <= NQ; ++j) row[j] = fma(sg, sh->v[r][j], row[j]);
    }
    __syncwarp(g.mask);
#pragma unroll
    for (int j = 0; j <= NQ; ++j) sh->J[g.t][j] = D_MW.v[g.t] * row[j];
    sh->T = T;
    __syncwarp(g.mask);
    const double bad = gmax(g, isfinite(dy) ? 0.0 : 1.0);
    return bad > 0.0 ? __longlong_as_double((long long)QNAN_BITS) : dy;
}

// LU with partial pivoting of the row-distributed matrix (lane t holds row t in a[]),
// in place, the diagonal holding 1/U_kk; pivot rows (the lowest row of the largest
// magnitude, as lu_factor) in piv[].  False in every lane when a pivot is zero or not
// finite, or a pivot column holds a non-finite value.
__device__ __forceinline__ bool glu(const Grp& g, double* a, int* piv) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
        const bool mine = g.t >= k;
        const double nonfin = gmax(g, (mine && !isfinite(a[k])) ? 1.0 : 0.0);
        double val = mine ? fabs(a[k]) : -1.0;
        int idx = g.t;
#pragma unroll
        for (int off = 1; off < G; off <<= 1) {
            const double ov = __shfl_xor_sync(g.mask, val, off);
            const int oi = __shfl_xor_sync(g.mask, idx, off);
            if (ov > val || (ov == val && oi < idx)) { val = ov; idx = oi; }
        }
        if (nonfin > 0.0 || !(val > 0.0)) return false;
        piv[k] = idx;
        if (idx != k) {
            const int partner = g.t == k ? idx : (g.t == idx ? k : g.t);
#pragma unroll
            for (int j = 0; j < NQ; ++j) a[j] = gget(g, a[j], partner);
        }
        double rk[NQ];
#pragma unroll
        for (int j = k; j < NQ; ++j) rk[j] = gget(g, a[j], k);
        const double inv = 1.0 / rk[k];
        if (g.t == k) a[k] = inv;  // the solves multiply by the reciprocal pivot
        if (g.t > k) {
            const double l = a[k] * inv;
            a[k] = l;
#pragma unroll
            for (int j = k + 1; j < NQ; ++j) a[j] = fma(-l, rk[j], a[j]);
        }
    }
    return true;
}

// Solves (LU) x = b with the row-distributed factors; b: the lane's component in and out.
__device__ __forceinline__ double gsolve(const Grp& g, const double* a, const int* piv, double b) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
        const int p = piv[k];
        if (p != k) b = gget(g, b, g.t == k ? p : (g.t == p ? k : g.t));
    }
#pragma unroll
    for (int j = 0; j < NQ - 1; ++j) {
        const double bj = gget(g, b, j);
        if (g.t > j) b = fma(-a[j], bj, b);
    }
#pragma unroll
    for (int j = NQ - 1; j >= 0; --j) {
        if (g.t == j) b *= a[j];
        const double xj = gget(g, b, j);
        if (g.t < j) b = fma(-a[j], xj, b);
    }
    return b;
}

// Per-group integrator state (every lane holds the same scalars).
struct GInt {
    double h, t, tend, rho, e, yN2, Tsave;
    double mom[3];
    int steps, attempts;
    bool rejectLast, rejectMore;
};

// WRMS norm of the group's components v against y0, y1 (scale atol + rtol max|y0|,|y1|)
// over the reference's NS - 1 unknowns; `extra`: the squared scaled term of the constant
// N2 where it is not zero.
template <int NS>
__device__ __forceinline__ double gwrms(const Grp& g, double v, double y0, double y1, double rtol, double atol,
                                        double extra = 0.0) {
    const double sc = atol + rtol * fmax(fabs(y0), fabs(y1));
    const double r = v / sc;
    const double s = gsum(g, r * r) + extra;
    return fmax(sqrt(s * (1.0 / (NS - 1))), 1e-10);
}

// One step attempt of the group's cell (cell_attempt).  y, f0 and J (the lane's row, NQ
// entries) are updated on acceptance.
template <int NS>
__device__ __forceinline__ int gattempt(const Grp& g, GInt& c, double& y, double& f0, double* J, double rtol,
                                        double atol, GShared* sh) {
    if (++c.attempts > 4 * MAX_STEPS) return CELL_MAXSTEPS;
    bool last = false;
    if (c.t + 1.01 * c.h >= c.tend) {
        c.h = c.tend - c.t;
        last = true;
    }
    double a[NQ];
    int piv[NQ];
    const double inv = 1.0 / (c.h * RGAMMA);
#pragma unroll
    for (int j = 0; j < NQ; ++j) a[j] = j == g.t ? -J[j] + inv : -J[j];
    bool ok = glu(g, a, piv);
    const double ih = 1.0 / c.h;
    double K[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) K[s] = 0.0;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        if (!ok) break;
        const int base = s * (s - 1) / 2;
        double fy;
        if (s == 0) {
            fy = f0;
        } else {
            double v = y;
#pragma unroll
            for (int j = 0; j < s; ++j) v = fma(RA[base + j], K[j], v);
            fy = grhs<NS>(c.rho, c.e, c.yN2, v, sh);
            ok = isfinite(fy);  // the same in every lane of the group
            if (!ok) break;
        }
        double v = fy;
#pragma unroll
        for (int j = 0; j < s; ++j) v = fma(RC[base + j] * ih, K[j], v);
        K[s] = gsolve(g, a, piv, v);
    }
    double err = __longlong_as_double(0x7ff0000000000000ll);  // +inf
    double yn = y;
    if (ok) {
        double v = y;
#pragma unroll
        for (int s = 0; s < 6; ++s) v = fma(RM[s], K[s], v);
        yn = v;
        err = gwrms<NS>(g, K[5], y, yn, rtol, atol);
        if (gmax(g, isfinite(v) ? 0.0 : 1.0) > 0.0) err = __longlong_as_double(0x7ff0000000000000ll);
    }
    if (!isfinite(err)) {
        sh->T = c.Tsave;
        c.h *= 0.25;
        c.rejectLast = true;
        if (!(c.h > 1e-300) || c.t + c.h == c.t) return CELL_FAIL;
        return CELL_CONTINUE;
    }
    double hnew = c.h * fmin(6.0, fmax(0.2, 0.9 / sqrt(sqrt(err))));
    if (err <= 1.0) {
        c.t = last ? c.tend : c.t + c.h;
        y = yn;
        if (c.rejectLast) hnew = fmin(hnew, c.h);
        c.rejectLast = c.rejectMore = false;
        ++c.steps;
        c.h = hnew;
        if (!(c.t < c.tend)) return CELL_DONE;
        if (c.steps >= MAX_STEPS) return CELL_MAXSTEPS;
        // f0 and the next step's Jacobian at the new y
        f0 = grhs_jac<NS>(c.rho, c.e, c.yN2, y, sh);
        if (!isfinite(f0)) return CELL_FAIL;
#pragma unroll
        for (int j = 0; j < NQ; ++j) J[j] = sh->J[g.t][j];
        c.Tsave = sh->T;
        return CELL_CONTINUE;
    }
    if (c.rejectMore) hnew = c.h * 0.1;
    c.rejectMore = c.rejectLast;
    c.rejectLast = true;
    sh->T = c.Tsave;
    c.h = hnew;
    if (!(c.h > 1e-300) || c.t + c.h == c.t) return CELL_FAIL;
    return CELL_CONTINUE;
}

// cell_begin_batched for the group's cell u (NS + 3 values, read by every lane).
// Returns CELL_CONTINUE, CELL_DONE (frozen-cell Taylor step) or CELL_FAIL.
template <int NS>
__device__ __forceinline__ int gbegin(const Grp& g, GInt& c, double& y, double& f0, double* J, const double* u,
                                      double dt, double rtol, double atol, double h_prev, GShared* sh) {
    if (!(dt > 0.0) || !isfinite(dt)) return CELL_FAIL;
    Props pr;
    if (!properties<NS>(u, pr, 1000.0)) return CELL_FAIL;
    double rho = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) rho += u[k];
    const double ir = 1.0 / rho;
    const double uu = u[NS] * ir, vv = u[NS + 1] * ir;
    c.rho = rho;
    c.e = u[NS + 2] * ir - 0.5 * (uu * uu + vv * vv);
    c.mom[0] = u[NS];
    c.mom[1] = u[NS + 1];
    c.mom[2] = u[NS + 2];
    c.yN2 = NS == 10 ? u[8] * ir : 0.0;
    y = u[g.t] * ir;
    __syncwarp(g.mask);
    sh->T = pr.T;
    f0 = grhs_jac<NS>(c.rho, c.e, c.yN2, y, sh);
    if (!isfinite(f0)) return CELL_FAIL;
#pragma unroll
    for (int j = 0; j < NQ; ++j) J[j] = sh->J[g.t][j];
    const double jn2 = NS == 10 ? sh->J[g.t][NQ] : 0.0;
    c.Tsave = sh->T;
    c.t = 0.0;
    c.tend = dt;
    c.steps = 0;
    c.attempts = 0;
    c.rejectLast = c.rejectMore = false;
    // frozen-cell screen (cell_begin_batched) in z_i = y_i / sc_i over the reference's
    // unknowns; with the AR extension the constant N2 has f0 = 0 and a zero Jacobian row,
    // but its column enters the row sums
    const double sc = atol + rtol * fabs(y);
    const double scn2 = NS == 10 ? atol + rtol * fabs(c.yN2) : 0.0;
    const double fz = gmax(g, fabs(f0) / sc);
    double rs = 0.0;
#pragma unroll
    for (int j = 0; j < NQ; ++j) rs = fma(fabs(J[j]), gget(g, sc, j), rs);
    if constexpr (NS == 10) rs = fma(fabs(jn2), scn2, rs);
    const double jz = gmax(g, rs / sc);
    const double aa = jz * dt;
    const double ea = aa <= 20.0 ? exp(aa) : 1e300;
    if (aa <= 20.0 && fz * dt * ea <= 1.0 && fz * dt * aa * aa * ea <= 6e-5) {
        double jf = 0.0;
#pragma unroll
        for (int j = 0; j < NQ; ++j) jf = fma(J[j], gget(g, f0, j), jf);
        y = fma(0.5 * dt * dt, jf, fma(dt, f0, y));
        c.t = dt;
        c.h = dt;
        return CELL_DONE;
    }
    if (h_prev > 0.0 && isfinite(h_prev)) {
        c.h = fmin(h_prev, dt);
    } else {
        const double Ts = sh->T;
        // d0 includes the constant N2 component (y/sc); f0 and the difference quotient
        // are zero there
        double ex = 0.0;
        if constexpr (NS == 10) {
            const double r = c.yN2 / (atol + rtol * fabs(c.yN2));
            ex = r * r;
        }
        const double d0 = gwrms<NS>(g, y, y, y, rtol, atol, ex), d1 = gwrms<NS>(g, f0, y, y, rtol, atol) * dt;
        const double hh = d1 < 1e-5 ? 1.0 : fmin(1.0, 0.01 * d0 / d1);
        const double yn = y + hh * dt * f0;
        const double fy = grhs<NS>(c.rho, c.e, c.yN2, yn, sh);
        const double d2 = isfinite(fy) ? gwrms<NS>(g, (fy - f0) / hh, y, y, rtol, atol) : 1e30;
        sh->T = Ts;
        const double mx = fmax(d1, d2);
        const double h1 = mx <= 1e-15 ? 1.0 : pow(0.01 / mx, 0.2);
        c.h = fmin(fmin(100.0 * hh, h1), 1.0) * dt;
    }
    c.h = fmin(c.h, dt);
    return CELL_CONTINUE;
}

// cell_end for the group's cell: the state (NS + 3 values) into every lane's u[] and the
// final admissibility check.
template <int NS>
__device__ __forceinline__ bool gend(const Grp& g, const GInt& c, double y, double* u, double T) {
    const bool badv = !isfinite(y) || y < -1e-13;
    if (gmax(g, badv ? 1.0 : 0.0) > 0.0) return false;
    const double mine = c.rho * fmax(0.0, y);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
        u[k] = gget(g, mine, k);
        s += u[k];
    }
    if constexpr (NS == 10) {
        u[8] = c.rho * fmax(0.0, c.yN2);
        s += u[8];
    }
    u[NS - 1] = c.rho - s;
    u[NS] = c.mom[0];
    u[NS + 1] = c.mom[1];
    u[NS + 2] = c.mom[2];
    Props pr;
    return properties<NS>(u, pr, T);
}

}  // namespace coop
}  // namespace hf
