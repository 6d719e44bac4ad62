// Per-cell chemistry device code shared by the forward chemistry kernels
// (hf_chem.cu) and the discrete adjoint (hf_adjoint.cu): NASA7 species thermo,
// mass-action kinetics of the generated H2_Li table with its analytic Jacobian,
// the constant-(rho, e) right-hand side of HyperFlow_V3/src/chemistry.cpp:36-53,
// and the Rodas4 cell integrator (Hairer & Wanner, Solving ODEs II, Sec. VI.7,
// KPP coefficient ordering and step controller).
//
// Pre-exponential factors live in __constant__ memory, one copy per translation
// unit (static); each unit that includes this header uploads them with
// upload_rate_constants() (hf::chem_set_rate_scale and hf::adjoint_set_rate_scale).
#pragma once
#include <utility>
#include "hf_device.cuh"
#include "hf_fastmath.cuh"
#include "hf_internal.h"

namespace hf {

static __constant__ double c_A[NR];
static __constant__ double c_A0[NR];

// A_r and A0_r of the table times scale[r] (1 when scale is null): a rate
// multiplier on reaction r (forward and reverse, both falloff limits).
static inline cudaError_t upload_rate_constants(const double* scale) {
    double a[NR], a0[NR];
    for (int r = 0; r < NR; ++r) {
        const double s = scale ? scale[r] : 1.0;
        a[r] = RXN[r].A * s;
        a0[r] = RXN[r].A0 * s;
    }
    cudaError_t e = cudaMemcpyToSymbol(c_A, a, sizeof(a));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_A0, a0, sizeof(a0));
}

// ---------------------------------------------------------------- species thermo
// g/RT = h/RT - s/R with NASA7: h/RT = a0 + a1/2 T + a2/3 T^2 + a3/4 T^3 + a4/5 T^4 + a5/T,
// s/R = a0 lnT + a1 T + a2/2 T^2 + a3/3 T^3 + a4/4 T^4 + a6.  Every species of the
// table switches range at T_mid = 1000 K, so one branch selects the range.
template <int NS, int RG>
__device__ __forceinline__ void species_g_h_r(double T, double lnT, double invT, double* g, double* hRT) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const double* a = D_NASA.c[RG][k];
        hRT[k] = fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25), a[2] * (1.0 / 3.0)), a[1] * 0.5), a[0]) +
                 a[5] * invT;
        const double sR = fma(a[0], lnT, fma(T, fma(T, fma(T, fma(T, a[4] * 0.25, a[3] * (1.0 / 3.0)), a[2] * 0.5), a[1]), a[6]));
        g[k] = hRT[k] - sR;
    }
}
template <int NS>
__device__ __forceinline__ void species_g_h(double T, double lnT, double invT, double* g, double* hRT) {
    if (T <= TMID) species_g_h_r<NS, 0>(T, lnT, invT, g, hRT);
    else species_g_h_r<NS, 1>(T, lnT, invT, g, hRT);
}

// ---------------------------------------------------------------- kinetics
template <int R, int NS>
__device__ __forceinline__ double third_body(const double* C, double Csum) {
    constexpr Reaction rx = RXN[R];
    double M = Csum;
#pragma unroll
    for (int k = 0; k < NS; ++k)
        if (rx.eff[k] != 1.0) M = fma(rx.eff[k] - 1.0, C[k], M);
    return M;
}
// log10 of a constant in [0.5, 2] at compile time: 2 atanh((x-1)/(x+1)) / ln 10 by
// its odd power series (|z| <= 1/3: 40 terms reach the last bit; within 1 ulp of the
// correctly rounded value for the Troe constants 0.8 and 0.5 of the table).
constexpr double const_log10(double x) {
    const double z = (x - 1.0) / (x + 1.0), z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 0; k < 40; ++k) {
        sum += term / (2 * k + 1);
        term *= z2;
    }
    return 2.0 * sum / 2.302585092994045684;
}

// Troe: log10 F and its partial derivatives (d log10F/d log10Pr, d log10F/dT).
template <int R>
__device__ __forceinline__ double troe_log10F(double T, double Pr, double* dPr, double* dT) {
    constexpr Reaction rx = RXN[R];
    constexpr bool noT3 = rx.troeT3 < 1e-20, noT1 = rx.troeT1 > 1e20;
    constexpr bool constFcent = noT3 && noT1 && !rx.hasT2;
    double Fcent, dFcent;
    if constexpr (constFcent) {
        Fcent = rx.troeA;
        dFcent = 0.0;
    } else {
        const double e3 = fexp(-T / rx.troeT3), e1 = fexp(-T / rx.troeT1);
        Fcent = (1 - rx.troeA) * e3 + rx.troeA * e1;
        dFcent = -(1 - rx.troeA) / rx.troeT3 * e3 - rx.troeA / rx.troeT1 * e1;
        if (rx.hasT2) {
            const double e2 = fexp(-rx.troeT2 / T);
            Fcent += e2;
            dFcent += rx.troeT2 / (T * T) * e2;
        }
    }
    const bool prc = !(Pr > 1e-300);
    double lFc;
    if constexpr (constFcent && rx.troeA >= 0.5 && rx.troeA <= 2.0) {
        constexpr double c = const_log10(rx.troeA);  // F_cent is a constant of the table
        lFc = c;
    } else {
        lFc = flog(fmax(Fcent, 1e-300)) * fm::INV_LN10;
    }
    const double lPr = flog(fmax(Pr, 1e-300)) * fm::INV_LN10;
    const double c = -0.4 - 0.67 * lFc, nn = 0.75 - 1.27 * lFc;
    const double x = lPr + c, den = nn - 0.14 * x;
    const double f1 = x / den;
    const double g = 1.0 / (1.0 + f1 * f1);
    if (dPr) *dPr = prc ? 0.0 : lFc * (-2.0 * f1 * g * g) * (nn / (den * den));
    if (dT) {
        const double df1 = (-0.67 * den - x * (-1.27 + 0.14 * 0.67)) / (den * den);
        const double dlF_dlFc = g + lFc * (-2.0 * f1 * g * g) * df1;
        *dT = (Fcent > 1e-300) ? dlF_dlFc * dFcent / (Fcent * 2.302585092994046) : 0.0;
    }
    return lFc * g;
}

// Temperature factors T^b exp(-E/T) of the rate constants, evaluated in one rolled
// loop (one exp body for all reactions): k_inf of every reaction, then k_0 of the
// falloff reactions in reaction order.  Kinds by (b, E): 1 (b = E = 0), 1/T and
// 1/T^2 (E = 0, b = -1, -2), exp(-E/T) (b = 0), T*T*exp(-E/T) (b = 2), otherwise
// exp(b lnT - E/T).
enum : int { ARR_ONE = 0, ARR_INVT = 1, ARR_INVT2 = 2, ARR_EXP = 3, ARR_T2EXP = 4, ARR_EXPB = 5 };
struct ArrTerm {
    int kind;
    double b, E;
};
constexpr int fall_index(int R) {
    int n = 0;
    for (int r = 0; r < R; ++r) n += RXN[r].type == RXN_FALLOFF ? 1 : 0;
    return n;
}
constexpr int NFALL = fall_index(NR);
struct ArrTable {
    ArrTerm t[NR + NFALL];
};
constexpr ArrTable make_arr() {
    ArrTable a{};
    for (int r = 0; r < NR; ++r) {
        const double b = RXN[r].b, E = RXN[r].EaR;
        const int kind = (b == 0.0 && E == 0.0)   ? ARR_ONE
                         : (E == 0.0 && b == -1.0) ? ARR_INVT
                         : (E == 0.0 && b == -2.0) ? ARR_INVT2
                         : (b == 0.0)              ? ARR_EXP
                         : (b == 2.0)              ? ARR_T2EXP
                                                   : ARR_EXPB;
        a.t[r] = ArrTerm{kind, b, E};
        if (RXN[r].type == RXN_FALLOFF) {
            const double b0 = RXN[r].b0, E0 = RXN[r].Ea0R;
            const int k0 = (b0 == 0.0 && E0 == 0.0) ? ARR_ONE : (b0 == 0.0) ? ARR_EXP : ARR_EXPB;
            a.t[NR + fall_index(r)] = ArrTerm{k0, b0, E0};
        }
    }
    return a;
}
__device__ constexpr ArrTable D_ARR = make_arr();

// Per-evaluation shared quantities.
template <int NS>
struct KinCtx {
    double T, lnT, invT, Csum;
    double eg[NS], ieg[NS];   // exp(g_k), exp(-g_k), g = g0/RT
    double hRT[NS];
    double rt_p0;             // R T / p0
    double ar[NR + NFALL];    // temperature factors of k_inf (reactions) and k_0 (falloff)
};
// ARR: also the rate constants' temperature factors (the kinetics of the forward
// chemistry; the adjoint evaluates its own).
template <int NS, bool ARR = true>
__device__ __forceinline__ void kin_setup(double T, const double* C, KinCtx<NS>& k) {
    k.T = T;
    k.lnT = flog(T);
    k.invT = 1.0 / T;
    double g[NS];
    species_g_h<NS>(T, k.lnT, k.invT, g, k.hRT);
#pragma unroll 1
    for (int s = 0; s < NS; ++s) {
        fexp_pair(g[s], k.eg[s], k.ieg[s]);
    }
    if constexpr (ARR) {
#pragma unroll 1
        for (int r = 0; r < NR + NFALL; ++r) {
            const ArrTerm a = D_ARR.t[r];
            double v;
            if (a.kind == ARR_ONE) {
                v = 1.0;
            } else if (a.kind == ARR_INVT) {
                v = k.invT;
            } else if (a.kind == ARR_INVT2) {
                v = k.invT * k.invT;
            } else {
                const double x = a.kind == ARR_EXPB ? fma(a.b, k.lnT, -a.E * k.invT) : -a.E * k.invT;
                const double ex = fexp(x);
                v = a.kind == ARR_T2EXP ? k.T * k.T * ex : ex;
            }
            k.ar[r] = v;
        }
    }
    double cs = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s) cs += C[s];
    k.Csum = cs;
    k.rt_p0 = RU * T * (1.0 / ONE_ATM);
}
template <int R, int NS>
__device__ __forceinline__ double kinf_T(const KinCtx<NS>& kc) {
    return kc.ar[R];
}
template <int R, int NS>
__device__ __forceinline__ double k0_T(const KinCtx<NS>& kc) {
    return kc.ar[NR + fall_index(R)];
}

// Rate constant k (third-body factor included) of reaction R.
template <int R, int NS>
__device__ __forceinline__ double rate_k(const KinCtx<NS>& kc, const double* C, double& M) {
    constexpr Reaction rx = RXN[R];
    const double kinf = c_A[R] * kinf_T<R, NS>(kc);
    if constexpr (rx.type == RXN_ELEMENTARY) {
        M = 0.0;
        return kinf;
    } else if constexpr (rx.type == RXN_THREE_BODY) {
        M = third_body<R, NS>(C, kc.Csum);
        return kinf * M;
    } else {
        M = third_body<R, NS>(C, kc.Csum);
        const double k0 = c_A0[R] * k0_T<R, NS>(kc);
        const double Pr = k0 * M / kinf;
        const double lF = troe_log10F<R>(kc.T, Pr, nullptr, nullptr);
        return kinf * (Pr / (1.0 + Pr)) * fexp(lF * fm::LN10);
    }
}

// 1/Kc = prod_reac exp(-g) prod_prod exp(g) (RT/p0)^dn
template <int R, int NS>
__device__ __forceinline__ double inv_kc(const KinCtx<NS>& kc) {
    constexpr Reaction rx = RXN[R];
    double v = 1.0;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) v *= kc.ieg[rx.reac[i]];
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) v *= kc.eg[rx.prod[i]];
    constexpr int dn = rx.nprod - rx.nreac;
    if constexpr (dn == 1) v *= kc.rt_p0;
    else if constexpr (dn == -1) v /= kc.rt_p0;
    else if constexpr (dn != 0) v *= pow(kc.rt_p0, (double)dn);
    return v;
}

template <int R, int NS>
__device__ __forceinline__ void add_rate(const KinCtx<NS>& kc, const double* C, double* w) {
    constexpr Reaction rx = RXN[R];
    double M;
    const double k = rate_k<R, NS>(kc, C, M);
    double pf = k, pr = k * inv_kc<R, NS>(kc);
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) pf *= C[rx.reac[i]];
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) pr *= C[rx.prod[i]];
    const double q = pf - pr;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) w[rx.reac[i]] -= q;
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) w[rx.prod[i]] += q;
}
template <int NS, size_t... Rs>
__device__ __forceinline__ void all_rates(const KinCtx<NS>& kc, const double* C, double* w, std::index_sequence<Rs...>) {
    (add_rate<(int)Rs, NS>(kc, C, w), ...);
}

// d(w_i)/dC_m into JC[i][m] (rows i < NS-1), d(w_i)/dT into JT[i]; with W, also the
// rate of progress into w exactly as add_rate computes it (same k, 1/Kc, products).
template <int R, int NS, bool W = false>
__device__ __forceinline__ void add_jac(const KinCtx<NS>& kc, const double* C, double* JC, double* JT,
                                        double* w = nullptr) {
    constexpr Reaction rx = RXN[R];
    constexpr int N = NS - 1;
    const double kinf = c_A[R] * kinf_T<R, NS>(kc);
    const double dlnkinf = rx.b * kc.invT + rx.EaR * kc.invT * kc.invT;
    double k, dkdT, dkdM = 0.0, M = 0.0;
    if constexpr (rx.type == RXN_ELEMENTARY) {
        k = kinf;
        dkdT = kinf * dlnkinf;
    } else if constexpr (rx.type == RXN_THREE_BODY) {
        M = third_body<R, NS>(C, kc.Csum);
        k = kinf * M;
        dkdT = k * dlnkinf;
        dkdM = kinf;
    } else {
        M = third_body<R, NS>(C, kc.Csum);
        const double k0 = c_A0[R] * k0_T<R, NS>(kc);
        const double dlnk0 = rx.b0 * kc.invT + rx.Ea0R * kc.invT * kc.invT;
        const double Pr = k0 * M / kinf;
        double dPr, dTF;
        const double lF = troe_log10F<R>(kc.T, Pr, &dPr, &dTF);
        const double F = fexp(lF * fm::LN10);
        const double dlnk_dlnPr = 1.0 - Pr / (1.0 + Pr) + dPr;
        k = kinf * (Pr / (1.0 + Pr)) * F;
        dkdT = k * (dlnkinf + dlnk_dlnPr * (dlnk0 - dlnkinf) + dTF);
        dkdM = M > 0.0 ? k * dlnk_dlnPr / M : k0 * F;
    }
    const double ikc = inv_kc<R, NS>(kc);
    if constexpr (W) {
        double pf = k, pr = k * ikc;
#pragma unroll
        for (int i = 0; i < rx.nreac; ++i) pf *= C[rx.reac[i]];
#pragma unroll
        for (int i = 0; i < rx.nprod; ++i) pr *= C[rx.prod[i]];
        const double q = pf - pr;
#pragma unroll
        for (int i = 0; i < rx.nreac; ++i) w[rx.reac[i]] -= q;
#pragma unroll
        for (int i = 0; i < rx.nprod; ++i) w[rx.prod[i]] += q;
    }
    double Pf = 1.0, Pb = 1.0;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) Pf *= C[rx.reac[i]];
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) Pb *= C[rx.prod[i]];
    const double net = Pf - ikc * Pb;
    // dlnKc/dT = sum nu h/RT / T - dn / T  (d(g/RT)/dT = -h/(R T^2))
    double dh = 0.0;
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) dh += kc.hRT[rx.prod[i]];
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) dh -= kc.hRT[rx.reac[i]];
    constexpr int dn = rx.nprod - rx.nreac;
    const double dlnKc = (dh - (double)dn) * kc.invT;
    const double dqdT = dkdT * net + k * ikc * dlnKc * Pb;
    // dq/dC_m (mass action part) for participants
    double dq[NS];
#pragma unroll
    for (int m = 0; m < NS; ++m) dq[m] = 0.0;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) {
        double p = k;
#pragma unroll
        for (int j = 0; j < rx.nreac; ++j)
            if (j != i) p *= C[rx.reac[j]];
        dq[rx.reac[i]] += p;
    }
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) {
        double p = k * ikc;
#pragma unroll
        for (int j = 0; j < rx.nprod; ++j)
            if (j != i) p *= C[rx.prod[j]];
        dq[rx.prod[i]] -= p;
    }
    if constexpr (rx.type != RXN_ELEMENTARY) {
        const double t = dkdM * net;
#pragma unroll
        for (int m = 0; m < NS; ++m) dq[m] = fma(t, rx.eff[m], dq[m]);
    }
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) {
        const int s = rx.reac[i];
        if (s < N) {
            JT[s] -= dqdT;
#pragma unroll
            for (int m = 0; m < NS; ++m) JC[s * NS + m] -= dq[m];
        }
    }
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) {
        const int s = rx.prod[i];
        if (s < N) {
            JT[s] += dqdT;
#pragma unroll
            for (int m = 0; m < NS; ++m) JC[s * NS + m] += dq[m];
        }
    }
}
template <int NS, size_t... Rs>
__device__ __forceinline__ void all_jac(const KinCtx<NS>& kc, const double* C, double* JC, double* JT,
                                        std::index_sequence<Rs...>) {
    (add_jac<(int)Rs, NS>(kc, C, JC, JT), ...);
}
template <int NS, size_t... Rs>
__device__ __forceinline__ void all_jac_rates(const KinCtx<NS>& kc, const double* C, double* JC, double* JT,
                                              double* w, std::index_sequence<Rs...>) {
    (add_jac<(int)Rs, NS, true>(kc, C, JC, JT, w), ...);
}

// ---------------------------------------------------------------- ODE pieces
template <int NS>
struct ChemCell {
    static constexpr int N = NS - 1;
    double y[N], f0[N], J[N * N];
    double h, t, tend, rho, e, T, Tsave;
    double mom[3];  // rho*u, rho*v, rho*E: chemistry leaves them unchanged
    int steps, attempts;
    bool rejectLast, rejectMore, needJ;
};

// composition of y (Y_0..Y_{N-1}; last species closes) -> z = Y/W, C = rho Y/W
template <int NS>
__device__ __forceinline__ void comp(const double* y, double rho, double* z, double* C) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NS - 1; ++k) {
        s += y[k];
        z[k] = y[k] * INVW.v[k];
        C[k] = rho * z[k];
    }
    z[NS - 1] = (1.0 - s) * INVW.v[NS - 1];
    C[NS - 1] = rho * z[NS - 1];
}

// chemistry.cpp:36-53
template <int NS>
__device__ __noinline__ bool chem_rhs(double rho, double e, double& T, const double* y, double* dy) {
    double z[NS], C[NS], m[6];
    comp<NS>(y, rho, z, C);
    double Tn = T;
    if (!solve_T<NS>(z, e, Tn, m)) return false;
    T = Tn;
    KinCtx<NS> kc;
    kin_setup<NS>(T, C, kc);
    double w[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) w[k] = 0.0;
    all_rates<NS>(kc, C, w, std::make_index_sequence<NR>{});
    bool ok = true;
    const double ir = 1.0 / rho;
#pragma unroll
    for (int k = 0; k < NS - 1; ++k) {
        dy[k] = w[k] * D_MW.v[k] * ir;
        ok = ok && isfinite(dy[k]);
    }
    return ok;
}

template <int NS>
__device__ __noinline__ bool chem_jac(double rho, double e, double& T, const double* y, double* J) {
    constexpr int N = NS - 1, L = NS - 1;
    double z[NS], C[NS], m[6];
    comp<NS>(y, rho, z, C);
    double Tn = T;
    if (!solve_T<NS>(z, e, Tn, m)) return false;
    T = Tn;
    KinCtx<NS> kc;
    kin_setup<NS>(T, C, kc);
    double JC[N * NS], JT[N];
#pragma unroll
    for (int i = 0; i < N * NS; ++i) JC[i] = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) JT[i] = 0.0;
    all_jac<NS>(kc, C, JC, JT, std::make_index_sequence<NR>{});
    // dT/dy_j = -(e_j - e_L)/cv, e_k = R T/W_k (h_k/RT - 1)
    const double cv = poly_cv(m, T);  // cv/R in the z-weighted units of the mixture
    double dTdy[N];
    const double eL = (kc.hRT[L] - 1.0) * INVW.v[L];
#pragma unroll
    for (int j = 0; j < N; ++j) dTdy[j] = -T * ((kc.hRT[j] - 1.0) * INVW.v[j] - eL) / cv;
    const double ir = 1.0 / rho;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const double cl = JC[i * NS + L] * INVW.v[L];
        const double ti = JT[i] * ir;
#pragma unroll
        for (int j = 0; j < N; ++j) J[i * N + j] = D_MW.v[i] * (JC[i * NS + j] * INVW.v[j] - cl + ti * dTdy[j]);
    }
    return true;
}

// chem_rhs and chem_jac at the same y from one temperature solve and one pass over
// the reactions: dy equals chem_rhs's result (same rate arithmetic, same order) and J
// chem_jac's.
template <int NS>
__device__ __noinline__ bool chem_rhs_jac(double rho, double e, double& T, const double* y, double* dy, double* J) {
    constexpr int N = NS - 1, L = NS - 1;
    double z[NS], C[NS], m[6];
    comp<NS>(y, rho, z, C);
    double Tn = T;
    if (!solve_T<NS>(z, e, Tn, m)) return false;
    T = Tn;
    KinCtx<NS> kc;
    kin_setup<NS>(T, C, kc);
    double JC[N * NS], JT[N], w[NS];
#pragma unroll
    for (int i = 0; i < N * NS; ++i) JC[i] = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) JT[i] = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) w[k] = 0.0;
    all_jac_rates<NS>(kc, C, JC, JT, w, std::make_index_sequence<NR>{});
    bool ok = true;
    const double ir = 1.0 / rho;
#pragma unroll
    for (int k = 0; k < NS - 1; ++k) {
        dy[k] = w[k] * D_MW.v[k] * ir;
        ok = ok && isfinite(dy[k]);
    }
    if (!ok) return false;
    const double cv = poly_cv(m, T);
    double dTdy[N];
    const double eL = (kc.hRT[L] - 1.0) * INVW.v[L];
#pragma unroll
    for (int j = 0; j < N; ++j) dTdy[j] = -T * ((kc.hRT[j] - 1.0) * INVW.v[j] - eL) / cv;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const double cl = JC[i * NS + L] * INVW.v[L];
        const double ti = JT[i] * ir;
#pragma unroll
        for (int j = 0; j < N; ++j) J[i * N + j] = D_MW.v[i] * (JC[i * NS + j] * INVW.v[j] - cl + ti * dTdy[j]);
    }
    return true;
}

// ---------------------------------------------------------------- Rodas4
__device__ constexpr double RA[15] = {
    1.544, 0.9466785280815826, 0.2557011698983284, 3.314825187068521, 2.896124015972201,
    0.9986419139977817, 1.221224509226641, 6.019134481288629, 12.53708332932087,
    -0.687886036105895, 1.221224509226641, 6.019134481288629, 12.53708332932087,
    -0.687886036105895, 1.0};
__device__ constexpr double RC[15] = {
    -5.6688, -2.430093356833875, -0.2063599157091915, -0.1073529058151375, -9.594562251023355,
    -20.47028614809616, 7.496443313967647, -10.24680431464352, -33.99990352819905,
    11.7089089320616, 8.083246795921522, -7.981132988064893, -31.52159432874371,
    16.31930543123136, -6.058818238834054};
__device__ constexpr double RM[6] = {1.221224509226641, 6.019134481288629, 12.53708332932087, -0.687886036105895, 1.0, 1.0};
constexpr double RGAMMA = 0.25;
constexpr long MAX_STEPS = 5000;

enum : int { CELL_CONTINUE = 0, CELL_DONE = 1, CELL_FAIL = 2, CELL_MAXSTEPS = 3 };

template <int N>
__device__ __forceinline__ double wrms(const double* v, const double* y0, const double* y1, double rtol, double atol) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const double sc = atol + rtol * fmax(fabs(y0[i]), fabs(y1[i]));
        const double r = v[i] / sc;
        s = fma(r, r, s);
    }
    return fmax(sqrt(s * (1.0 / N)), 1e-10);
}

// LU with partial pivoting in place (P A = L U); the diagonal holds 1/U_kk.
template <int N>
__device__ __forceinline__ bool lu_factor(double* A, int* piv) {
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
        int p = k;
        double best = fabs(A[k * N + k]);
        for (int i = k + 1; i < N; ++i) {
            const double v = fabs(A[i * N + k]);
            if (v > best) { best = v; p = i; }
        }
        if (!(best > 0.0) || !isfinite(best)) return false;
        piv[k] = p;
        if (p != k) {
#pragma unroll
            for (int j = 0; j < N; ++j) { const double t = A[k * N + j]; A[k * N + j] = A[p * N + j]; A[p * N + j] = t; }
        }
        const double inv = 1.0 / A[k * N + k];
        A[k * N + k] = inv;  // the solves multiply by the reciprocal pivot
        for (int i = k + 1; i < N; ++i) {
            const double l = A[i * N + k] * inv;
            A[i * N + k] = l;
            for (int j = k + 1; j < N; ++j) A[i * N + j] = fma(-l, A[k * N + j], A[i * N + j]);
        }
    }
    return true;
}
template <int N>
__device__ __forceinline__ void lu_solve(const double* A, const int* piv, double* b) {
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
        const int p = piv[k];
        if (p != k) { const double t = b[k]; b[k] = b[p]; b[p] = t; }
    }
#pragma unroll 1
    for (int i = 1; i < N; ++i)
        for (int j = 0; j < i; ++j) b[i] = fma(-A[i * N + j], b[j], b[i]);
#pragma unroll 1
    for (int i = N - 1; i >= 0; --i) {
        for (int j = i + 1; j < N; ++j) b[i] = fma(-A[i * N + j], b[j], b[i]);
        b[i] *= A[i * N + i];  // reciprocal pivot
    }
}

// Loads a cell and prepares the integration (chemistry.cpp:55-62 + the starting
// step of the integrator).  Returns CELL_CONTINUE or CELL_FAIL.
template <int NS>
__device__ __noinline__ int cell_begin(ChemCell<NS>& c, const double* u, double dt, double rtol, double atol) {
    constexpr int N = NS - 1;
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
    c.T = pr.T;
#pragma unroll
    for (int k = 0; k < N; ++k) c.y[k] = u[k] * ir;
    // f0 and the first step's Jacobian
    if (!chem_rhs_jac<NS>(c.rho, c.e, c.T, c.y, c.f0, c.J)) return CELL_FAIL;
    c.Tsave = c.T;
    // starting step: Hairer's estimate in time scaled by the interval
    {
        const double Ts = c.T;
        const double d0 = wrms<N>(c.y, c.y, c.y, rtol, atol), d1 = wrms<N>(c.f0, c.y, c.y, rtol, atol) * dt;
        const double hh = d1 < 1e-5 ? 1.0 : fmin(1.0, 0.01 * d0 / d1);
        double yn[N], fy[N];
#pragma unroll
        for (int i = 0; i < N; ++i) yn[i] = c.y[i] + hh * dt * c.f0[i];
        double d2;
        if (chem_rhs<NS>(c.rho, c.e, c.T, yn, fy)) {
#pragma unroll
            for (int i = 0; i < N; ++i) fy[i] = (fy[i] - c.f0[i]) / hh;
            d2 = wrms<N>(fy, c.y, c.y, rtol, atol);
        } else {
            d2 = 1e30;
        }
        c.T = Ts;
        const double mx = fmax(d1, d2);
        const double h1 = mx <= 1e-15 ? 1.0 : pow(0.01 / mx, 0.2);
        c.h = fmin(fmin(100.0 * hh, h1), 1.0) * dt;
    }
    c.h = fmin(c.h, dt);
    c.t = 0.0;
    c.tend = dt;
    c.steps = 0;
    c.attempts = 0;
    c.rejectLast = c.rejectMore = false;
    c.needJ = false;
    return CELL_CONTINUE;
}

// One step attempt (the body of the KPP accept loop).
template <int NS>
__device__ __noinline__ int cell_attempt(ChemCell<NS>& c, double rtol, double atol) {
    constexpr int N = NS - 1;
    if (c.needJ) {
        if (c.steps >= MAX_STEPS) return CELL_MAXSTEPS;
        if (!chem_jac<NS>(c.rho, c.e, c.T, c.y, c.J)) return CELL_FAIL;
        c.Tsave = c.T;
        c.needJ = false;
    }
    if (++c.attempts > 4 * MAX_STEPS) return CELL_MAXSTEPS;
    bool last = false;
    if (c.t + 1.01 * c.h >= c.tend) { c.h = c.tend - c.t; last = true; }
    double Mx[N * N], K[6][N], yn[N], fy[N];
    int piv[N];
    const double inv = 1.0 / (c.h * RGAMMA);
#pragma unroll
    for (int i = 0; i < N * N; ++i) Mx[i] = -c.J[i];
#pragma unroll
    for (int i = 0; i < N; ++i) Mx[i * N + i] += inv;
    bool ok = lu_factor<N>(Mx, piv);
    const double ih = 1.0 / c.h;
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        if (!ok) break;
        const int base = s * (s - 1) / 2;
        if (s == 0) {
#pragma unroll
            for (int i = 0; i < N; ++i) fy[i] = c.f0[i];
        } else {
#pragma unroll
            for (int i = 0; i < N; ++i) {
                double v = c.y[i];
#pragma unroll
                for (int j = 0; j < s; ++j) v = fma(RA[base + j], K[j][i], v);
                yn[i] = v;
            }
            ok = chem_rhs<NS>(c.rho, c.e, c.T, yn, fy);
            if (!ok) break;
        }
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = fy[i];
#pragma unroll
            for (int j = 0; j < s; ++j) v = fma(RC[base + j] * ih, K[j][i], v);
            K[s][i] = v;
        }
        lu_solve<N>(Mx, piv, K[s]);
    }
    double err = __longlong_as_double(0x7ff0000000000000ll);  // +inf
    if (ok) {
        double ev[N];
        bool fin = true;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = c.y[i];
#pragma unroll
            for (int s = 0; s < 6; ++s) v = fma(RM[s], K[s][i], v);
            yn[i] = v;
            ev[i] = K[5][i];
            fin = fin && isfinite(v);
        }
        err = wrms<N>(ev, c.y, yn, rtol, atol);
        if (!fin) err = __longlong_as_double(0x7ff0000000000000ll);
    }
    if (!isfinite(err)) {
        c.T = c.Tsave;
        c.h *= 0.25;
        c.rejectLast = true;
        if (!(c.h > 1e-300) || c.t + c.h == c.t) return CELL_FAIL;
        return CELL_CONTINUE;
    }
    double hnew = c.h * fmin(6.0, fmax(0.2, 0.9 / sqrt(sqrt(err))));
    if (err <= 1.0) {
        c.t = last ? c.tend : c.t + c.h;
#pragma unroll
        for (int i = 0; i < N; ++i) c.y[i] = yn[i];
        if (c.rejectLast) hnew = fmin(hnew, c.h);
        c.rejectLast = c.rejectMore = false;
        ++c.steps;
        c.h = hnew;
        if (!(c.t < c.tend)) return CELL_DONE;
        if (c.steps >= MAX_STEPS) return CELL_MAXSTEPS;
        // f0 and the next step's Jacobian at the new y
        if (!chem_rhs_jac<NS>(c.rho, c.e, c.T, c.y, c.f0, c.J)) return CELL_FAIL;
        c.Tsave = c.T;
        return CELL_CONTINUE;
    }
    if (c.rejectMore) hnew = c.h * 0.1;
    c.rejectMore = c.rejectLast;
    c.rejectLast = true;
    c.T = c.Tsave;
    c.h = hnew;
    if (!(c.h > 1e-300) || c.t + c.h == c.t) return CELL_FAIL;
    return CELL_CONTINUE;
}

// chemistry.cpp:63-70: clip, close the mass with the last species, final check.
// Writes the whole state u (momentum and energy as they came in).
template <int NS>
__device__ __noinline__ bool cell_end(const ChemCell<NS>& c, double* u) {
    constexpr int N = NS - 1;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const double v = c.y[k];
        if (!isfinite(v) || v < -1e-13) return false;
        u[k] = c.rho * fmax(0.0, v);
        s += u[k];
    }
    u[N] = c.rho - s;
    u[NS] = c.mom[0];
    u[NS + 1] = c.mom[1];
    u[NS + 2] = c.mom[2];
    Props pr;
    return properties<NS>(u, pr, c.T);
}

// ---------------------------------------------------------------- batched form
// Batched-form start of a cell (extension to the reference's per-call CVODE
// restart).  After f0 = f(y0) and J = df/dy at y0:
//  * frozen-cell screen: in the scaled variables z_i = y_i / sc_i
//    (sc_i = atol + rtol |y_i|), with a = ||J_z||_inf dt, if a <= 20,
//    ||f0_z||_inf dt e^a <= 1 and ||f0_z||_inf dt a^2 e^a / 6 <= 1e-5, the interval
//    is taken as one second-order Taylor step y1 = y0 + dt f0 + dt^2/2 J f0: for the
//    linearised system its remainder sum_{k>=3} dt^k/k! J^(k-1) f0 is bounded by
//    the last expression, i.e. below 1e-5 tolerance units;
//  * otherwise the first step size is the cell's proposed step from the previous
//    call (h_prev > 0), else the same starting-step estimate as cell_begin; the
//    Jacobian just formed is the first step's Jacobian.
// Returns CELL_DONE (screened), CELL_CONTINUE or CELL_FAIL.
template <int NS>
__device__ __noinline__ int cell_begin_batched(ChemCell<NS>& c, const double* u, double dt, double rtol, double atol,
                                               double h_prev) {
    constexpr int N = NS - 1;
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
    c.T = pr.T;
#pragma unroll
    for (int k = 0; k < N; ++k) c.y[k] = u[k] * ir;
    if (!chem_rhs_jac<NS>(c.rho, c.e, c.T, c.y, c.f0, c.J)) return CELL_FAIL;
    c.Tsave = c.T;
    c.t = 0.0;
    c.tend = dt;
    c.steps = 0;
    c.attempts = 0;
    c.rejectLast = c.rejectMore = false;
    c.needJ = false;
    double sc[N], fz = 0.0, jz = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        sc[i] = atol + rtol * fabs(c.y[i]);
        fz = fmax(fz, fabs(c.f0[i]) / sc[i]);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        double r = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) r = fma(fabs(c.J[i * N + j]), sc[j], r);
        jz = fmax(jz, r / sc[i]);
    }
    // remainder of the second-order Taylor step for the linearised system:
    // ||R||_z <= fz dt * a^2 e^a / 6 with a = jz dt; the whole change stays below
    // fz dt e^a <= 1 tolerance unit, so J is constant over the interval to far
    // better than the tolerance
    const double a = jz * dt;
    const double ea = a <= 20.0 ? exp(a) : 1e300;
    if (a <= 20.0 && fz * dt * ea <= 1.0 && fz * dt * a * a * ea <= 6e-5) {
        double jf[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < N; ++j) v = fma(c.J[i * N + j], c.f0[j], v);
            jf[i] = v;
        }
#pragma unroll
        for (int i = 0; i < N; ++i) c.y[i] = fma(0.5 * dt * dt, jf[i], fma(dt, c.f0[i], c.y[i]));
        c.t = dt;
        c.h = dt;
        return CELL_DONE;
    }
    if (h_prev > 0.0 && isfinite(h_prev)) {
        c.h = fmin(h_prev, dt);
    } else {
        const double Ts = c.T;
        const double d0 = wrms<N>(c.y, c.y, c.y, rtol, atol), d1 = wrms<N>(c.f0, c.y, c.y, rtol, atol) * dt;
        const double hh = d1 < 1e-5 ? 1.0 : fmin(1.0, 0.01 * d0 / d1);
        double yn[N], fy[N];
#pragma unroll
        for (int i = 0; i < N; ++i) yn[i] = c.y[i] + hh * dt * c.f0[i];
        double d2;
        if (chem_rhs<NS>(c.rho, c.e, c.T, yn, fy)) {
#pragma unroll
            for (int i = 0; i < N; ++i) fy[i] = (fy[i] - c.f0[i]) / hh;
            d2 = wrms<N>(fy, c.y, c.y, rtol, atol);
        } else {
            d2 = 1e30;
        }
        c.T = Ts;
        const double mx = fmax(d1, d2);
        const double h1 = mx <= 1e-15 ? 1.0 : pow(0.01 / mx, 0.2);
        c.h = fmin(fmin(100.0 * hh, h1), 1.0) * dt;
    }
    return CELL_CONTINUE;
}

}  // namespace hf
