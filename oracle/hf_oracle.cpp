// CPU oracle for the HyperFlow V3 reacting-Euler step.  TEST INFRASTRUCTURE ONLY:
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg call it to check
// results; the GPU library never links, loads or calls it.
//
// It restates, in plain C++17 on the reference's own AoS state layout
// (12 doubles per cell: rhoY_0..rhoY_8, rho*u, rho*v, rho*E), the semantics of
//   HyperFlow_V3/src/solver.hpp:17-30        state layout, density, internal energy
//   HyperFlow_V3/src/physics.cpp:4-48        properties, hllc, minmod, admissible
//   HyperFlow_V3/src/BlockAMR.cpp:202-270    Euler stage, wall override, update, Heun
//   HyperFlow_V3/src/BlockAMR.cpp:286-346    validate, repairRoundoff, stableDt
//   HyperFlow_V3/src/BlockAMR.cpp:400-419    Strang step with rollback and dt halving
//   HyperFlow_V3/src/FlowBoundary.hpp:7-37 + BlockAMR.cpp:48-59 + AMReX FillPatch order
//   HyperFlow_V3/src/ConservativeInterp.cpp:18-51  coarse->fine interpolation
//   HyperFlow_V3/src/chemistry.cpp:36-76, chemistry_batch.cpp:21-50
// The third-party arithmetic the reference calls (Cantera 3.2.0 ideal-gas NASA7
// thermo, setState_UV, GasKinetics net production rates; SUNDIALS 7.5.0 CVODE) is
// not present here, so it is restated from the published formulas:
//   * NASA7 cp/R, h/RT, s/R; T <= T_mid uses the low range.
//   * UV inversion: Newton on T, converged to machine precision (Cantera stops at
//     1e-11 relative from whatever guess the phase held; see properties()).
//   * Mass-action kinetics, third-body [M] with efficiencies, Troe falloff
//     (Gilbert et al. 1983, Cantera's TroeRate), reverse rates from Kc built from
//     standard-state Gibbs energies at p0 = 1 atm.
//   * The stiff integrator is Rodas4 (Hairer & Wanner 1996, "Solving ODEs II",
//     Sec. VI.7), with the coefficients of the KPP rosenbrock integrator
//     (Sandu et al. 1997), WRMS error weights atol + rtol*|y| as in CVODE, and
//     Hairer's initial step estimate.  It replaces CVODE BDF; the ODE itself
//     (8 unknowns Y_0..Y_7, N2 dependent, T from the UV inversion at every RHS)
//     is exactly the reference's.
// Parity status: the ghost-fill semantics are pinned exactly against the
// known-answer values of HyperFlow_V3/tests/boundary_check.cpp.  The thermo and
// kinetics restatement of Cantera is otherwise parity unpinned (Cantera absent);
// it is checked by identities (equilibrium detailed balance, element
// conservation, UV round trips, h(T) continuity) in tests/test_oracle.py.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../hyperflow_gb300/csrc/mech_h2li.h"

namespace {
using namespace hfmech;

int NS = 9;                 // active species count (9 = H2_Li.yaml, 10 = with inert AR)
inline int NV() { return NS + 3; }
inline int MX() { return NS; }
inline int MY() { return NS + 1; }
inline int EN() { return NS + 2; }
constexpr int MAXV = NS_MAX + 3;
constexpr double R = GAS_CONSTANT;

// ---------------------------------------------------------------- flop counting
// The thermo, UV inversion and kinetics functions below are templates on the scalar
// type: the oracle runs them on double; on Fl they count their own floating-point work
// (add, sub, mul, div, sqrt: one flop each; exp, log, log10, pow: transcendental calls,
// counted apart), which gives the FP64 work of one right-hand side and one Jacobian
// as this restatement does it.  Operations between constants (the mechanism's table
// values) are folded at compile time and not counted.
thread_local long g_fl_ops = 0, g_fl_trans = 0;
struct Fl {
    double v;
    Fl() = default;
    Fl(double x) : v(x) {}
};
inline Fl operator+(Fl a, Fl b) { ++g_fl_ops; return Fl(a.v + b.v); }
inline Fl operator-(Fl a, Fl b) { ++g_fl_ops; return Fl(a.v - b.v); }
inline Fl operator*(Fl a, Fl b) { ++g_fl_ops; return Fl(a.v * b.v); }
inline Fl operator/(Fl a, Fl b) { ++g_fl_ops; return Fl(a.v / b.v); }
inline Fl operator-(Fl a) { return Fl(-a.v); }
inline Fl& operator+=(Fl& a, Fl b) { a = a + b; return a; }
inline Fl& operator-=(Fl& a, Fl b) { a = a - b; return a; }
inline Fl& operator*=(Fl& a, Fl b) { a = a * b; return a; }
inline Fl& operator/=(Fl& a, Fl b) { a = a / b; return a; }
inline bool operator<(Fl a, Fl b) { return a.v < b.v; }
inline bool operator<=(Fl a, Fl b) { return a.v <= b.v; }
inline bool operator>(Fl a, Fl b) { return a.v > b.v; }
inline bool operator>=(Fl a, Fl b) { return a.v >= b.v; }
inline double val(double x) { return x; }
inline double val(Fl x) { return x.v; }
inline double xexp(double x) { return std::exp(x); }
inline double xlog(double x) { return std::log(x); }
inline double xlog10(double x) { return std::log10(x); }
inline double xpow(double x, double y) { return std::pow(x, y); }
inline double xsqrt(double x) { return std::sqrt(x); }
inline double xfabs(double x) { return std::fabs(x); }
inline double xmax(double a, double b) { return std::max(a, b); }
inline double xmin(double a, double b) { return std::min(a, b); }
inline bool xfinite(double x) { return std::isfinite(x); }
inline double xcopysign(double a, double b) { return std::copysign(a, b); }
inline Fl xexp(Fl x) { ++g_fl_trans; return Fl(std::exp(x.v)); }
inline Fl xlog(Fl x) { ++g_fl_trans; return Fl(std::log(x.v)); }
inline Fl xlog10(Fl x) { ++g_fl_trans; return Fl(std::log10(x.v)); }
inline Fl xpow(Fl x, Fl y) { ++g_fl_trans; return Fl(std::pow(x.v, y.v)); }
inline Fl xsqrt(Fl x) { ++g_fl_ops; return Fl(std::sqrt(x.v)); }
inline Fl xfabs(Fl x) { return Fl(std::fabs(x.v)); }
inline Fl xmax(Fl a, Fl b) { return Fl(std::max(a.v, b.v)); }
inline Fl xmin(Fl a, Fl b) { return Fl(std::min(a.v, b.v)); }
inline bool xfinite(Fl x) { return std::isfinite(x.v); }
inline Fl xcopysign(Fl a, Fl b) { return Fl(std::copysign(a.v, b.v)); }
// Newton iterations of the UV inversion when counting (a fixed count makes the flop
// figure independent of the state): 0 = iterate to convergence
thread_local int g_fixed_newton = 0;

// ---------------------------------------------------------------- thermo
const double* nasa(int k, double T) { return T <= T_MID[k] ? NASA_LOW[k] : NASA_HIGH[k]; }
template <class F>
F cp_R(int k, F T) {
    const double* a = nasa(k, val(T));
    return a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])));
}
template <class F>
F h_RT(int k, F T) {
    const double* a = nasa(k, val(T));
    return a[0] + T * (a[1] / 2 + T * (a[2] / 3 + T * (a[3] / 4 + T * a[4] / 5))) + a[5] / T;
}
template <class F>
F s_R(int k, F T) {
    const double* a = nasa(k, val(T));
    return a[0] * xlog(T) + T * (a[1] + T * (a[2] / 2 + T * (a[3] / 3 + T * a[4] / 4))) + a[6];
}
// specific internal energy and cv of a composition (mass fractions, not normalised)
template <class F>
F mix_e(const F* Y, F T) {
    F s = 0;
    for (int k = 0; k < NS; ++k) s += Y[k] / MW[k] * (h_RT(k, T) - 1.0);
    return R * T * s;
}
template <class F>
F mix_cv(const F* Y, F T) {
    F s = 0;
    for (int k = 0; k < NS; ++k) s += Y[k] / MW[k] * (cp_R(k, T) - 1.0);
    return R * s;
}
template <class F>
F inv_mmw(const F* Y) {
    F s = 0;
    for (int k = 0; k < NS; ++k) s += Y[k] / MW[k];
    return s;
}

// Newton iteration T <- T + (e_target - e(T))/cv(T), stopped once the applied
// correction is below 1e-10*T: Newton converges quadratically, so T is then at
// rounding level.  Steps are clipped to +-1000 K and T is kept positive.  The
// NASA7 ranges meet at T_mid = 1000 K with a small jump in e(T); an energy inside
// that jump has no root, and Newton then flips across T_mid with sub-kelvin steps:
// two consecutive such flips return T_mid itself.  Returns false if it does not
// converge in 60 iterations or leaves the finite positive range.
template <class F>
bool solve_T(const F* Y, F e, F& T) {
    if (!(T > 0) || !xfinite(T)) T = 1000.0;
    int flips = 0;
    const int fixed = g_fixed_newton;
    for (int it = 0; it < (fixed > 0 ? fixed : 60); ++it) {
        F dT = (e - mix_e(Y, T)) / mix_cv(Y, T);
        if (!xfinite(dT)) return false;
        dT = xmin(F(1000.0), xmax(F(-1000.0), dT));
        F Tn = T + dT;
        if (Tn <= 0) Tn = 0.5 * T;
        const bool converged = xfabs(Tn - T) <= 1e-10 * Tn;
        if (fixed > 0) { T = Tn; continue; }
        if (converged) { T = Tn; return true; }
        flips = ((T <= 1000.0) != (Tn <= 1000.0) && xfabs(Tn - T) < 0.5) ? flips + 1 : 0;
        if (flips >= 2) { T = 1000.0; return true; }
        T = Tn;
    }
    return fixed > 0;
}

// The flux-path functions below are templates on the scalar type as well (double for
// the oracle, Fl for the flux path's flop count, or_flux_flops).
template <class F>
F density(const F* q) {
    F r = 0;
    for (int k = 0; k < NS; ++k) r += q[k];
    return r;
}
template <class F>
F internal_energy(const F* q) {
    const F rho = density(q);
    const F u = q[MX()] / rho, v = q[MY()] / rho;
    return q[EN()] / rho - 0.5 * (u * u + v * v);
}

template <class F>
struct PropsT { F p, a, T; };
using Props = PropsT<double>;

// physics.cpp:4-15.  T_guess is the starting temperature of the UV Newton solve.
template <class F>
bool properties(const F* q, PropsT<F>& s, F T_guess = F(1000.0)) {
    for (int n = 0; n < NV(); ++n) if (!xfinite(q[n])) return false;
    const F rho = density(q);
    if (!(rho > 0)) return false;
    for (int k = 0; k < NS; ++k) if (q[k] < 0) return false;
    F Y[NS_MAX];
    for (int k = 0; k < NS; ++k) Y[k] = q[k] / rho;
    F T = T_guess;
    if (!solve_T(Y, internal_energy(q), T)) return false;
    const F z = inv_mmw(Y);
    const F cv = mix_cv(Y, T), cp = cv + R * z;
    s.T = T;
    s.p = rho * R * T * z;
    s.a = xsqrt(cp / cv * R * T * z);
    return s.T > 0 && s.p > 0 && s.a > 0 && xfinite(s.a);
}

// physics.cpp:17-38
template <class F>
void hllc(const F* l, const F* r, int n, PropsT<F> pl, PropsT<F> pr, F* out) {
    const int E = EN();
    const F rl = density(l), rr = density(r), ul = l[n] / rl, ur = r[n] / rr;
    const F sl = xmin(ul - pl.a, ur - pr.a), sr = xmax(ul + pl.a, ur + pr.a);
    auto flux = [&](const F* q, F v, F p, F* f) {
        for (int m = 0; m < NV(); ++m) f[m] = v * q[m];
        f[n] += p;
        f[E] += p * v;
    };
    if (sl >= 0) { flux(l, ul, pl.p, out); return; }
    if (sr <= 0) { flux(r, ur, pr.p, out); return; }
    const F dl = rl * (sl - ul), dr = rr * (sr - ur);
    const F sm = (pr.p - pl.p + dl * ul - dr * ur) / (dl - dr);
    const bool left = sm >= 0;
    const F* q = left ? l : r;
    const F v = left ? ul : ur, s = left ? sl : sr, p = left ? pl.p : pr.p;
    F star[MAXV], f[MAXV];
    const F scale = (s - v) / (s - sm);
    for (int m = 0; m < NV(); ++m) star[m] = q[m] * scale;
    const F rs = density(star);
    star[n] = rs * sm;
    star[E] += rs * (sm - v) * (sm + p / (density(q) * (s - v)));
    flux(q, v, p, f);
    for (int m = 0; m < NV(); ++m) out[m] = f[m] + s * (star[m] - q[m]);
}

// physics.cpp:40-44
template <class F>
F minmod1(F x, F y) {
    return x * y > 0 ? xcopysign(xmin(xfabs(x), xfabs(y)), x) : F(0.);
}
// MUSCL face states of the stage (BlockAMR.cpp:218-219) from the 4-cell stencil
template <class F>
void muscl_face(const F* qa, const F* qb, const F* qc, const F* qd, F* L, F* Rr) {
    for (int n = 0; n < NV(); ++n) {
        L[n] = qb[n] + 0.5 * minmod1(qb[n] - qa[n], qc[n] - qb[n]);
        Rr[n] = qc[n] - 0.5 * minmod1(qc[n] - qb[n], qd[n] - qc[n]);
    }
}
// flux divergence update of one cell (BlockAMR.cpp:234-243)
template <class F>
void cell_update(const F* q, const F* fl, const F* fr, const F* fb, const F* ft, F cx, F cy, F* out) {
    for (int n = 0; n < NV(); ++n) out[n] = q[n] - cx * (fr[n] - fl[n]) - cy * (ft[n] - fb[n]);
}

// ---------------------------------------------------------------- kinetics
template <class F>
struct RatesT { F kf[NR], kr[NR], qf[NR], qr[NR]; };
using Rates = RatesT<double>;

// Troe falloff factor F(T, Pr) and, optionally, d ln F / d ln Pr and d ln F / dT.
template <class F>
F troe_F(const Reaction& rx, F T, F Pr, F* dlnF_dlnPr = nullptr, F* dlnF_dT = nullptr) {
    const F e3 = xexp(-T / rx.troeT3), e1 = xexp(-T / rx.troeT1);
    F Fcent = (1 - rx.troeA) * e3 + rx.troeA * e1;
    F dFcent = -(1 - rx.troeA) / rx.troeT3 * e3 - rx.troeA / rx.troeT1 * e1;
    if (rx.hasT2) {
        const F e2 = xexp(-rx.troeT2 / T);
        Fcent += e2;
        dFcent += rx.troeT2 / (T * T) * e2;
    }
    const bool fc_clamped = !(Fcent > 1e-300), pr_clamped = !(Pr > 1e-300);
    const F lFc = xlog10(xmax(Fcent, F(1e-300)));
    const F lPr = xlog10(xmax(Pr, F(1e-300)));
    const F c = -0.4 - 0.67 * lFc, nn = 0.75 - 1.27 * lFc;
    const F x = lPr + c, den = nn - 0.14 * x;
    const F f1 = x / den;
    const F g = 1 / (1 + f1 * f1);
    const F lF = lFc * g;
    if (dlnF_dlnPr) {
        // d log10 F / d log10 Pr = lFc * (-2 f1 g^2) * df1/dx,  df1/dx = nn/den^2
        *dlnF_dlnPr = pr_clamped ? F(0.0) : lFc * (-2 * f1 * g * g) * (nn / (den * den));
    }
    if (dlnF_dT) {
        // through Fcent: dx/dlFc = -0.67, dnn/dlFc = -1.27
        const F df1 = (-0.67 * den - x * (-1.27 + 0.14 * 0.67)) / (den * den);
        const F dlF_dlFc = g + lFc * (-2 * f1 * g * g) * df1;
        const F dlFc_dT = fc_clamped ? F(0.0) : dFcent / (Fcent * std::log(10.0));
        *dlnF_dT = dlF_dlFc * dlFc_dT * std::log(10.0);
    }
    return xpow(F(10.0), lF);
}

// Rate multipliers (sensitivity parameters p_r = ln multiplier_r): reaction r's
// forward rate constant, and with it the reverse one, is scaled by multiplier_r;
// for falloff reactions both limits are scaled, so Pr is unchanged.  Per thread,
// so finite-difference runs of different cells can perturb different reactions.
// A process-wide set (or_set_rate_mult) applies where no per-thread set is active.
thread_local const double* tl_rate_mult = nullptr;
double g_rate_mult[NR];
bool g_rate_mult_on = false;
inline double rate_mult(int r) { return tl_rate_mult ? tl_rate_mult[r] : (g_rate_mult_on ? g_rate_mult[r] : 1.0); }

// Rates of progress (kmol/m^3/s) at T and molar concentrations C.
template <class F>
void progress(F T, const F* C, RatesT<F>& out) {
    F g[NS_MAX];
    for (int k = 0; k < NS; ++k) g[k] = h_RT(k, T) - s_R(k, T);
    const F lnT = xlog(T), c0 = xlog(ONE_ATM / (R * T));
    for (int r = 0; r < NR; ++r) {
        const Reaction& rx = RXN[r];
        F M = 0;
        if (rx.type != RXN_ELEMENTARY) for (int k = 0; k < NS; ++k) M += rx.eff[k] * C[k];
        F k = rx.A * rate_mult(r) * xexp(rx.b * lnT - rx.EaR / T);
        if (rx.type == RXN_FALLOFF) {
            const F k0 = rx.A0 * rate_mult(r) * xexp(rx.b0 * lnT - rx.Ea0R / T);
            const F Pr = k0 * M / k;
            k = k * (Pr / (1 + Pr)) * troe_F(rx, T, Pr);
        } else if (rx.type == RXN_THREE_BODY) {
            k *= M;
        }
        F dG = 0;
        int dn = 0;
        for (int i = 0; i < rx.nprod; ++i) { dG += g[rx.prod[i]]; ++dn; }
        for (int i = 0; i < rx.nreac; ++i) { dG -= g[rx.reac[i]]; --dn; }
        const F Kc = xexp(-dG + dn * c0);
        F qf = k, qr = k / Kc;
        for (int i = 0; i < rx.nreac; ++i) qf *= C[rx.reac[i]];
        for (int i = 0; i < rx.nprod; ++i) qr *= C[rx.prod[i]];
        out.kf[r] = k;
        out.kr[r] = k / Kc;
        out.qf[r] = qf;
        out.qr[r] = qr;
    }
}

template <class F>
void net_production(F T, const F* C, F* wdot) {
    RatesT<F> rt;
    progress(T, C, rt);
    for (int k = 0; k < NS; ++k) wdot[k] = 0;
    for (int r = 0; r < NR; ++r) {
        const F q = rt.qf[r] - rt.qr[r];
        for (int i = 0; i < RXN[r].nreac; ++i) wdot[RXN[r].reac[i]] -= q;
        for (int i = 0; i < RXN[r].nprod; ++i) wdot[RXN[r].prod[i]] += q;
    }
}

// ---------------------------------------------------------------- chemistry ODE
// chemistry.cpp:36-53: unknowns y = Y_0..Y_{NS-2}; the last species closes the
// mass; rho and e are fixed; T is re-solved from e at every evaluation.
template <class F>
struct ChemCellT {
    F rho, e, T;            // T is the warm start of the next UV solve
    long nrhs = 0, njac = 0;
};
using ChemCell = ChemCellT<double>;

template <class F>
bool chem_rhs(ChemCellT<F>& c, const F* y, F* dy) {
    const int n = NS - 1;
    F Y[NS_MAX];
    F s = 0;
    for (int k = 0; k < n; ++k) { Y[k] = y[k]; s += y[k]; }
    Y[n] = 1 - s;
    F T = c.T;
    if (!solve_T(Y, c.e, T)) return false;
    c.T = T;
    F C[NS_MAX], w[NS_MAX];
    for (int k = 0; k < NS; ++k) C[k] = c.rho * Y[k] / MW[k];
    net_production(T, C, w);
    for (int k = 0; k < n; ++k) {
        dy[k] = w[k] * MW[k] / c.rho;
        if (!xfinite(dy[k])) return false;
    }
    ++c.nrhs;
    return true;
}

// Jacobian d(dy)/dy by one-sided differences, column j perturbed by
// sqrt(eps)*max(|y_j|, 1e-10) (test helper; the integrator uses analytic()).
bool chem_jac_fd(ChemCell& c, const double* y, const double* f0, double* J) {
    const int n = NS - 1;
    double yp[NS_MAX], fp[NS_MAX];
    for (int j = 0; j < n; ++j) {
        std::copy(y, y + n, yp);
        const double d = std::sqrt(std::numeric_limits<double>::epsilon()) * std::max(std::fabs(y[j]), 1e-10);
        yp[j] += d;
        const double T0 = c.T;
        if (!chem_rhs(c, yp, fp)) return false;
        c.T = T0;
        for (int i = 0; i < n; ++i) J[i * n + j] = (fp[i] - f0[i]) / d;
    }
    return true;
}

// Analytic Jacobian of the reference ODE.  With C_k = rho Y_k / W_k,
//   d(dy_i)/dy_j = W_i/rho * sum_r nu_ir [ sum_m dq_r/dC_m dC_m/dy_j + dq_r/dT dT/dy_j ]
// where dC_m/dy_j = rho/W_j [m==j] - rho/W_last [m==last], and at fixed (rho, e)
// dT/dy_j = -(e_j - e_last)/cv with e_k the species specific internal energies.
template <class F>
bool chem_jac(ChemCellT<F>& c, const F* y, F* J) {
    const int n = NS - 1, L = NS - 1;
    F Y[NS_MAX];
    F s = 0;
    for (int k = 0; k < n; ++k) { Y[k] = y[k]; s += y[k]; }
    Y[n] = 1 - s;
    F T = c.T;
    if (!solve_T(Y, c.e, T)) return false;
    c.T = T;
    F C[NS_MAX];
    for (int k = 0; k < NS; ++k) C[k] = c.rho * Y[k] / MW[k];
    // dq_r/dC_m and dq_r/dT
    F dqdC[NR][NS_MAX], dqdT[NR];
    F g[NS_MAX], dgdT[NS_MAX];
    for (int k = 0; k < NS; ++k) {
        g[k] = h_RT(k, T) - s_R(k, T);
        dgdT[k] = -h_RT(k, T) / T;  // d(g/RT)/dT = -h/(R T^2)
    }
    const F lnT = xlog(T), c0 = xlog(ONE_ATM / (R * T));
    for (int r = 0; r < NR; ++r) {
        const Reaction& rx = RXN[r];
        for (int m = 0; m < NS; ++m) dqdC[r][m] = 0;
        F M = 0;
        if (rx.type != RXN_ELEMENTARY) for (int k = 0; k < NS; ++k) M += rx.eff[k] * C[k];
        const F kinf = rx.A * rate_mult(r) * xexp(rx.b * lnT - rx.EaR / T);
        const F dlnkinf = rx.b / T + rx.EaR / (T * T);
        F k = kinf, dkdT = kinf * dlnkinf, dkdM = 0;
        if (rx.type == RXN_THREE_BODY) {
            dkdM = kinf;
            k = kinf * M;
            dkdT = dkdT * M;
        } else if (rx.type == RXN_FALLOFF) {
            const F k0 = rx.A0 * rate_mult(r) * xexp(rx.b0 * lnT - rx.Ea0R / T);
            const F dlnk0 = rx.b0 / T + rx.Ea0R / (T * T);
            const F Pr = k0 * M / kinf;
            F dlnF_dlnPr = 0, dlnF_dT = 0;
            const F Ft = troe_F(rx, T, Pr, &dlnF_dlnPr, &dlnF_dT);
            // ln k = ln kinf + ln Pr - ln(1+Pr) + ln F(T, Pr)
            const F dlnk_dlnPr = 1 - Pr / (1 + Pr) + dlnF_dlnPr;
            k = kinf * Pr / (1 + Pr) * Ft;
            const F dlnPr_dT = dlnk0 - dlnkinf;
            dkdT = k * (dlnkinf + dlnk_dlnPr * dlnPr_dT + dlnF_dT);
            dkdM = M > 0 ? k * dlnk_dlnPr / M : k0 * Ft;  // limit M->0: k ~ k0*M*F
        }
        F dG = 0, dGdT = 0;
        int dn = 0;
        for (int i = 0; i < rx.nprod; ++i) { dG += g[rx.prod[i]]; dGdT += dgdT[rx.prod[i]]; ++dn; }
        for (int i = 0; i < rx.nreac; ++i) { dG -= g[rx.reac[i]]; dGdT -= dgdT[rx.reac[i]]; --dn; }
        const F Kc = xexp(-dG + dn * c0);
        const F dlnKc = -dGdT - dn / T;
        F Pf = 1, Pr_ = 1;
        for (int i = 0; i < rx.nreac; ++i) Pf *= C[rx.reac[i]];
        for (int i = 0; i < rx.nprod; ++i) Pr_ *= C[rx.prod[i]];
        const F kr = k / Kc;
        // mass-action derivatives: d/dC_m of prod C over the list = sum over occurrences
        for (int i = 0; i < rx.nreac; ++i) {
            F p = k;
            for (int j = 0; j < rx.nreac; ++j) if (j != i) p *= C[rx.reac[j]];
            dqdC[r][rx.reac[i]] += p;
        }
        for (int i = 0; i < rx.nprod; ++i) {
            F p = kr;
            for (int j = 0; j < rx.nprod; ++j) if (j != i) p *= C[rx.prod[j]];
            dqdC[r][rx.prod[i]] -= p;
        }
        if (rx.type != RXN_ELEMENTARY) {
            const F net_over_k = Pf - Pr_ / Kc;  // q = k * net_over_k
            for (int m = 0; m < NS; ++m) dqdC[r][m] += dkdM * rx.eff[m] * net_over_k;
        }
        dqdT[r] = dkdT * Pf - (dkdT - k * dlnKc) / Kc * Pr_;
    }
    // dT/dy_j
    F ek[NS_MAX];
    for (int k2 = 0; k2 < NS; ++k2) ek[k2] = R * T / MW[k2] * (h_RT(k2, T) - 1.0);
    const F cv = mix_cv(Y, T);
    F dTdy[NS_MAX];
    for (int j = 0; j < n; ++j) dTdy[j] = -(ek[j] - ek[L]) / cv;
    // dw_i/dy_j
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) J[i * n + j] = 0;
    for (int r = 0; r < NR; ++r) {
        const Reaction& rx = RXN[r];
        F dq[NS_MAX];
        for (int j = 0; j < n; ++j)
            dq[j] = dqdC[r][j] * c.rho / MW[j] - dqdC[r][L] * c.rho / MW[L] + dqdT[r] * dTdy[j];
        for (int i = 0; i < rx.nreac; ++i) {
            const int sp = rx.reac[i];
            if (sp < n) for (int j = 0; j < n; ++j) J[sp * n + j] -= dq[j];
        }
        for (int i = 0; i < rx.nprod; ++i) {
            const int sp = rx.prod[i];
            if (sp < n) for (int j = 0; j < n; ++j) J[sp * n + j] += dq[j];
        }
    }
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) J[i * n + j] *= MW[i] / c.rho;
    ++c.njac;
    return true;
}

// LU with partial pivoting, in place (P A = L U, the diagonal holding 1/U_kk, which the
// solves multiply by); returns false for a singular matrix.
bool lu_factor(double* A, int* piv, int n) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::fabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i) if (std::fabs(A[i * n + k]) > best) { best = std::fabs(A[i * n + k]); p = i; }
        if (!(best > 0) || !std::isfinite(best)) return false;
        piv[k] = p;
        if (p != k) for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
        const double inv = 1.0 / A[k * n + k];
        A[k * n + k] = inv;
        for (int i = k + 1; i < n; ++i) {
            const double l = A[i * n + k] * inv;
            A[i * n + k] = l;
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
        }
    }
    return true;
}
void lu_solve(const double* A, const int* piv, double* b, int n) {
    for (int k = 0; k < n; ++k) if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int i = 1; i < n; ++i) for (int j = 0; j < i; ++j) b[i] -= A[i * n + j] * b[j];
    for (int i = n - 1; i >= 0; --i) {
        for (int j = i + 1; j < n; ++j) b[i] -= A[i * n + j] * b[j];
        b[i] *= A[i * n + i];
    }
}

// Rodas4 tableau (KPP ordering: A and C strictly lower triangular, row-major).
constexpr int RS = 6;
constexpr double RA[15] = {
    1.544, 0.9466785280815826, 0.2557011698983284, 3.314825187068521, 2.896124015972201,
    0.9986419139977817, 1.221224509226641, 6.019134481288629, 12.53708332932087,
    -0.687886036105895, 1.221224509226641, 6.019134481288629, 12.53708332932087,
    -0.687886036105895, 1.0};
constexpr double RC[15] = {
    -5.6688, -2.430093356833875, -0.2063599157091915, -0.1073529058151375, -9.594562251023355,
    -20.47028614809616, 7.496443313967647, -10.24680431464352, -33.99990352819905,
    11.7089089320616, 8.083246795921522, -7.981132988064893, -31.52159432874371,
    16.31930543123136, -6.058818238834054};
constexpr double RM[RS] = {1.221224509226641, 6.019134481288629, 12.53708332932087, -0.687886036105895, 1.0, 1.0};
constexpr double RE[RS] = {0, 0, 0, 0, 0, 1.0};
constexpr double RGAMMA = 0.25;

struct ChemResult { int status; long steps, rejected; };
enum { CHEM_OK = 0, CHEM_FAIL = 1, CHEM_MAXSTEPS = 2 };

double wrms(const double* v, const double* y0, const double* y1, int n, double rtol, double atol) {
    double s = 0;
    for (int i = 0; i < n; ++i) {
        const double sc = atol + rtol * std::max(std::fabs(y0[i]), std::fabs(y1[i]));
        const double r = v[i] / sc;
        s += r * r;
    }
    return std::max(std::sqrt(s / n), 1e-10);
}

// Rodas4 over [0, tend] for an autonomous system Sys with
//   bool rhs(const double* y, double* f), bool jac(const double* y, double* J),
//   void save(), void restore()   (save/restore the warm-start state of rhs).
// Controller as in KPP's Rosenbrock driver: FacMin 0.2, FacMax 6, FacSafe 0.9,
// FacRej 0.1 on a repeated rejection, no step growth right after a rejection;
// the Jacobian and f(y) are formed once per accepted point and reused across
// rejected attempts.  h0 > 0 fixes the first step (no estimate); fixed != 0 turns
// the controller off (every step accepted, used only for order checks).
// max_steps bounds accepted steps like CVodeSetMaxNumSteps.  rec (optional)
// receives the step size of every accepted step.
template <class Sys>
ChemResult rosenbrock(Sys& sys, int n, double* y, double tend, double rtol, double atol, long max_steps,
                      double h0, int fixed, std::vector<double>* rec = nullptr) {
    ChemResult res{CHEM_OK, 0, 0};
    double f0[NS_MAX], J[NS_MAX * NS_MAX], Mx[NS_MAX * NS_MAX], K[RS][NS_MAX], yn[NS_MAX], fy[NS_MAX], err[NS_MAX];
    int piv[NS_MAX];
    if (!sys.rhs(y, f0)) return {CHEM_FAIL, 0, 0};
    double h = h0;
    if (!(h > 0)) {
        // Hairer's starting step (Solving ODEs I, Sec. II.4, order p = 4) applied in
        // time scaled by the interval (t' = t/tend), taking the whole interval when
        // the scaled derivatives vanish (a frozen mixture).
        sys.save();
        const double d0 = wrms(y, y, y, n, rtol, atol), d1 = wrms(f0, y, y, n, rtol, atol) * tend;
        const double hh = d1 < 1e-5 ? 1.0 : std::min(1.0, 0.01 * d0 / d1);
        for (int i = 0; i < n; ++i) yn[i] = y[i] + hh * tend * f0[i];
        double d2 = 0;
        if (sys.rhs(yn, fy)) {
            for (int i = 0; i < n; ++i) err[i] = (fy[i] - f0[i]) / hh;
            d2 = wrms(err, y, y, n, rtol, atol);
        } else {
            d2 = 1e30;
        }
        sys.restore();
        const double mx = std::max(d1, d2);
        const double h1 = mx <= 1e-15 ? 1.0 : std::pow(0.01 / mx, 0.2);
        h = std::min(std::min(100 * hh, h1), 1.0) * tend;
    }
    h = std::min(h, tend);
    double t = 0;
    bool rejectLast = false, rejectMore = false;
    long attempts = 0;
    while (t < tend) {
        if (res.steps >= max_steps) { res.status = CHEM_MAXSTEPS; return res; }
        if (!sys.jac(y, J)) { res.status = CHEM_FAIL; return res; }
        sys.save();
        for (;;) {  // until accepted
            if (++attempts > 4 * max_steps) { res.status = CHEM_MAXSTEPS; return res; }
            bool last = false;
            if (t + 1.01 * h >= tend) { h = tend - t; last = true; }
            const double inv = 1.0 / (h * RGAMMA);
            for (int i = 0; i < n * n; ++i) Mx[i] = -J[i];
            for (int i = 0; i < n; ++i) Mx[i * n + i] += inv;
            bool ok = lu_factor(Mx, piv, n);
            for (int s = 0; ok && s < RS; ++s) {
                const int base = s * (s - 1) / 2;
                if (s == 0) {
                    for (int i = 0; i < n; ++i) fy[i] = f0[i];
                } else {
                    for (int i = 0; i < n; ++i) yn[i] = y[i];
                    for (int j = 0; j < s; ++j) for (int i = 0; i < n; ++i) yn[i] += RA[base + j] * K[j][i];
                    ok = sys.rhs(yn, fy);
                    if (!ok) break;
                }
                for (int i = 0; i < n; ++i) K[s][i] = fy[i];
                for (int j = 0; j < s; ++j) {
                    const double cc = RC[base + j] / h;
                    for (int i = 0; i < n; ++i) K[s][i] += cc * K[j][i];
                }
                lu_solve(Mx, piv, K[s], n);
            }
            double e = std::numeric_limits<double>::infinity();
            if (ok) {
                for (int i = 0; i < n; ++i) { yn[i] = y[i]; err[i] = 0; }
                for (int s = 0; s < RS; ++s) for (int i = 0; i < n; ++i) {
                    yn[i] += RM[s] * K[s][i];
                    err[i] += RE[s] * K[s][i];
                }
                e = wrms(err, y, yn, n, rtol, atol);
                for (int i = 0; i < n; ++i) if (!std::isfinite(yn[i])) e = std::numeric_limits<double>::infinity();
            }
            if (fixed && std::isfinite(e)) e = 0.5;
            if (!std::isfinite(e)) {
                // failed evaluation: CVODE treats a recoverable RHS error by cutting h
                sys.restore();
                ++res.rejected;
                h *= 0.25;
                rejectLast = true;
                if (!(h > 1e-300) || t + h == t) { res.status = CHEM_FAIL; return res; }
                continue;
            }
            double hnew = h * std::min(6.0, std::max(0.2, 0.9 / std::pow(e, 0.25)));
            if (fixed) hnew = h;
            if (e <= 1.0) {
                if (rec) rec->push_back(h);
                t = last ? tend : t + h;
                for (int i = 0; i < n; ++i) y[i] = yn[i];
                if (rejectLast) hnew = std::min(hnew, h);
                rejectLast = rejectMore = false;
                ++res.steps;
                h = hnew;
                break;
            }
            if (rejectMore) hnew = h * 0.1;
            rejectMore = rejectLast;
            rejectLast = true;
            ++res.rejected;
            sys.restore();
            h = hnew;
            if (!(h > 1e-300) || t + h == t) { res.status = CHEM_FAIL; return res; }
        }
        if (t < tend && !sys.rhs(y, f0)) { res.status = CHEM_FAIL; return res; }
    }
    return res;
}

struct ChemSys {
    ChemCell& c;
    double Tsaved = 0;
    bool rhs(const double* y, double* f) { return chem_rhs(c, y, f); }
    bool jac(const double* y, double* J) { return chem_jac(c, y, J); }
    void save() { Tsaved = c.T; }
    void restore() { c.T = Tsaved; }
};

ChemResult rodas4(ChemCell& c, double* y, double dt, double rtol, double atol, long max_steps) {
    ChemSys sys{c};
    return rosenbrock(sys, NS - 1, y, dt, rtol, atol, max_steps, 0.0, 0);
}

// chemistry.cpp:55-76 on one cell (AoS state of NV doubles).  steps_out: attempts
// (accepted + rejected); accepted_out (optional): accepted steps.
int chem_advance(double* u, double dt, double rtol, double atol, long max_steps, long* steps_out,
                 long* accepted_out = nullptr) {
    if (!(dt > 0) || !std::isfinite(dt)) return CHEM_FAIL;
    Props pr;
    if (!properties(u, pr, 1000.0)) return CHEM_FAIL;
    ChemCell c;
    c.rho = density(u);
    c.e = internal_energy(u);
    c.T = pr.T;
    const int n = NS - 1;
    double y[NS_MAX];
    for (int k = 0; k < n; ++k) y[k] = u[k] / c.rho;
    ChemResult r = rodas4(c, y, dt, rtol, atol, max_steps);
    if (steps_out) *steps_out = r.steps + r.rejected;
    if (accepted_out) *accepted_out = r.steps;
    if (r.status != CHEM_OK) return r.status;
    double s = 0;
    for (int k = 0; k < n; ++k) {
        if (!std::isfinite(y[k]) || y[k] < -1e-13) return CHEM_FAIL;
        u[k] = c.rho * std::max(0., y[k]);
    }
    for (int k = 0; k < n; ++k) s += u[k];
    u[n] = c.rho - s;
    if (!properties(u, pr, c.T)) return CHEM_FAIL;
    return CHEM_OK;
}

// ---------------------------------------------------------------- sensitivities
// Rodas4 along a given sequence of accepted step sizes, without error control:
// the frozen-step map whose derivative a discrete adjoint of the accepted steps
// computes (the same stage arithmetic as rosenbrock()'s accepted path).
template <class Sys>
bool rosenbrock_replay(Sys& sys, int n, double* y, const double* hs, long nh) {
    double f0[NS_MAX], J[NS_MAX * NS_MAX], Mx[NS_MAX * NS_MAX], K[RS][NS_MAX], yn[NS_MAX], fy[NS_MAX];
    int piv[NS_MAX];
    for (long st = 0; st < nh; ++st) {
        const double h = hs[st];
        if (!sys.rhs(y, f0) || !sys.jac(y, J)) return false;
        const double inv = 1.0 / (h * RGAMMA);
        for (int i = 0; i < n * n; ++i) Mx[i] = -J[i];
        for (int i = 0; i < n; ++i) Mx[i * n + i] += inv;
        if (!lu_factor(Mx, piv, n)) return false;
        for (int s = 0; s < RS; ++s) {
            const int base = s * (s - 1) / 2;
            if (s == 0) {
                for (int i = 0; i < n; ++i) fy[i] = f0[i];
            } else {
                for (int i = 0; i < n; ++i) yn[i] = y[i];
                for (int j = 0; j < s; ++j) for (int i = 0; i < n; ++i) yn[i] += RA[base + j] * K[j][i];
                if (!sys.rhs(yn, fy)) return false;
            }
            for (int i = 0; i < n; ++i) K[s][i] = fy[i];
            for (int j = 0; j < s; ++j) {
                const double cc = RC[base + j] / h;
                for (int i = 0; i < n; ++i) K[s][i] += cc * K[j][i];
            }
            lu_solve(Mx, piv, K[s], n);
        }
        for (int i = 0; i < n; ++i) {
            double v = y[i];
            for (int s = 0; s < RS; ++s) v += RM[s] * K[s][i];
            if (!std::isfinite(v)) return false;
            y[i] = v;
        }
    }
    return true;
}

// One chemistry call (chemistry.cpp:55-76) on AoS cell u, recording the accepted
// step sizes into rec, or (hs != null) replaying nh given steps.
int chem_substep(double* u, double dt, double rtol, double atol, std::vector<double>* rec, const double* hs,
                 long nh) {
    if (!(dt > 0) || !std::isfinite(dt)) return CHEM_FAIL;
    Props pr;
    if (!properties(u, pr, 1000.0)) return CHEM_FAIL;
    ChemCell c;
    c.rho = density(u);
    c.e = internal_energy(u);
    c.T = pr.T;
    const int n = NS - 1;
    double y[NS_MAX];
    for (int k = 0; k < n; ++k) y[k] = u[k] / c.rho;
    ChemSys sys{c};
    if (hs) {
        if (!rosenbrock_replay(sys, n, y, hs, nh)) return CHEM_FAIL;
    } else {
        const ChemResult r = rosenbrock(sys, n, y, dt, rtol, atol, 5000, 0.0, 0, rec);
        if (r.status != CHEM_OK) return r.status;
    }
    double s = 0;
    for (int k = 0; k < n; ++k) {
        if (!std::isfinite(y[k]) || y[k] < -1e-13) return CHEM_FAIL;
        u[k] = c.rho * std::max(0., y[k]);
    }
    for (int k = 0; k < n; ++k) s += u[k];
    u[n] = c.rho - s;
    if (!properties(u, pr, c.T)) return CHEM_FAIL;
    return CHEM_OK;
}

// Objectives of a 0D constant-(rho, e) run of nsub chemistry calls of dt each,
// from T_n and p_n at the call boundaries t_n = n dt (build-defined: the
// reference has no sensitivity code):
//   ignition delay: the time T first reaches T_0 + dT, interpolated linearly in t
//     between the two boundaries around the crossing (NaN if it never does);
//   peak pressure: max_n p_n;  final temperature: T_nsub.
enum { OBJ_IGNITION = 0, OBJ_PEAK_PRESSURE = 1, OBJ_FINAL_T = 2 };

double objective_value(int obj, const std::vector<double>& T, const std::vector<double>& p, double dt, double dT) {
    if (obj == OBJ_FINAL_T) return T.back();
    if (obj == OBJ_PEAK_PRESSURE) return *std::max_element(p.begin(), p.end());
    const double Ts = T[0] + dT;
    for (size_t n = 0; n + 1 < T.size(); ++n)
        if (T[n + 1] >= Ts) return n * dt + dt * (Ts - T[n]) / (T[n + 1] - T[n]);
    return std::numeric_limits<double>::quiet_NaN();
}

// Runs one cell; rec/counts record the accepted steps of every call, or hs/hcounts
// replay them.  Returns a CHEM_* status.
int cell_objective(const double* u0, double dt, int nsub, int obj, double dT, double rtol, double atol,
                   std::vector<double>* rec, std::vector<long>* counts, const double* hs, const long* hcounts,
                   double* J) {
    const int nv = NV();
    double u[MAXV];
    std::copy(u0, u0 + nv, u);
    std::vector<double> T, p;
    Props pr;
    if (!properties(u, pr, 1000.0)) return CHEM_FAIL;
    T.push_back(pr.T);
    p.push_back(pr.p);
    long off = 0;
    for (int n = 0; n < nsub; ++n) {
        const size_t before = rec ? rec->size() : 0;
        const int st = chem_substep(u, dt, rtol, atol, rec, hs ? hs + off : nullptr, hs ? hcounts[n] : 0);
        if (st != CHEM_OK) return st;
        if (rec && counts) counts->push_back((long)(rec->size() - before));
        if (hs) off += hcounts[n];
        if (!properties(u, pr, T.back())) return CHEM_FAIL;
        T.push_back(pr.T);
        p.push_back(pr.p);
    }
    *J = objective_value(obj, T, p, dt, dT);
    return CHEM_OK;
}

// Order check system: r' = r(1-r^2), theta' = 1 written in Cartesian form,
//   y0' = -y1 + y0 (1 - y0^2 - y1^2),  y1' = y0 + y1 (1 - y0^2 - y1^2),
// whose exact solution is r(t) = 1/sqrt(1 + (1/r0^2 - 1) e^{-2t}), theta = theta0 + t.
struct CircleSys {
    bool rhs(const double* y, double* f) {
        const double s = 1 - y[0] * y[0] - y[1] * y[1];
        f[0] = -y[1] + y[0] * s;
        f[1] = y[0] + y[1] * s;
        return true;
    }
    bool jac(const double* y, double* J) {
        const double s = 1 - y[0] * y[0] - y[1] * y[1];
        J[0] = s - 2 * y[0] * y[0];
        J[1] = -1 - 2 * y[0] * y[1];
        J[2] = 1 - 2 * y[0] * y[1];
        J[3] = s - 2 * y[1] * y[1];
        return true;
    }
    void save() {}
    void restore() {}
};

// ---------------------------------------------------------------- grid
}  // namespace

extern "C" {

// Boundary kinds, as the reference's JSON strings (BlockAMR.cpp:38-59).
enum { OR_BC_REFLECTING = 0, OR_BC_TRANSMISSIVE = 1, OR_BC_INFLOW = 2, OR_BC_WEDGE = 3 };

struct or_grid {
    int nx, ny;            // cells of the (single-box) level domain
    double dx, dy, xlo, ylo;
    int periodic[2];
    int bc_lo[2], bc_hi[2];
    double inlet[MAXV];    // the fixed inflow state ("fresh", BlockAMR.cpp:67,132-136)
    double wedge_start;
};

// Rate multipliers for every later call (null: none).
void or_set_rate_mult(const double* m) {
    g_rate_mult_on = m != nullptr;
    if (m) for (int r = 0; r < NR; ++r) g_rate_mult[r] = m[r];
}

int or_set_species(int ns) {
    if (ns != 9 && ns != 10) return -1;
    NS = ns;
    return 0;
}
int or_nspecies() { return NS; }
double or_molecular_weight(int k) { return MW[k]; }

void or_species_thermo(double T, double* cp, double* h, double* s) {
    for (int k = 0; k < NS; ++k) {
        cp[k] = cp_R(k, T);
        h[k] = h_RT(k, T);
        s[k] = s_R(k, T);
    }
}
double or_mix_e(const double* Y, double T) { return mix_e(Y, T); }
double or_mix_cv(const double* Y, double T) { return mix_cv(Y, T); }

// Batched properties over count AoS states; status[i] = 1 if inadmissible.
void or_properties(const double* q, int64_t count, double* p, double* a, double* T, int* status) {
    for (int64_t i = 0; i < count; ++i) {
        Props s{0, 0, 0};
        const bool ok = properties(q + i * NV(), s);
        status[i] = ok ? 0 : 1;
        p[i] = s.p;
        a[i] = s.a;
        T[i] = s.T;
    }
}

void or_hllc(const double* l, const double* r, int n, const double* pl, const double* pr, double* out) {
    hllc(l, r, n, Props{pl[0], pl[1], pl[2]}, Props{pr[0], pr[1], pr[2]}, out);
}

void or_minmod(const double* a, const double* b, double* out, int count) {
    for (int i = 0; i < count; ++i) out[i] = minmod1(a[i], b[i]);
}

void or_net_production(double T, const double* C, double* wdot) { net_production(T, C, wdot); }
void or_progress(double T, const double* C, double* kf, double* kr, double* qf, double* qr) {
    Rates rt;
    progress(T, C, rt);
    for (int r = 0; r < NR; ++r) { kf[r] = rt.kf[r]; kr[r] = rt.kr[r]; qf[r] = rt.qf[r]; qr[r] = rt.qr[r]; }
}

int or_chem_rhs(double rho, double e, const double* y, double* T, double* dy) {
    ChemCell c;
    c.rho = rho; c.e = e; c.T = *T;
    const bool ok = chem_rhs(c, y, dy);
    *T = c.T;
    return ok ? 0 : 1;
}
int or_chem_jac(double rho, double e, const double* y, double* T, double* J, int fd) {
    ChemCell c;
    c.rho = rho; c.e = e; c.T = *T;
    bool ok;
    if (fd) {
        double f0[NS_MAX];
        ok = chem_rhs(c, y, f0) && chem_jac_fd(c, y, f0, J);
    } else {
        ok = chem_jac(c, y, J);
    }
    *T = c.T;
    return ok ? 0 : 1;
}

// One cell through chemistry.cpp:55-76; returns 0 ok, 1 failure, 2 step limit.
int or_chem_advance(double* u, double dt, double rtol, double atol, long max_steps, long* steps) {
    return chem_advance(u, dt, rtol, atol, max_steps, steps);
}

// Fixed-step Rodas4 on the order-check system (y has 2 entries).
void or_rodas4_circle(double* y, double tend, int nsteps) {
    CircleSys s;
    rosenbrock(s, 2, y, tend, 1e-6, 1e-6, 1L << 40, tend / nsteps, 1);
}

// chemistry_batch.cpp:21-50.  Advances count AoS cells (one dt, or dt_cell[i]
// when dt_cell is non-null) with OpenMP schedule(dynamic,8); all-or-nothing.
// Returns -1 on success, else the lowest failing index (the field is unchanged).
int64_t or_chem_batch(double* U, int64_t count, double dt, const double* dt_cell, double rtol,
                      double atol, int threads, long* steps_out) {
    const int nv = NV();
    std::vector<double> trial(U, U + count * nv);
    std::vector<int> fail(count, 0);
    std::vector<long> steps(count, 0);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
    for (int64_t k = 0; k < count; ++k) {
        long st = 0;
        fail[k] = chem_advance(&trial[k * nv], dt_cell ? dt_cell[k] : dt, rtol, atol, 5000, &st);
        steps[k] = st;
    }
    if (steps_out) for (int64_t k = 0; k < count; ++k) steps_out[k] = steps[k];
    for (int64_t k = 0; k < count; ++k) if (fail[k]) return k;
    std::copy(trial.begin(), trial.end(), U);
    return -1;
}

// Accepted and rejected Rodas4 steps per cell of a batch (U is not changed); cells
// that fail report -1 accepted steps.
void or_chem_batch_stats(const double* U, int64_t count, double dt, const double* dt_cell, double rtol, double atol,
                         int threads, long* accepted, long* rejected) {
    const int nv = NV();
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
    for (int64_t k = 0; k < count; ++k) {
        double u[MAXV];
        std::copy(U + k * nv, U + (k + 1) * nv, u);
        long att = 0, acc = 0;
        const int st = chem_advance(u, dt_cell ? dt_cell[k] : dt, rtol, atol, 5000, &att, &acc);
        accepted[k] = st == CHEM_OK ? acc : -1;
        rejected[k] = att - acc;
    }
}

// FP64 work of one right-hand side and one analytic Jacobian of the chemistry ODE at
// (rho, e, y) with the UV inversion taking exactly `newton` iterations from T: out[0]
// flops and out[1] transcendental calls of the RHS, out[2] and out[3] of the Jacobian.
void or_chem_flops(double rho, double e, const double* y, double T, int newton, double* out) {
    const int n = NS - 1;
    ChemCellT<Fl> c;
    c.rho = rho;
    c.e = e;
    Fl yy[NS_MAX], f[NS_MAX], J[NS_MAX * NS_MAX];
    for (int k = 0; k < n; ++k) yy[k] = y[k];
    g_fixed_newton = newton;
    for (int which = 0; which < 2; ++which) {
        c.T = T;
        g_fl_ops = g_fl_trans = 0;
        if (which == 0) chem_rhs(c, yy, f);
        else chem_jac(c, yy, J);
        out[2 * which] = (double)g_fl_ops;
        out[2 * which + 1] = (double)g_fl_trans;
    }
    g_fixed_newton = 0;
}

// FP64 work of the flux path as this restatement does it (flops: add, sub, mul, div,
// sqrt), with every UV inversion taking exactly `newton` iterations from the stage's
// starting guess of 1000 K.  From a 4-cell stencil along direction dir (AoS, NV each):
// out[0] the flops of one face (MUSCL on both sides, the EOS of the two face states,
// HLLC), out[1] of one cell's flux-divergence update and validation (one EOS), out[2]
// of one cell's Heun combine, out[3] the transcendental calls of a face.
void or_flux_flops(const double* stencil, int dir, int newton, double* out) {
    const int nv = NV();
    Fl q[4][MAXV], L[MAXV], Rr[MAXV], f[MAXV], o[MAXV];
    for (int c = 0; c < 4; ++c)
        for (int n = 0; n < nv; ++n) q[c][n] = stencil[c * nv + n];
    g_fixed_newton = newton;
    g_fl_ops = g_fl_trans = 0;
    muscl_face(q[0], q[1], q[2], q[3], L, Rr);
    PropsT<Fl> pl, pr, pc;
    properties(L, pl);
    properties(Rr, pr);
    hllc(L, Rr, dir == 0 ? MX() : MY(), pl, pr, f);
    out[0] = (double)g_fl_ops;
    out[3] = (double)g_fl_trans;
    g_fl_ops = 0;
    cell_update(q[1], f, f, f, f, Fl(0.1), Fl(0.1), o);
    properties(o, pc);
    out[1] = (double)g_fl_ops;
    g_fl_ops = 0;
    for (int n = 0; n < nv; ++n) o[n] = 0.5 * q[1][n] + 0.5 * o[n];
    out[2] = (double)g_fl_ops;
    g_fixed_newton = 0;
}

// Objective (OBJ_*) of count AoS cells over nsub adaptive chemistry calls of dt
// each; mult: NR rate multipliers (null = 1).  Returns -1, or the lowest failing cell.
int64_t or_chem_objective(const double* U0, int64_t count, double dt, int nsub, int obj, double dT, double rtol,
                          double atol, const double* mult, int threads, double* J) {
    const int nv = NV();
    std::vector<int> fail(count, 0);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t k = 0; k < count; ++k) {
        tl_rate_mult = mult;
        fail[k] = cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, nullptr, nullptr, nullptr, nullptr, &J[k]);
        tl_rate_mult = nullptr;
    }
    for (int64_t k = 0; k < count; ++k) if (fail[k]) return k;
    return -1;
}

// Central differences of the objective in p_r = ln multiplier_r, r = 0..NR-1,
// step fd_h, into grad[k*NR + r]; J[k] is the unperturbed objective.  frozen != 0
// replays each cell's accepted step sequence of the unperturbed run (the map a
// discrete adjoint differentiates); frozen == 0 re-runs the adaptive integrator.
int64_t or_chem_sens_fd(const double* U0, int64_t count, double dt, int nsub, int obj, double dT, double rtol,
                        double atol, double fd_h, int frozen, int threads, double* J, double* grad) {
    const int nv = NV();
    std::vector<int> fail(count, 0);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t k = 0; k < count; ++k) {
        double mult[NR];
        for (int r = 0; r < NR; ++r) mult[r] = 1.0;
        tl_rate_mult = mult;
        std::vector<double> rec;
        std::vector<long> counts;
        int st = cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, &rec, &counts, nullptr, nullptr, &J[k]);
        for (int r = 0; st == CHEM_OK && r < NR; ++r) {
            double Jp = 0, Jm = 0;
            mult[r] = std::exp(fd_h);
            st = frozen ? cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, nullptr, nullptr, rec.data(),
                                         counts.data(), &Jp)
                        : cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, nullptr, nullptr, nullptr,
                                         nullptr, &Jp);
            mult[r] = std::exp(-fd_h);
            if (st == CHEM_OK)
                st = frozen ? cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, nullptr, nullptr, rec.data(),
                                             counts.data(), &Jm)
                            : cell_objective(&U0[k * nv], dt, nsub, obj, dT, rtol, atol, nullptr, nullptr, nullptr,
                                             nullptr, &Jm);
            mult[r] = 1.0;
            grad[k * NR + r] = (Jp - Jm) / (2 * fd_h);
        }
        tl_rate_mult = nullptr;
        fail[k] = st;
    }
    for (int64_t k = 0; k < count; ++k) if (fail[k]) return k;
    return -1;
}

// ---------------------------------------------------------------- ghost fill
// Ghosted AoS level array, 2 ghost layers: index ((j+2)*(nx+4)+(i+2))*NV+n.
static inline double& at(const or_grid* g, double* U, int i, int j, int n) {
    return U[((int64_t)(j + 2) * (g->nx + 4) + (i + 2)) * NV() + n];
}
static inline double atc(const or_grid* g, const double* U, int i, int j, int n) {
    return U[((int64_t)(j + 2) * (g->nx + 4) + (i + 2)) * NV() + n];
}

// BlockAMR.cpp:48-59: BC per side/direction/component in AMReX terms.
enum { BCT_INT = 0, BCT_FOEXTRAP = 1, BCT_EVEN = 2, BCT_ODD = 3, BCT_EXT = 4 };
static int bctype(const or_grid* g, int d, int hi, int n) {
    if (g->periodic[d]) return BCT_INT;
    const int kind = hi ? g->bc_hi[d] : g->bc_lo[d];
    if (kind == OR_BC_INFLOW || kind == OR_BC_WEDGE) return BCT_EXT;
    if (kind == OR_BC_REFLECTING) return n == (d == 0 ? MX() : MY()) ? BCT_ODD : BCT_EVEN;
    return BCT_FOEXTRAP;
}

// AMReX filcc_cell: x-direction rule, then the y-direction rule (the later one
// wins in corners); ext_dir and int_dir leave the cell alone.
static void filcc(const or_grid* g, double* U, int i, int j) {
    const int ihi = g->nx - 1, jhi = g->ny - 1;
    for (int n = 0; n < NV(); ++n) {
        if (i < 0 || i > ihi) {
            const int t = bctype(g, 0, i > ihi, n);
            const int src = i < 0 ? -i - 1 : 2 * ihi - i + 1;
            if (t == BCT_FOEXTRAP) at(g, U, i, j, n) = at(g, U, i < 0 ? 0 : ihi, j, n);
            else if (t == BCT_EVEN) at(g, U, i, j, n) = at(g, U, src, j, n);
            else if (t == BCT_ODD) at(g, U, i, j, n) = -at(g, U, src, j, n);
        }
        if (j < 0 || j > jhi) {
            const int t = bctype(g, 1, j > jhi, n);
            const int src = j < 0 ? -j - 1 : 2 * jhi - j + 1;
            if (t == BCT_FOEXTRAP) at(g, U, i, j, n) = at(g, U, i, j < 0 ? 0 : jhi, n);
            else if (t == BCT_EVEN) at(g, U, i, j, n) = at(g, U, i, src, n);
            else if (t == BCT_ODD) at(g, U, i, j, n) = -at(g, U, i, src, n);
        }
    }
}

// FlowBoundary.hpp:12-36
static void flow_boundary(const or_grid* g, double* U, int i, int j) {
    const bool mixedBottom = !g->periodic[1] && g->bc_lo[1] == OR_BC_WEDGE;
    const bool below = j < 0;
    const int iv[2] = {i, j}, hiE[2] = {g->nx - 1, g->ny - 1};
    for (int n = 0; n < NV(); ++n) {
        bool fixed = false;
        for (int d = 0; d < 2; ++d) {
            const bool mixed = mixedBottom && d == 1 && below;
            fixed = fixed || (iv[d] < 0 && bctype(g, d, 0, n) == BCT_EXT && !mixed);
            fixed = fixed || (iv[d] > hiE[d] && bctype(g, d, 1, n) == BCT_EXT);
        }
        if (fixed) { at(g, U, i, j, n) = g->inlet[n]; continue; }
        if (mixedBottom && below) {
            const double x = g->xlo + (i + 0.5) * g->dx;
            const bool wall = x >= g->wedge_start;
            const int jj = wall ? -j - 1 : 0;
            const int ii = std::min(std::max(i, 0), g->nx - 1);
            double v = at(g, U, ii, jj, n);
            if (wall && n == MY()) v = -v;
            at(g, U, i, j, n) = v;
        }
    }
}

// FillPatchSingleLevel on a one-box level: periodic images first (FillBoundary),
// then physical BCs on faces (outside the periodically grown domain in one
// direction), then on corners (outside in both); each cell gets filcc then the
// FlowBoundary functor (AMReX GpuBndryFuncFab order).
void or_fill_ghosts(const or_grid* g, double* U) {
    const int nx = g->nx, ny = g->ny;
    auto in_g = [&](int i, int d) { return g->periodic[d] || (i >= 0 && i < (d == 0 ? nx : ny)); };
    for (int j = -2; j < ny + 2; ++j) for (int i = -2; i < nx + 2; ++i) {
        const bool inside = i >= 0 && i < nx && j >= 0 && j < ny;
        if (inside || !in_g(i, 0) || !in_g(j, 1)) continue;
        const int si = ((i % nx) + nx) % nx, sj = ((j % ny) + ny) % ny;
        for (int n = 0; n < NV(); ++n) at(g, U, i, j, n) = at(g, U, si, sj, n);
    }
    for (int pass = 1; pass <= 2; ++pass)
        for (int j = -2; j < ny + 2; ++j) for (int i = -2; i < nx + 2; ++i) {
            const int out = !in_g(i, 0) + !in_g(j, 1);
            if (out != pass) continue;
            filcc(g, U, i, j);
            flow_boundary(g, U, i, j);
        }
}

// ---------------------------------------------------------------- Euler stage
// Threads of the flux, update and validation loops.  1 (default) is the reference's
// threading (BlockAMR::euler runs its MFIter loops on one thread); more threads give
// the same results (every face and cell is computed independently).
static int g_flux_threads = 1;
extern "C" void or_set_flux_threads(int t) { g_flux_threads = t > 0 ? t : omp_get_max_threads(); }

// BlockAMR.cpp:210-243 on a one-box level.  Ug: ghosted input (ghosts filled).
// Uout: ghosted output (interior written).  fx: (ny)x(nx+1) faces, fy: (ny+1)x(nx)
// faces, AoS NV each (may be null).  Returns 0, or 2 when a face's fallback cell
// state is itself inadmissible (properties() throws inside the flux loop of
// BlockAMR.cpp:223, which the reference does not catch before run()'s rollback).
int or_euler_stage(const or_grid* g, const double* Ug, double* Uout, double h, int first_order,
                   double* fx_out, double* fy_out) {
    const int nx = g->nx, ny = g->ny, nv = NV();
    std::vector<double> fx((size_t)ny * (nx + 1) * nv), fy((size_t)(ny + 1) * nx * nv);
    const bool loWall[2] = {!g->periodic[0] && (g->bc_lo[0] == OR_BC_REFLECTING || g->bc_lo[0] == OR_BC_WEDGE),
                            !g->periodic[1] && (g->bc_lo[1] == OR_BC_REFLECTING || g->bc_lo[1] == OR_BC_WEDGE)};
    const bool hiWall[2] = {!g->periodic[0] && g->bc_hi[0] == OR_BC_REFLECTING,
                            !g->periodic[1] && g->bc_hi[1] == OR_BC_REFLECTING};
    const bool mixedBottom = !g->periodic[1] && g->bc_lo[1] == OR_BC_WEDGE;
    const int nt = g_flux_threads;
    int fail = 0;
    for (int d = 0; d < 2; ++d) {
        const int di = d == 0, dj = d == 1;
        const int fnx = nx + di, fny = ny + dj;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1) reduction(| : fail)
        for (int j = 0; j < fny; ++j) for (int i = 0; i < fnx; ++i) {
            double qa[MAXV], qb[MAXV], qc[MAXV], qd[MAXV], L[MAXV], Rr[MAXV], f[MAXV];
            for (int n = 0; n < nv; ++n) {
                qa[n] = atc(g, Ug, i - 2 * di, j - 2 * dj, n);
                qb[n] = atc(g, Ug, i - di, j - dj, n);
                qc[n] = atc(g, Ug, i, j, n);
                qd[n] = atc(g, Ug, i + di, j + dj, n);
            }
            muscl_face(qa, qb, qc, qd, L, Rr);
            if (first_order) for (int n = 0; n < nv; ++n) { L[n] = qb[n]; Rr[n] = qc[n]; }
            Props pl, pr;
            if (!properties(L, pl)) { std::copy(qb, qb + nv, L); }
            if (!properties(Rr, pr)) { std::copy(qc, qc + nv, Rr); }
            // properties() of the fallback states (the reference throws here if even
            // the cell states are inadmissible; ghost-filled valid data never are).
            if (!properties(L, pl) || !properties(Rr, pr)) { fail = 1; continue; }
            hllc(L, Rr, d == 0 ? MX() : MY(), pl, pr, f);
            const int coord = d == 0 ? i : j;
            const double x = g->xlo + (i + 0.5) * g->dx;
            const bool lowWall = loWall[d] && !(d == 1 && mixedBottom && x < g->wedge_start);
            if ((coord == 0 && lowWall) || (coord == (d == 0 ? nx : ny) && hiWall[d])) {
                for (int k = 0; k < NS; ++k) f[k] = 0.;
                f[d == 0 ? MY() : MX()] = 0.;
                f[EN()] = 0.;
            }
            double* dst = d == 0 ? &fx[((size_t)j * (nx + 1) + i) * nv] : &fy[((size_t)j * nx + i) * nv];
            std::copy(f, f + nv, dst);
        }
    }
    if (fail) return 2;
    const double cx = h / g->dx, cy = h / g->dy;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) {
        const double* fl = &fx[((size_t)j * (nx + 1) + i) * nv];
        const double* fr = fl + nv;
        const double* fb = &fy[((size_t)j * nx + i) * nv];
        const double* ft = &fy[((size_t)(j + 1) * nx + i) * nv];
        double q[MAXV], o[MAXV];
        for (int n = 0; n < nv; ++n) q[n] = atc(g, Ug, i, j, n);
        cell_update(q, fl, fr, fb, ft, cx, cy, o);
        for (int n = 0; n < nv; ++n) at(g, Uout, i, j, n) = o[n];
    }
    if (fx_out) std::copy(fx.begin(), fx.end(), fx_out);
    if (fy_out) std::copy(fy.begin(), fy.end(), fy_out);
    return 0;
}

// BlockAMR.cpp:299-334 on a one-level grid (every cell is a leaf, equal volume).
// Returns 0 ok, 1 on materially negative species / insufficient donor.
int or_repair_roundoff(const or_grid* g, double* Ug, long* repairs) {
    const int nx = g->nx, ny = g->ny;
    const double vol = g->dx * g->dy;
    double peak[NS_MAX] = {0}, deficit[NS_MAX] = {0}, dmass[NS_MAX] = {0};
    int di[NS_MAX], dj[NS_MAX];
    bool has[NS_MAX] = {false};
    for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) for (int n = 0; n < NS; ++n) {
        const double v = at(g, Ug, i, j, n);
        peak[n] = std::max(peak[n], v);
        if (v * vol > dmass[n]) { dmass[n] = v * vol; di[n] = i; dj[n] = j; has[n] = true; }
    }
    long count = 0;
    for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) for (int n = 0; n < NS; ++n) {
        const double v = at(g, Ug, i, j, n);
        if (v >= 0) continue;
        if (!std::isfinite(v) || -v > 64 * std::numeric_limits<double>::epsilon() * peak[n]) return 1;
        deficit[n] += -v * vol;
        at(g, Ug, i, j, n) = 0.;
        ++count;
    }
    for (int n = 0; n < NS; ++n) if (deficit[n] > 0) {
        if (!has[n] || !(dmass[n] > deficit[n])) return 1;
        at(g, Ug, di[n], dj[n], n) -= deficit[n] / vol;
    }
    if (repairs) *repairs += count;
    // NaN species never pass the loop above (v >= 0 is false, isfinite false -> 1).
    return 0;
}

// BlockAMR.cpp:286-298: 0 if every cell is admissible, else 1.
int or_validate(const or_grid* g, const double* Ug) {
    const int nt = g_flux_threads;
    int bad = 0;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1) reduction(| : bad)
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) {
        double q[MAXV];
        for (int n = 0; n < NV(); ++n) q[n] = atc(g, Ug, i, j, n);
        Props p;
        if (!properties(q, p)) bad = 1;
    }
    return bad;
}

struct or_stats { long first_order_stages, roundoff_repairs, retries, chem_failures; };

// One composite Euler stage with repair/validate and the first-order redo
// (BlockAMR.cpp:202-265); U (ghosted) is replaced on success.
static int euler(const or_grid* g, double* U, double h, or_stats* st) {
    const size_t sz = (size_t)(g->nx + 4) * (g->ny + 4) * NV();
    std::vector<double> next(U, U + sz);
    or_fill_ghosts(g, U);
    for (int fo = 0; fo < 2; ++fo) {
        std::copy(U, U + sz, next.begin());
        int bad = or_euler_stage(g, U, next.data(), h, fo, nullptr, nullptr);
        if (bad == 2) return 1;
        long reps = 0;
        if (!bad) bad = or_repair_roundoff(g, next.data(), &reps);
        if (!bad) bad = or_validate(g, next.data());
        if (!bad) {
            if (st) { st->roundoff_repairs += reps; if (fo) ++st->first_order_stages; }
            std::copy(next.begin(), next.end(), U);
            return 0;
        }
    }
    return 1;
}

// BlockAMR.cpp:266-270
int or_flow(const or_grid* g, double* U, double h, or_stats* st) {
    const size_t sz = (size_t)(g->nx + 4) * (g->ny + 4) * NV();
    std::vector<double> old(U, U + sz);
    if (euler(g, U, h, st)) return 1;
    if (euler(g, U, h, st)) return 1;
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) for (int n = 0; n < NV(); ++n)
        at(g, U, i, j, n) = 0.5 * at(g, old.data(), i, j, n) + 0.5 * at(g, U, i, j, n);
    return or_validate(g, U);
}

// BlockAMR.cpp:271-285 on a one-level grid.
int or_react(const or_grid* g, double* U, double dt, double rtol, double atol, int threads) {
    const int nv = NV();
    std::vector<double> batch((size_t)g->nx * g->ny * nv);
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) for (int n = 0; n < nv; ++n)
        batch[((size_t)j * g->nx + i) * nv + n] = at(g, U, i, j, n);
    if (or_chem_batch(batch.data(), (int64_t)g->nx * g->ny, dt, nullptr, rtol, atol, threads, nullptr) >= 0) return 1;
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) for (int n = 0; n < nv; ++n)
        at(g, U, i, j, n) = batch[((size_t)j * g->nx + i) * nv + n];
    return or_validate(g, U);
}

// A run of Strang steps with given step sizes whose chemistry calls record their
// accepted step sizes (or_run_record), and its frozen replay (or_run_replay): the map
// a discrete adjoint of the run differentiates.  No dt halving: a failed step fails.
struct or_run_tape {
    int nsteps = 0;
    std::vector<double> dts;
    std::vector<std::vector<std::vector<double>>> h;  // [step][cell] accepted step sizes
};

static int react_frozen(const or_grid* g, double* U, double dt, double rtol, double atol, int threads,
                        std::vector<std::vector<double>>* rec, const std::vector<std::vector<double>>* rep) {
    const int nv = NV();
    const int64_t nc = (int64_t)g->nx * g->ny;
    std::vector<double> batch((size_t)nc * nv);
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) for (int n = 0; n < nv; ++n)
        batch[((size_t)j * g->nx + i) * nv + n] = at(g, U, i, j, n);
    if (rec) rec->assign(nc, {});
    std::vector<int> fail(nc, 0);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
    for (int64_t k = 0; k < nc; ++k) {
        const std::vector<double>* hs = rep ? &(*rep)[k] : nullptr;
        fail[k] = chem_substep(&batch[k * nv], dt, rtol, atol, rec ? &(*rec)[k] : nullptr, hs ? hs->data() : nullptr,
                               hs ? (long)hs->size() : 0);
    }
    for (int64_t k = 0; k < nc; ++k) if (fail[k]) return 1;
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) for (int n = 0; n < nv; ++n)
        at(g, U, i, j, n) = batch[((size_t)j * g->nx + i) * nv + n];
    return or_validate(g, U);
}

void* or_run_record(const or_grid* g, double* U, int nsteps, const double* dts, double rtol, double atol,
                    int threads) {
    auto* t = new or_run_tape();
    t->nsteps = nsteps;
    t->dts.assign(dts, dts + nsteps);
    t->h.resize(nsteps);
    for (int n = 0; n < nsteps; ++n) {
        const double h = dts[n];
        if (or_flow(g, U, 0.5 * h, nullptr) || react_frozen(g, U, h, rtol, atol, threads, &t->h[n], nullptr) ||
            or_flow(g, U, 0.5 * h, nullptr)) {
            delete t;
            return nullptr;
        }
    }
    return t;
}

int or_run_replay(const void* tape, const or_grid* g, double* U, double rtol, double atol, int threads) {
    const auto* t = static_cast<const or_run_tape*>(tape);
    for (int n = 0; n < t->nsteps; ++n) {
        const double h = t->dts[n];
        if (or_flow(g, U, 0.5 * h, nullptr) || react_frozen(g, U, h, rtol, atol, threads, nullptr, &t->h[n]) ||
            or_flow(g, U, 0.5 * h, nullptr))
            return 1;
    }
    return 0;
}

void or_run_free(void* tape) { delete static_cast<or_run_tape*>(tape); }

// BlockAMR.cpp:335-346
double or_cfl_dt(const or_grid* g, const double* U, double cfl) {
    double rate = 0;
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) {
        double q[MAXV];
        for (int n = 0; n < NV(); ++n) q[n] = atc(g, U, i, j, n);
        Props p;
        if (!properties(q, p)) return -1;
        const double rho = density(q);
        rate = std::max(rate, (std::fabs(q[MX()] / rho) + p.a) / g->dx + (std::fabs(q[MY()] / rho) + p.a) / g->dy);
    }
    return cfl / rate;
}

// BlockAMR.cpp:413-418: flow(dt/2); react(dt); flow(dt/2) with rollback and dt
// halving up to 18 attempts.  *dt is updated to the accepted interval.
int or_strang_step(const or_grid* g, double* U, double* dt, int chemistry, double rtol, double atol,
                   int threads, or_stats* st) {
    const size_t sz = (size_t)(g->nx + 4) * (g->ny + 4) * NV();
    std::vector<double> backup(U, U + sz);
    double h = *dt;
    for (int attempt = 0; attempt < 18; ++attempt) {
        bool ok = or_flow(g, U, 0.5 * h, st) == 0;
        if (ok && chemistry) ok = or_react(g, U, h, rtol, atol, threads) == 0;
        if (ok) ok = or_flow(g, U, 0.5 * h, st) == 0;
        if (ok) { *dt = h; return 0; }
        std::copy(backup.begin(), backup.end(), U);
        if (st) ++st->retries;
        h *= 0.5;
    }
    return 1;
}

// ConservativeInterp.cpp:18-51 for one coarse cell: q and its 4 neighbours
// (AoS, order: q, xm, xp, ym, yp) -> 4 children (a + 2b ordering: (0,0),(1,0),(0,1),(1,1)).
// Returns the theta used.
double or_interp_cell(const double* q, const double* xm, const double* xp, const double* ym,
                      const double* yp, double* children) {
    const int nv = NV();
    double sx[MAXV], sy[MAXV];
    for (int n = 0; n < nv; ++n) {
        sx[n] = minmod1(q[n] - xm[n], xp[n] - q[n]);
        sy[n] = minmod1(q[n] - ym[n], yp[n] - q[n]);
    }
    double theta = 1.;
    bool accepted = false;
    for (int attempt = 0; attempt < 48; ++attempt) {
        bool good = true;
        for (int b = 0; b < 2 && good; ++b) for (int a = 0; a < 2 && good; ++a) {
            double child[MAXV];
            for (int n = 0; n < nv; ++n)
                child[n] = q[n] + theta * ((a ? 0.25 : -0.25) * sx[n] + (b ? 0.25 : -0.25) * sy[n]);
            Props p;
            good = properties(child, p);
        }
        if (good) { accepted = true; break; }
        theta *= 0.5;
    }
    if (!accepted) theta = 0.;
    for (int b = 0; b < 2; ++b) for (int a = 0; a < 2; ++a)
        for (int n = 0; n < nv; ++n)
            children[(b * 2 + a) * nv + n] = q[n] + theta * ((a ? 0.25 : -0.25) * sx[n] + (b ? 0.25 : -0.25) * sy[n]);
    return theta;
}


// ---------------------------------------------------------------- block-AMR operations
// BlockAMR::totals (BlockAMR.cpp:347-355) over count AoS cells of one level: sums of
// U (or |U|) times the cell volume in long double, cells whose mask byte is 0 skipped.
void or_totals(const double* U, int64_t count, const unsigned char* mask, double vol, int absolute, double* out) {
    const int nv = NV();
    long double sum[MAXV] = {0};
    for (int64_t c = 0; c < count; ++c) {
        if (mask && !mask[c]) continue;
        for (int n = 0; n < nv; ++n) {
            const double v = U[c * nv + n];
            sum[n] += static_cast<long double>(absolute ? std::fabs(v) : v) * vol;
        }
    }
    for (int n = 0; n < nv; ++n) out[n] = static_cast<double>(sum[n]);
}

// average_down (AMReX amrex_avgdown, ratio 2, equal volumes; BlockAMR.cpp:157-159):
// coarse = 0.25 * (sum of the four children, accumulated jref-major, iref-minor).
// fine: (nyf, nxf, NV) AoS with nxf, nyf even; coarse: (nyf/2, nxf/2, NV).
void or_average_down(const double* fine, int nxf, int nyf, double* coarse) {
    const int nv = NV(), nxc = nxf / 2, nyc = nyf / 2;
    for (int j = 0; j < nyc; ++j) for (int i = 0; i < nxc; ++i) for (int n = 0; n < nv; ++n) {
        double c = 0.0;
        for (int jr = 0; jr < 2; ++jr) for (int ir = 0; ir < 2; ++ir)
            c += fine[((size_t)(2 * j + jr) * nxf + (2 * i + ir)) * nv + n];
        coarse[((size_t)j * nxc + i) * nv + n] = 0.25 * c;
    }
}

// Reflux (FluxRegister CrseInit(-h dy_c) / FineAdd(+h dy_f) / ClearInternalBorders /
// Reflux(scale 1), BlockAMR.cpp:247-255) for one coarse level covering its domain.
//   Uc: (nyc, nxc, NV) updated coarse cells; fxc: (nyc, nxc+1, NV), fyc: (nyc+1, nxc, NV)
//   coarse face fluxes; boxes[b] = {filo, fjlo, fihi, fjhi} fine-level boxes (even
//   lo, odd hi); fxf + xoff[b]: box b's fine x-face fluxes (nyf, nxf+1, NV), fyf +
//   yoff[b]: (nyf+1, nxf, NV).
// Every uncovered coarse cell gathers, in the fixed order x-lo, x-hi, y-lo, y-hi face,
// the register h (sum_fine dA_f F_f - dA_c F_c) of each face whose neighbour cell is
// covered by a fine box, subtracting it on its high face and adding it on its low face
// (divided by the coarse volume).  Periodic directions wrap the neighbour.
void or_reflux(double* Uc, int nxc, int nyc, int periodic_x, int periodic_y, const double* fxc, const double* fyc,
               int nbox, const int* boxes, const double* fxf, const int64_t* xoff, const double* fyf,
               const int64_t* yoff, double h, double dxc, double dyc) {
    const int nv = NV();
    std::vector<int> cover((size_t)nxc * nyc, -1);
    for (int b = 0; b < nbox; ++b)
        for (int cj = boxes[4 * b + 1] / 2; cj <= boxes[4 * b + 3] / 2; ++cj)
            for (int ci = boxes[4 * b] / 2; ci <= boxes[4 * b + 2] / 2; ++ci) cover[(size_t)cj * nxc + ci] = b;
    const double dxf = 0.5 * dxc, dyf = 0.5 * dyc, vol = dxc * dyc;
    for (int j = 0; j < nyc; ++j) for (int i = 0; i < nxc; ++i) {
        if (cover[(size_t)j * nxc + i] >= 0) continue;
        for (int side = 0; side < 4; ++side) {
            const int d = side / 2, hi = side % 2;  // face on the hi side of this cell?
            int ni = i + (d == 0 ? (hi ? 1 : -1) : 0), nj = j + (d == 1 ? (hi ? 1 : -1) : 0);
            if (ni < 0 || ni >= nxc) { if (!periodic_x) continue; ni = (ni + nxc) % nxc; }
            if (nj < 0 || nj >= nyc) { if (!periodic_y) continue; nj = (nj + nyc) % nyc; }
            const int b = cover[(size_t)nj * nxc + ni];
            if (b < 0) continue;
            const int* B = boxes + 4 * b;
            const int nxf = B[2] - B[0] + 1, nyf = B[3] - B[1] + 1;
            for (int n = 0; n < nv; ++n) {
                double Fc, F1, F2, dAc, dAf;
                if (d == 0) {
                    // the face between this cell and (ni, nj), on the fine box's lo x side when
                    // this cell is to its left
                    const int cface = hi ? i + 1 : i;
                    Fc = fxc[((size_t)j * (nxc + 1) + cface) * nv + n];
                    const int fi = hi ? 0 : nxf;  // fine face index in the box
                    const int fj0 = 2 * nj - B[1];
                    F1 = fxf[xoff[b] + ((size_t)fj0 * (nxf + 1) + fi) * nv + n];
                    F2 = fxf[xoff[b] + ((size_t)(fj0 + 1) * (nxf + 1) + fi) * nv + n];
                    dAc = dyc;
                    dAf = dyf;
                } else {
                    const int cface = hi ? j + 1 : j;
                    Fc = fyc[((size_t)cface * nxc + i) * nv + n];
                    const int fj = hi ? 0 : nyf;
                    const int fi0 = 2 * ni - B[0];
                    F1 = fyf[yoff[b] + ((size_t)fj * nxf + fi0) * nv + n];
                    F2 = fyf[yoff[b] + ((size_t)fj * nxf + fi0 + 1) * nv + n];
                    dAc = dxc;
                    dAf = dxf;
                }
                const double reg = -h * dAc * Fc + h * dAf * (F1 + F2);
                Uc[((size_t)j * nxc + i) * nv + n] += (hi ? -reg : reg) / vol;
            }
        }
    }
}

struct or_tag_criteria {
    double pressure_tag, temperature_tag, fuel_rate_tag, density_tag;  // density_tag <= 0: off
    int chemistry, box_only, has_box;
    double box[4], velocity[2];
};

// BlockAMR::ErrorEst (BlockAMR.cpp:170-200) on a ghosted one-level array (ghosts
// filled), plus the relative density-jump criterion (extension, off when
// density_tag <= 0).  tags: (ny, nx) bytes, 1 = tagged.  Returns 1 if a cell on a
// criterion's stencil is inadmissible (properties() throws there), else 0.
int or_tag(const or_grid* g, const double* Ug, double t, const or_tag_criteria* c, unsigned char* tags) {
    const int nv = NV();
    for (int j = 0; j < g->ny; ++j) for (int i = 0; i < g->nx; ++i) {
        const double x = g->xlo + (i + 0.5) * g->dx - c->velocity[0] * t;
        const double y = g->ylo + (j + 0.5) * g->dy - c->velocity[1] * t;
        bool marked = c->has_box && x >= c->box[0] && x <= c->box[1] && y >= c->box[2] && y <= c->box[3];
        if (!c->box_only) {
            double q[MAXV];
            for (int n = 0; n < nv; ++n) q[n] = atc(g, Ug, i, j, n);
            Props p;
            if (!properties(q, p)) return 1;
            for (int d = 0; d < 2; ++d) {
                const int di = d == 0, dj = d == 1;
                double ql[MAXV], qr[MAXV];
                for (int n = 0; n < nv; ++n) {
                    ql[n] = atc(g, Ug, i - di, j - dj, n);
                    qr[n] = atc(g, Ug, i + di, j + dj, n);
                }
                Props pl, pr;
                if (!properties(ql, pl) || !properties(qr, pr)) return 1;
                const double jump = std::max(std::fabs(pl.p - p.p) / std::min(pl.p, p.p),
                                             std::fabs(pr.p - p.p) / std::min(pr.p, p.p));
                const double temp = std::max(std::fabs(pl.T - p.T) / std::min(pl.T, p.T),
                                             std::fabs(pr.T - p.T) / std::min(pr.T, p.T));
                marked = marked || jump > c->pressure_tag || temp > c->temperature_tag;
                if (c->density_tag > 0) {
                    const double r = density(q), rl = density(ql), rr = density(qr);
                    const double rj = std::max(std::fabs(rl - r) / std::min(rl, r), std::fabs(rr - r) / std::min(rr, r));
                    marked = marked || rj > c->density_tag;
                }
            }
            if (c->chemistry) {
                double C[NS_MAX], w[NS_MAX];
                const double rho = density(q);
                for (int k = 0; k < NS; ++k) C[k] = q[k] / MW[k];
                net_production(p.T, C, w);
                marked = marked || -w[0] * MW[0] / rho > c->fuel_rate_tag;
            }
        }
        tags[(size_t)j * g->nx + i] = marked ? 1 : 0;
    }
    return 0;
}
}  // extern "C"
