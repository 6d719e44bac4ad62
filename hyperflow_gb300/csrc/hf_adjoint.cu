// Discrete adjoint of the chemistry calls (a build-defined extension: the
// reference has no sensitivity code).  A 0D cell at constant (rho, e) is advanced
// by ncalls chemistry calls of dt each, every call exactly as Chemistry::advance
// (HyperFlow_V3/src/chemistry.cpp:55-76, here the plain Rodas4 integration of
// hf_kinetics.cuh: adaptive steps, clip y >= -1e-13 to 0, last species closes the
// mass).  An objective J of the temperatures / pressures at the call boundaries
// is differentiated with respect to p_r = ln(multiplier_r) of every reaction
// (the multiplier scales the forward and reverse rate constants; for falloff
// reactions both limits) and to the initial mass fractions.
//
// Differentiated map: the accepted step sequence of the run is frozen (the step
// sizes are constants), so the map is a composition of Rodas4 steps
//     y+ = y + sum_s m_s K_s,   (I/(h g) - J(y)) K_s = f(Y_s) + sum_j c_sj/h K_j,
//     Y_s = y + sum_j a_sj K_j,
// and of the clips at call ends.  Its reverse sweep per step, from ybar = dJ/dy+:
//     Kbar_s = m_s ybar (+ later stages), Rbar_s = M^-T Kbar_s,
//     Ybar_s = J(Y_s)^T Rbar_s, pbar += f_p(Y_s)^T Rbar_s,
//     G = sum_s Rbar_s K_s^T,   ybar += grad_y <J(y), G>,  pbar += grad_p <J(y), G>.
// The last line is the second-derivative term (J depends on y and p).  With
// f_i = W_i/rho sum_r nu_ir q_r, <J, G> = sum_r D_{beta_r} q_r (a directional
// derivative of reaction r's rate of progress along beta_r = G^T diag(W/rho) nu_r),
// so its gradient is one forward-mode (dual number) pass through each reaction's
// analytic gradient, plus the curvature of T(y) from the fixed-energy constraint.
//
// Memory: checkpoints of the state every K calls; in the reverse sweep a segment
// of K calls is recomputed from its checkpoint, storing the state at every call
// boundary and the tape of accepted steps (y, h, T); a segment whose tape exceeds
// its capacity recomputes each call again from the stored boundary states.
#include "hf_kinetics.cuh"

namespace hf {

cudaError_t adjoint_set_rate_scale(const double* scale) { return upload_rate_constants(scale); }

// ---------------------------------------------------------------- dual numbers
struct Dual {
    double v, d;
    __device__ Dual(double v_ = 0.0, double d_ = 0.0) : v(v_), d(d_) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fma(a.d, b.v, a.v * b.d)}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { a = a * b; return a; }
// Math functions generic in the scalar (double or Dual), named apart from the
// math library's so that both overloads resolve exactly.
__device__ __forceinline__ double sexp(double a) { return exp(a); }
__device__ __forceinline__ double slog10(double a) { return log10(a); }
__device__ __forceinline__ double sexp10(double a) { return exp10(a); }
__device__ __forceinline__ double spow(double a, double n) { return pow(a, n); }
__device__ __forceinline__ double sfmax(double a, double c) { return fmax(a, c); }
__device__ __forceinline__ Dual sexp(Dual a) { const double e = exp(a.v); return {e, e * a.d}; }
__device__ __forceinline__ Dual slog10(Dual a) { return {log10(a.v), a.d / (a.v * 2.302585092994046)}; }
__device__ __forceinline__ Dual sexp10(Dual a) { const double e = exp10(a.v); return {e, e * 2.302585092994046 * a.d}; }
__device__ __forceinline__ Dual spow(Dual a, double n) { const double p = pow(a.v, n); return {p, n * p / a.v * a.d}; }
__device__ __forceinline__ Dual sfmax(Dual a, double c) { return a.v > c ? a : Dual(c, 0.0); }
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(Dual a) { return a.v; }

// ---------------------------------------------------------------- kinetics in scalar S
// Views of the per-evaluation quantities of KinCtx in scalar S.  PlainView gives
// the values; DualView gives (value, d value/dT * dT) for a temperature tangent
// dT, i.e. the directional derivative of every temperature function.
template <int NS>
struct PlainView {
    const KinCtx<NS>& k;
    __device__ double T() const { return k.T; }
    __device__ double lnT() const { return k.lnT; }
    __device__ double invT() const { return k.invT; }
    __device__ double hRT(int s) const { return k.hRT[s]; }
    __device__ double eg(int s) const { return k.eg[s]; }
    __device__ double ieg(int s) const { return k.ieg[s]; }
    __device__ double rt_p0() const { return k.rt_p0; }
    __device__ double Csum() const { return k.Csum; }
};
template <int NS>
struct DualView {
    const KinCtx<NS>& k;
    const double* cpR;  // cp/R of every species at T
    double dT, dCsum;
    // d(g/RT)/dT = -(h/RT)/T;  d(h/RT)/dT = (cp/R - h/RT)/T
    __device__ Dual T() const { return {k.T, dT}; }
    __device__ Dual lnT() const { return {k.lnT, k.invT * dT}; }
    __device__ Dual invT() const { return {k.invT, -k.invT * k.invT * dT}; }
    __device__ Dual hRT(int s) const { return {k.hRT[s], (cpR[s] - k.hRT[s]) * k.invT * dT}; }
    __device__ Dual eg(int s) const { return {k.eg[s], -k.eg[s] * k.hRT[s] * k.invT * dT}; }
    __device__ Dual ieg(int s) const { return {k.ieg[s], k.ieg[s] * k.hRT[s] * k.invT * dT}; }
    __device__ Dual rt_p0() const { return {k.rt_p0, k.rt_p0 * k.invT * dT}; }
    __device__ Dual Csum() const { return {k.Csum, dCsum}; }
};

template <int R, class S>
__device__ __forceinline__ S arrhenius_S(S T, S lnT, S invT) {
    constexpr double b = RXN[R].b, E = RXN[R].EaR;
    if constexpr (b == 0.0 && E == 0.0) return S(1.0);
    else if constexpr (E == 0.0 && b == -1.0) return invT;
    else if constexpr (E == 0.0 && b == -2.0) return invT * invT;
    else if constexpr (b == 0.0) return sexp(-E * invT);
    else if constexpr (b == 2.0) return T * T * sexp(-E * invT);
    else return sexp(b * lnT - E * invT);
}
template <int R, class S>
__device__ __forceinline__ S arrhenius0_S(S lnT, S invT) {
    constexpr double b = RXN[R].b0, E = RXN[R].Ea0R;
    if constexpr (b == 0.0 && E == 0.0) return S(1.0);
    else if constexpr (b == 0.0) return sexp(-E * invT);
    else return sexp(b * lnT - E * invT);
}
// Troe log10 F and its partials (d log10F / d log10Pr, d ln F / dT) in scalar S.
template <int R, class S>
__device__ __forceinline__ S troe_S(S T, S Pr, S& dPr, S& dT) {
    constexpr Reaction rx = RXN[R];
    constexpr bool noT3 = rx.troeT3 < 1e-20, noT1 = rx.troeT1 > 1e20;
    S Fcent, dFcent;
    if constexpr (noT3 && noT1 && !rx.hasT2) {
        Fcent = S(rx.troeA);
        dFcent = S(0.0);
    } else {
        const S e3 = sexp(-T / rx.troeT3), e1 = sexp(-T / rx.troeT1);
        Fcent = (1 - rx.troeA) * e3 + rx.troeA * e1;
        dFcent = -(1 - rx.troeA) / rx.troeT3 * e3 - rx.troeA / rx.troeT1 * e1;
        if constexpr (rx.hasT2) {
            const S e2 = sexp(-rx.troeT2 / T);
            Fcent += e2;
            dFcent += rx.troeT2 / (T * T) * e2;
        }
    }
    const bool prc = !(val(Pr) > 1e-300);
    const S lFc = slog10(sfmax(Fcent, 1e-300));
    const S lPr = slog10(sfmax(Pr, 1e-300));
    const S c = -0.4 - 0.67 * lFc, nn = 0.75 - 1.27 * lFc;
    const S x = lPr + c, den = nn - 0.14 * x;
    const S f1 = x / den;
    const S g = 1.0 / (1.0 + f1 * f1);
    dPr = prc ? S(0.0) : lFc * (-2.0 * f1 * g * g) * (nn / (den * den));
    const S df1 = (-0.67 * den - x * (-1.27 + 0.14 * 0.67)) / (den * den);
    const S dlF_dlFc = g + lFc * (-2.0 * f1 * g * g) * df1;
    dT = (val(Fcent) > 1e-300) ? dlF_dlFc * dFcent / (Fcent * 2.302585092994046) : S(0.0);
    return lFc * g;
}

// Rate of progress q of reaction R (multiplier included) and its gradient
// dq/dC_m (m < NS), dq/dT, in scalar S (the forward chemistry's add_rate/add_jac).
template <int R, int NS, class S, class V>
__device__ __forceinline__ void rxn_grad(const V& kv, const S* C, S& q, S* dq, S& dqdT) {
    constexpr Reaction rx = RXN[R];
    const S T = kv.T(), lnT = kv.lnT(), invT = kv.invT();
    const S kinf = c_A[R] * arrhenius_S<R, S>(T, lnT, invT);
    const S dlnkinf = rx.b * invT + rx.EaR * invT * invT;
    S k, dkdT, dkdM = S(0.0), M = S(0.0);
    if constexpr (rx.type != RXN_ELEMENTARY) {
        M = kv.Csum();
#pragma unroll
        for (int m = 0; m < NS; ++m)
            if (rx.eff[m] != 1.0) M += (rx.eff[m] - 1.0) * C[m];
    }
    if constexpr (rx.type == RXN_ELEMENTARY) {
        k = kinf;
        dkdT = kinf * dlnkinf;
    } else if constexpr (rx.type == RXN_THREE_BODY) {
        k = kinf * M;
        dkdT = k * dlnkinf;
        dkdM = kinf;
    } else {
        const S k0 = c_A0[R] * arrhenius0_S<R, S>(lnT, invT);
        const S dlnk0 = rx.b0 * invT + rx.Ea0R * invT * invT;
        const S Pr = k0 * M / kinf;
        S dPr, dTF;
        const S lF = troe_S<R, S>(T, Pr, dPr, dTF);
        const S F = sexp10(lF);
        const S dlnk_dlnPr = 1.0 - Pr / (1.0 + Pr) + dPr;
        k = kinf * (Pr / (1.0 + Pr)) * F;
        dkdT = k * (dlnkinf + dlnk_dlnPr * (dlnk0 - dlnkinf) + dTF);
        dkdM = val(M) > 0.0 ? k * dlnk_dlnPr / M : k0 * F;
    }
    S ikc = S(1.0);
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) ikc *= kv.ieg(rx.reac[i]);
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) ikc *= kv.eg(rx.prod[i]);
    constexpr int dn = rx.nprod - rx.nreac;
    if constexpr (dn == 1) ikc *= kv.rt_p0();
    else if constexpr (dn == -1) ikc = ikc / kv.rt_p0();
    else if constexpr (dn != 0) ikc *= spow(kv.rt_p0(), (double)dn);
    S Pf = S(1.0), Pb = S(1.0);
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) Pf *= C[rx.reac[i]];
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) Pb *= C[rx.prod[i]];
    const S net = Pf - ikc * Pb;
    S dh = S(0.0);
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) dh += kv.hRT(rx.prod[i]);
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) dh -= kv.hRT(rx.reac[i]);
    const S dlnKc = (dh - (double)dn) * invT;
    dqdT = dkdT * net + k * ikc * dlnKc * Pb;
    q = k * net;
#pragma unroll
    for (int m = 0; m < NS; ++m) dq[m] = S(0.0);
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i) {
        S p = k;
#pragma unroll
        for (int j = 0; j < rx.nreac; ++j)
            if (j != i) p *= C[rx.reac[j]];
        dq[rx.reac[i]] += p;
    }
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i) {
        S p = k * ikc;
#pragma unroll
        for (int j = 0; j < rx.nprod; ++j)
            if (j != i) p *= C[rx.prod[j]];
        dq[rx.prod[i]] -= p;
    }
    if constexpr (rx.type != RXN_ELEMENTARY) {
        const S t = dkdM * net;
#pragma unroll
        for (int m = 0; m < NS; ++m) dq[m] += t * rx.eff[m];
    }
}

// alpha_r = sum_i wbar_i W_i/rho nu_ir over the unknowns i < NS-1
template <int R, int NS>
__device__ __forceinline__ double rxn_weight(const double* wbar, double ir) {
    constexpr Reaction rx = RXN[R];
    double a = 0.0;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i)
        if (rx.reac[i] < NS - 1) a -= wbar[rx.reac[i]] * D_MW.v[rx.reac[i]];
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i)
        if (rx.prod[i] < NS - 1) a += wbar[rx.prod[i]] * D_MW.v[rx.prod[i]];
    return a * ir;
}

template <int R, int NS>
__device__ __forceinline__ void vjp_rxn(const KinCtx<NS>& kc, const double* C, const double* wbar, double ir,
                                        double* gC, double& gT, double& wf, double* pbar) {
    const double a = rxn_weight<R, NS>(wbar, ir);
    double q, dq[NS], dqdT;
    rxn_grad<R, NS, double>(PlainView<NS>{kc}, C, q, dq, dqdT);
    pbar[R] = fma(a, q, pbar[R]);
    wf = fma(a, q, wf);
#pragma unroll
    for (int m = 0; m < NS; ++m) gC[m] = fma(a, dq[m], gC[m]);
    gT = fma(a, dqdT, gT);
}
template <int NS, size_t... Rs>
__device__ __forceinline__ void all_vjp(const KinCtx<NS>& kc, const double* C, const double* wbar, double ir,
                                        double* gC, double& gT, double& wf, double* pbar, std::index_sequence<Rs...>) {
    (vjp_rxn<(int)Rs, NS>(kc, C, wbar, ir, gC, gT, wf, pbar), ...);
}

// cp/R and d(cp/R)/dT of every species
template <int NS>
__device__ __forceinline__ void species_cp(double T, double* cpR, double* dcpR) {
    const int rg = T <= TMID ? 0 : 1;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const double* a = D_NASA.c[rg][k];
        cpR[k] = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
        dcpR[k] = fma(T, fma(T, fma(T, 4.0 * a[4], 3.0 * a[3]), 2.0 * a[2]), a[1]);
    }
}

// Constant-(rho, e) temperature derivatives at y (R units: e_k/R = T (h_k/RT - 1)/W_k,
// cv_k/R = (cp_k/R - 1)/W_k):  dT/dy_j = -(e_j - e_L)/cv.
template <int NS>
__device__ __forceinline__ void temp_grad(const KinCtx<NS>& kc, const double* cpR, const double* y, double* dTdy,
                                          double* cvk, double& cv, double& ETT, const double* dcpR) {
    constexpr int N = NS - 1, L = NS - 1;
    double YL = 1.0;
#pragma unroll
    for (int k = 0; k < N; ++k) YL -= y[k];
    cv = 0.0;
    ETT = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        cvk[k] = (cpR[k] - 1.0) * INVW.v[k];
        const double Yk = k < N ? y[k] : YL;
        cv = fma(Yk, cvk[k], cv);
        if (dcpR) ETT = fma(Yk, dcpR[k] * INVW.v[k], ETT);
    }
    const double eL = kc.T * (kc.hRT[L] - 1.0) * INVW.v[L];
#pragma unroll
    for (int j = 0; j < N; ++j) dTdy[j] = -(kc.T * (kc.hRT[j] - 1.0) * INVW.v[j] - eL) / cv;
}

// ybar = J(y)^T wbar (the vector-Jacobian product of the right-hand side) and
// pbar += f_p(y)^T wbar; re (may be null) += (wbar . df/drho, wbar . df/de), the
// derivatives at fixed y of f = W/rho w(C = rho z(y), T(y, e)):
//   df/drho = -f/rho + W/rho dw/dC z,   df/de = W/rho dw/dT / (R cv).
// T: guess in, converged temperature out.
template <int NS>
__device__ __noinline__ bool chem_vjp(double rho, double e, double& T, const double* y, const double* wbar,
                                      double* ybar, double* pbar, double* re) {
    constexpr int N = NS - 1, L = NS - 1;
    double z[NS], C[NS], m[6];
    comp<NS>(y, rho, z, C);
    double Tn = T;
    if (!solve_T<NS>(z, e, Tn, m)) return false;
    T = Tn;
    KinCtx<NS> kc;
    kin_setup<NS, false>(T, C, kc);
    double cpR[NS], dcpR[NS], cvk[NS], dTdy[N], cv, ETT;
    species_cp<NS>(T, cpR, dcpR);
    temp_grad<NS>(kc, cpR, y, dTdy, cvk, cv, ETT, nullptr);
    double gC[NS], gT = 0.0, wf = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) gC[k] = 0.0;
    all_vjp<NS>(kc, C, wbar, 1.0 / rho, gC, gT, wf, pbar, std::make_index_sequence<NR>{});
    // inside the small jump of e(T) at T_mid the inversion returns T_mid, which does
    // not move with y or e: no derivative through T there
    const bool stuck = T == TMID;
    const double cl = rho * gC[L] * INVW.v[L];
#pragma unroll
    for (int j = 0; j < N; ++j) ybar[j] = rho * gC[j] * INVW.v[j] - cl + (stuck ? 0.0 : dTdy[j] * gT);
    if (re) {
        double zg = 0.0;
#pragma unroll
        for (int k = 0; k < NS; ++k) zg = fma(z[k], gC[k], zg);
        re[0] += zg - wf / rho;
        if (!stuck) re[1] += gT / (RU * cv);
    }
    return true;
}

template <int R, int NS>
__device__ __forceinline__ void hess_rxn(const KinCtx<NS>& kc, const double* cpR, const double* C, const double* G,
                                         const double* dTdy, double rho, double ir, double* gC, double& gT, double* wT,
                                         double* pbar) {
    constexpr Reaction rx = RXN[R];
    constexpr int N = NS - 1, L = NS - 1;
    // beta_j = sum_i nu_ir W_i/rho G_ij
    double beta[N];
#pragma unroll
    for (int j = 0; j < N; ++j) beta[j] = 0.0;
#pragma unroll
    for (int i = 0; i < rx.nreac; ++i)
        if (rx.reac[i] < N) {
            const double w = -D_MW.v[rx.reac[i]] * ir;
#pragma unroll
            for (int j = 0; j < N; ++j) beta[j] = fma(w, G[rx.reac[i] * N + j], beta[j]);
        }
#pragma unroll
    for (int i = 0; i < rx.nprod; ++i)
        if (rx.prod[i] < N) {
            const double w = D_MW.v[rx.prod[i]] * ir;
#pragma unroll
            for (int j = 0; j < N; ++j) beta[j] = fma(w, G[rx.prod[i] * N + j], beta[j]);
        }
    // tangent of (C, T) along beta
    Dual Cd[NS];
    double sb = 0.0, dT = 0.0, dCs = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const double d = rho * beta[k] * INVW.v[k];
        Cd[k] = Dual(C[k], d);
        dCs += d;
        sb += beta[k];
        dT = fma(dTdy[k], beta[k], dT);
    }
    const double dL = -rho * sb * INVW.v[L];
    Cd[L] = Dual(C[L], dL);
    dCs += dL;
    Dual q, dq[NS], dqdT;
    rxn_grad<R, NS, Dual>(DualView<NS>{kc, cpR, dT, dCs}, Cd, q, dq, dqdT);
    pbar[R] += q.d;
#pragma unroll
    for (int m = 0; m < NS; ++m) gC[m] += dq[m].d;
    gT += dqdT.d;
#pragma unroll
    for (int j = 0; j < N; ++j) wT[j] = fma(dqdT.v, beta[j], wT[j]);
}
template <int NS, size_t... Rs>
__device__ __forceinline__ void all_hess(const KinCtx<NS>& kc, const double* cpR, const double* C, const double* G,
                                         const double* dTdy, double rho, double ir, double* gC, double& gT, double* wT,
                                         double* pbar, std::index_sequence<Rs...>) {
    (hess_rxn<(int)Rs, NS>(kc, cpR, C, G, dTdy, rho, ir, gC, gT, wT, pbar), ...);
}

// ybar += grad_y <J(y), G>, pbar += grad_p <J(y), G> (G row-major N x N).
//   grad_y sum_r D_beta q_r = C'^T (d2q/dC dtan) + dT/dy (d2q/dT dtan) + H_T (sum_r dq_r/dT beta_r)
// with the Hessian of T(y) at fixed (rho, e):
//   T_jm = -(E_TT T_j T_m + (cv_m - cv_L) T_j + (cv_j - cv_L) T_m) / cv.
// re (may be null) += the derivatives of <J, G> in rho and e at fixed y:
//   d/drho = sum_r [ z . tan(dq_r/dC) - dq_r/dT dT_r / rho ],
//   d/de   = [ sum_r tan(dq_r/dT) - (sum_j (cv_j - cv_L) w_j + E_TT dT/dy . w) / cv ] / (R cv),
// w = sum_r dq_r/dT beta_r, tan() the dual tangent along beta_r.
template <int NS>
__device__ __noinline__ bool chem_hess(double rho, double e, double& T, const double* y, const double* G, double* ybar,
                                       double* pbar, double* re) {
    constexpr int N = NS - 1, L = NS - 1;
    double z[NS], C[NS], m[6];
    comp<NS>(y, rho, z, C);
    double Tn = T;
    if (!solve_T<NS>(z, e, Tn, m)) return false;
    T = Tn;
    KinCtx<NS> kc;
    kin_setup<NS, false>(T, C, kc);
    double cpR[NS], dcpR[NS], cvk[NS], dTdy[N], cv, ETT;
    species_cp<NS>(T, cpR, dcpR);
    temp_grad<NS>(kc, cpR, y, dTdy, cvk, cv, ETT, dcpR);
    double gC[NS], gT = 0.0, wT[N];
#pragma unroll
    for (int k = 0; k < NS; ++k) gC[k] = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) wT[k] = 0.0;
    all_hess<NS>(kc, cpR, C, G, dTdy, rho, 1.0 / rho, gC, gT, wT, pbar, std::make_index_sequence<NR>{});
    double tw = 0.0, cw = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        tw = fma(dTdy[j], wT[j], tw);
        cw = fma(cvk[j] - cvk[L], wT[j], cw);
    }
    // at the T_mid jump T(y, e) = T_mid does not move: the matrix J keeps its
    // dT/dy formula, whose y-derivative at fixed T is the only curvature left
    const bool stuck = T == TMID;
    const double cl = rho * gC[L] * INVW.v[L], icv = 1.0 / cv;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const double hT = stuck ? -(cvk[j] - cvk[L]) * tw * icv
                                : -(ETT * dTdy[j] * tw + dTdy[j] * cw + (cvk[j] - cvk[L]) * tw) * icv;
        ybar[j] += rho * gC[j] * INVW.v[j] - cl + (stuck ? 0.0 : dTdy[j] * gT) + hT;
    }
    if (re) {
        double zg = 0.0;
#pragma unroll
        for (int k = 0; k < NS; ++k) zg = fma(z[k], gC[k], zg);
        re[0] += zg - tw / rho;
        if (!stuck) re[1] += (gT - (cw + ETT * tw) * icv) * icv / RU;
    }
    return true;
}

// Solves M^T x = b with the factors of lu_factor (P M = L U): U^T w = b,
// L^T v = w, x = P^T v.
template <int N>
__device__ __forceinline__ void lu_solve_T(const double* A, const int* piv, double* b) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
#pragma unroll
        for (int j = 0; j < i; ++j) b[i] = fma(-A[j * N + i], b[j], b[i]);
        b[i] *= A[i * N + i];  // lu_factor stores the reciprocal pivots
    }
#pragma unroll
    for (int i = N - 2; i >= 0; --i)
#pragma unroll
        for (int j = i + 1; j < N; ++j) b[i] = fma(-A[j * N + i], b[j], b[i]);
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
        const int p = piv[k];
        if (p != k) {
#pragma unroll
            for (int i = k + 1; i < N; ++i)
                if (i == p) { const double t = b[k]; b[k] = b[i]; b[i] = t; }
        }
    }
}

// Reverse sweep of one accepted Rodas4 step from y with step h (T: temperature
// guess): lam = dJ/dy+ in, dJ/dy out; pbar accumulates dJ/dp and re (may be null)
// dJ/drho, dJ/de (the step depends on them through f and J).
template <int NS>
__device__ __noinline__ bool step_adjoint(double rho, double e, double T, const double* y, double h, double* lam,
                                          double* pbar, double* re) {
    constexpr int N = NS - 1;
    double Mx[N * N], K[6][N], Y[N], f[N];
    int piv[N];
    if (!chem_jac<NS>(rho, e, T, y, Mx)) return false;
    const double inv = 1.0 / (h * RGAMMA), ih = 1.0 / h;
#pragma unroll
    for (int i = 0; i < N * N; ++i) Mx[i] = -Mx[i];
#pragma unroll
    for (int i = 0; i < N; ++i) Mx[i * N + i] += inv;
    if (!lu_factor<N>(Mx, piv)) return false;
    // stages (the accepted attempt of cell_attempt)
    for (int s = 0; s < 6; ++s) {
        const int base = s * (s - 1) / 2;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = y[i];
            for (int j = 0; j < s; ++j) v = fma(RA[base + j], K[j][i], v);
            Y[i] = v;
        }
        if (!chem_rhs<NS>(rho, e, T, Y, f)) return false;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = f[i];
            for (int j = 0; j < s; ++j) v = fma(RC[base + j] * ih, K[j][i], v);
            K[s][i] = v;
        }
        lu_solve<N>(Mx, piv, K[s]);
    }
    // reverse
    double Kb[6][N], yb[N], G[N * N];
#pragma unroll
    for (int i = 0; i < N; ++i) yb[i] = lam[i];
    for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int i = 0; i < N; ++i) Kb[s][i] = RM[s] * lam[i];
#pragma unroll
    for (int i = 0; i < N * N; ++i) G[i] = 0.0;
    for (int s = 5; s >= 0; --s) {
        const int base = s * (s - 1) / 2;
        double Rb[N];
#pragma unroll
        for (int i = 0; i < N; ++i) Rb[i] = Kb[s][i];
        lu_solve_T<N>(Mx, piv, Rb);
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) G[i * N + j] = fma(Rb[i], K[s][j], G[i * N + j]);
        for (int j = 0; j < s; ++j) {
            const double c = RC[base + j] * ih;
#pragma unroll
            for (int i = 0; i < N; ++i) Kb[j][i] = fma(c, Rb[i], Kb[j][i]);
        }
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double v = y[i];
            for (int j = 0; j < s; ++j) v = fma(RA[base + j], K[j][i], v);
            Y[i] = v;
        }
        double Yb[N];
        if (!chem_vjp<NS>(rho, e, T, Y, Rb, Yb, pbar, re)) return false;
#pragma unroll
        for (int i = 0; i < N; ++i) yb[i] += Yb[i];
        for (int j = 0; j < s; ++j) {
#pragma unroll
            for (int i = 0; i < N; ++i) Kb[j][i] = fma(RA[base + j], Yb[i], Kb[j][i]);
        }
    }
    if (!chem_hess<NS>(rho, e, T, y, G, yb, pbar, re)) return false;
#pragma unroll
    for (int i = 0; i < N; ++i) lam[i] = yb[i];
    return true;
}

// ---------------------------------------------------------------- cell runs
// One chemistry call on the conserved state u (cell_begin / cell_attempt /
// cell_end), optionally appending every accepted step (y, h, T) to the tape at
// slot nrec (stored while nrec < cap).  clip receives bit k when y_k was clipped.
template <int NS>
__device__ int run_call(double* u, double dt, double rtol, double atol, double* tape, int64_t tstride, int& nrec,
                        int cap, uint32_t& clip) {
    constexpr int N = NS - 1;
    ChemCell<NS> c;
    int r = cell_begin<NS>(c, u, dt, rtol, atol);
    while (r == CELL_CONTINUE) {
        double yp[N];
#pragma unroll
        for (int k = 0; k < N; ++k) yp[k] = c.y[k];
        const double Tp = c.T;
        const double he = (c.t + 1.01 * c.h >= c.tend) ? c.tend - c.t : c.h;
        const int s0 = c.steps;
        r = cell_attempt<NS>(c, rtol, atol);
        if (tape && c.steps > s0) {
            if (nrec < cap) {
                double* t = tape + (int64_t)nrec * (N + 2) * tstride;
#pragma unroll
                for (int k = 0; k < N; ++k) t[k * tstride] = yp[k];
                t[N * tstride] = he;
                t[(N + 1) * tstride] = Tp;
            }
            ++nrec;
        }
    }
    if (r != CELL_DONE) return r;
    clip = 0;
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (c.y[k] < 0.0) clip |= 1u << k;
    return cell_end<NS>(c, u) ? CELL_DONE : CELL_FAIL;
}

// dT/dy and dp/dy of the state u (y = u/rho at fixed rho, e).
template <int NS>
__device__ bool state_grads(const double* u, double* dT, double* dp, double& T) {
    constexpr int N = NS - 1;
    double rho = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) rho += u[k];
    const double ir = 1.0 / rho;
    const double uu = u[NS] * ir, vv = u[NS + 1] * ir;
    const double e = u[NS + 2] * ir - 0.5 * (uu * uu + vv * vv);
    double y[N], z[NS], C[NS], m[6];
#pragma unroll
    for (int k = 0; k < N; ++k) y[k] = u[k] * ir;
    comp<NS>(y, rho, z, C);
    if (!solve_T<NS>(z, e, T, m)) return false;
    KinCtx<NS> kc;
    kin_setup<NS, false>(T, C, kc);
    double cpR[NS], dcpR[NS], cvk[NS], cv, ETT;
    species_cp<NS>(T, cpR, dcpR);
    temp_grad<NS>(kc, cpR, y, dT, cvk, cv, ETT, nullptr);
    double zs = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) zs += z[k];
    // p = rho R T sum_k Y_k/W_k
#pragma unroll
    for (int j = 0; j < N; ++j) dp[j] = rho * RU * (zs * dT[j] + T * (INVW.v[j] - INVW.v[NS - 1]));
    return true;
}

}  // namespace hf

// ---------------------------------------------------------------- kernel
namespace hf {
namespace {

enum { OBJ_IGNITION = HF_OBJ_IGNITION_DELAY, OBJ_PEAK_PRESSURE = HF_OBJ_PEAK_PRESSURE, OBJ_FINAL_T = HF_OBJ_FINAL_T };

// Forward pass: ncalls calls with checkpoints (ckpt may be null), objective
// bookkeeping; then (BACKWARD) the reverse sweep.  One thread per cell.  The
// forward-only instantiation carries none of the reverse sweep's registers or stack.
#pragma nv_diag_suppress 128  // the forward-only instantiation ends before the reverse sweep's loops
template <int NS, bool BACKWARD>
__global__ void __launch_bounds__(32) k_chem_adjoint(AdjointArgs a) {
    constexpr int N = NS - 1, NV = NS + 3;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.chunk) return;
    const int64_t gi = a.i0 + i;
    const int64_t cst = a.chunk;  // stride of the scratch arrays
    double u[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) u[n] = a.U0[gi + n * a.cs];
    auto fail_cell = [&](int code) {
        a.fail[gi] = code;
        atomicOr(&a.st->flags, code == CELL_MAXSTEPS ? ST_MAXSTEPS : ST_CHEM_FAIL);
        atomicMin(&a.st->bad_cell, (unsigned long long)gi);
        a.J[gi] = __longlong_as_double(0x7ff8000000000000ll);
    };
    Props pr;
    if (!properties<NS>(u, pr, 1000.0)) { fail_cell(CELL_FAIL); return; }
    const double T0 = pr.T, Ts = T0 + a.dT;
    int n_ign = -1, n_pmax = 0;
    double Ta = 0.0, Tb = 0.0, pmax = pr.p, Tprev = T0;
    unsigned long long steps = 0;
    for (int n = 0; n < a.ncalls; ++n) {
        if (a.ckpt && n % a.K == 0) {
            double* c = a.ckpt + (int64_t)(n / a.K) * NV * cst;
#pragma unroll
            for (int v = 0; v < NV; ++v) c[v * cst + i] = u[v];
        }
        int nrec = 0;
        uint32_t clip = 0;
        const int r = run_call<NS>(u, a.dt, a.rtol, a.atol, nullptr, 0, nrec, 0, clip);
        if (r != CELL_DONE) { fail_cell(r == CELL_MAXSTEPS ? CELL_MAXSTEPS : CELL_FAIL); return; }
        if (!properties<NS>(u, pr, Tprev)) { fail_cell(CELL_FAIL); return; }
        if (n_ign < 0 && pr.T >= Ts) { n_ign = n; Ta = Tprev; Tb = pr.T; }
        if (pr.p > pmax) { pmax = pr.p; n_pmax = n + 1; }
        Tprev = pr.T;
    }
    double Jv;
    if (a.objective == OBJ_FINAL_T) Jv = Tprev;
    else if (a.objective == OBJ_PEAK_PRESSURE) Jv = pmax;
    else Jv = n_ign < 0 ? __longlong_as_double(0x7ff8000000000000ll)
                        : n_ign * a.dt + a.dt * (Ts - Ta) / (Tb - Ta);
    a.J[gi] = Jv;
    a.fail[gi] = 0;
    if constexpr (!BACKWARD) return;
    double pbar[NR], lam[N];
#pragma unroll
    for (int r = 0; r < NR; ++r) pbar[r] = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) lam[k] = 0.0;
    const bool active = !(a.objective == OBJ_IGNITION && n_ign < 0);
    // seed dJ/dy_n at call boundary n (state un)
    auto seed = [&](int n, const double* un) -> bool {
        double w = 0.0;
        bool useT = true;
        if (a.objective == OBJ_FINAL_T) {
            if (n == a.ncalls) w = 1.0;
        } else if (a.objective == OBJ_PEAK_PRESSURE) {
            if (n == n_pmax) { w = 1.0; useT = false; }
        } else {
            const double d = Tb - Ta;
            if (n == n_ign) w = a.dt * (Ts - Tb) / (d * d);
            else if (n == n_ign + 1) w = -a.dt * (Ts - Ta) / (d * d);
            if (n == 0) w += a.dt / d;  // through the threshold T_0 + dT
        }
        if (w == 0.0) return true;
        double gT[N], gp[N], T = 1000.0;
        if (!state_grads<NS>(un, gT, gp, T)) return false;
#pragma unroll
        for (int k = 0; k < N; ++k) lam[k] = fma(w, useT ? gT[k] : gp[k], lam[k]);
        return true;
    };
    bool ok = active;
    const int nseg = (a.ncalls + a.K - 1) / a.K;
    for (int sg = nseg - 1; ok && sg >= 0; --sg) {
        const int n0 = sg * a.K, n1 = min(n0 + a.K, a.ncalls);
        // recompute the segment: boundary states and the tape of accepted steps
        const double* c = a.ckpt + (int64_t)sg * NV * cst;
#pragma unroll
        for (int v = 0; v < NV; ++v) { u[v] = c[v * cst + i]; a.seg[v * cst + i] = u[v]; }
        int nrec = 0;
        for (int n = n0; ok && n < n1; ++n) {
            uint32_t clip = 0;
            const int before = nrec;
            ok = run_call<NS>(u, a.dt, a.rtol, a.atol, a.tape + i, cst, nrec, a.cap, clip) == CELL_DONE;
            a.nstep[(int64_t)(n - n0) * cst + i] = nrec - before;
            a.clipm[(int64_t)(n - n0) * cst + i] = clip;
            double* sb = a.seg + (int64_t)(n - n0 + 1) * NV * cst;
#pragma unroll
            for (int v = 0; v < NV; ++v) sb[v * cst + i] = u[v];
        }
        const bool overflow = nrec > a.cap;
        if (ok && sg == nseg - 1) {
            double ue[NV];
            const double* sb = a.seg + (int64_t)(n1 - n0) * NV * cst;
#pragma unroll
            for (int v = 0; v < NV; ++v) ue[v] = sb[v * cst + i];
            ok = seed(n1, ue);
        }
        int end = nrec;
        for (int n = n1 - 1; ok && n >= n0; --n) {
            const uint32_t clip = a.clipm[(int64_t)(n - n0) * cst + i];
#pragma unroll
            for (int k = 0; k < N; ++k)
                if (clip & (1u << k)) lam[k] = 0.0;
            const int cnt = a.nstep[(int64_t)(n - n0) * cst + i];
            double un[NV];
            const double* sb = a.seg + (int64_t)(n - n0) * NV * cst;
#pragma unroll
            for (int v = 0; v < NV; ++v) un[v] = sb[v * cst + i];
            int base = end - cnt;
            end = base;
            if (overflow) {
                // recompute this call alone into the start of the tape
                double uc[NV];
#pragma unroll
                for (int v = 0; v < NV; ++v) uc[v] = un[v];
                int nr = 0;
                uint32_t cl = 0;
                ok = run_call<NS>(uc, a.dt, a.rtol, a.atol, a.tape + i, cst, nr, a.cap, cl) == CELL_DONE && nr == cnt;
                base = 0;
            }
            double rho = 0.0;
#pragma unroll
            for (int k = 0; k < NS; ++k) rho += un[k];
            const double ir = 1.0 / rho;
            const double uu = un[NS] * ir, vv = un[NS + 1] * ir;
            const double e = un[NS + 2] * ir - 0.5 * (uu * uu + vv * vv);
            for (int s = cnt - 1; ok && s >= 0; --s) {
                const double* t = a.tape + i + (int64_t)(base + s) * (N + 2) * cst;
                double ys[N];
#pragma unroll
                for (int k = 0; k < N; ++k) ys[k] = t[k * cst];
                ok = step_adjoint<NS>(rho, e, t[(N + 1) * cst], ys, t[N * cst], lam, pbar, nullptr);
                ++steps;
            }
            if (ok) ok = seed(n, un);
        }
    }
    if (active && !ok) { fail_cell(CELL_FAIL); return; }
    atomicAdd(&a.st->steps, steps);
#pragma unroll
    for (int r = 0; r < NR; ++r) a.dJdp[(int64_t)r * a.count + gi] = pbar[r];
    if (a.dJdy0) {
#pragma unroll
        for (int k = 0; k < N; ++k) a.dJdy0[(int64_t)k * a.count + gi] = lam[k];
    }
}

#pragma nv_diag_default 128

// Adjoint of the react phase of a Strang step on the cells of a ghosted patch: one
// chemistry call (plain form, the frozen accepted steps recomputed into the tape)
// per cell.  ubar_in = (du_out/du_in)^T ubar_out through
//   u_in -> (y = u_k/rho, rho = sum u_k, e = E/rho - |m|^2/(2 rho^2)) -> Rodas4 steps
//   -> clip -> u_out_k = rho max(0, y_k), u_out_L = rho - sum u_out_k, m and E unchanged,
// and pcell[r][cell] += dJ/d ln A_r of the cell.  One thread per cell of [i0, i0+chunk).
template <int NS>
__global__ void __launch_bounds__(32) k_chem_call_adjoint(hf_patch P, const double* __restrict__ U,
                                                          const double* __restrict__ ubar_out,
                                                          double* __restrict__ ubar_in, double dt, double rtol,
                                                          double atol, double* __restrict__ tape, int cap, int64_t i0,
                                                          int64_t chunk, double* __restrict__ pcell, DevStatus* st) {
    constexpr int N = NS - 1, NV = NS + 3;
    const int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = (int64_t)P.nx * P.ny, i = i0 + li;
    if (li >= chunk || i >= nc) return;
    const int ci = (int)(i % P.nx), cj = (int)(i / P.nx);
    const int64_t g = P.offset + (int64_t)(cj + P.ng) * P.pitch + (ci + P.ng);
    double u[NV], ub[NV], uc[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        u[n] = U[g + n * P.comp_stride];
        ub[n] = ubar_out[g + n * P.comp_stride];
        uc[n] = u[n];
    }
    int nrec = 0;
    uint32_t clip = 0;
    const int r = run_call<NS>(uc, dt, rtol, atol, tape + li, chunk, nrec, cap, clip);
    double out[NV];
#pragma unroll
    for (int n = 0; n < NV; ++n) out[n] = 0.0;
    bool ok = r == CELL_DONE && nrec <= cap;
    if (ok) {
        double rho = 0.0;
#pragma unroll
        for (int k = 0; k < NS; ++k) rho += u[k];
        const double ir = 1.0 / rho;
        const double mx = u[NS], my = u[NS + 1], E = u[NS + 2];
        const double e = E * ir - 0.5 * ((mx * ir) * (mx * ir) + (my * ir) * (my * ir));
        // output side: u_out_k = rho Y'_k (k < N), u_out_L = rho (1 - sum Y'_k)
        double lam[N], rhob = ub[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const double d = ub[k] - ub[N];
            lam[k] = (clip >> k & 1u) ? 0.0 : rho * d;
            rhob = fma(uc[k] * ir, d, rhob);
        }
        double pb[NR], re[2] = {0.0, 0.0};
#pragma unroll
        for (int q = 0; q < NR; ++q) pb[q] = 0.0;
        for (int s = nrec - 1; ok && s >= 0; --s) {
            const double* t = tape + li + (int64_t)s * (N + 2) * chunk;
            double ys[N];
#pragma unroll
            for (int k = 0; k < N; ++k) ys[k] = t[k * chunk];
            ok = step_adjoint<NS>(rho, e, t[(N + 1) * chunk], ys, t[N * chunk], lam, pb, re);
        }
        if (ok) {
#pragma unroll
            for (int q = 0; q < NR; ++q) pcell[(int64_t)q * nc + i] += pb[q];
            // input side: y_k = u_k / rho, rho = sum u_k, e(E, m, rho)
            rhob += re[0];
#pragma unroll
            for (int k = 0; k < N; ++k) {
                out[k] = lam[k] * ir;
                rhob = fma(-lam[k] * u[k] * ir, ir, rhob);
            }
            const double eb = re[1];
            out[NS + 2] = ub[NS + 2] + eb * ir;
            out[NS] = ub[NS] - eb * mx * ir * ir;
            out[NS + 1] = ub[NS + 1] - eb * my * ir * ir;
            rhob += eb * (-E * ir * ir + (mx * mx + my * my) * ir * ir * ir);
#pragma unroll
            for (int k = 0; k < NS; ++k) out[k] += rhob;
        }
    }
    if (!ok) {
        atomicOr(&st->flags, ST_CHEM_FAIL);
        atomicMin(&st->bad_cell, (unsigned long long)i);
    }
#pragma unroll
    for (int n = 0; n < NV; ++n) ubar_in[g + n * P.comp_stride] = out[n];
}

}  // namespace

cudaError_t launch_chem_call_adjoint(int ns, const hf_patch& P, const double* U, const double* ubar_out,
                                     double* ubar_in, double dt, double rtol, double atol, double* tape, int cap,
                                     int64_t i0, int64_t chunk, double* pcell, DevStatus* st, cudaStream_t s,
                                     int64_t* launches) {
    if (chunk <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((chunk + 31) / 32);
    if (ns == 9)
        k_chem_call_adjoint<9><<<grid, 32, 0, s>>>(P, U, ubar_out, ubar_in, dt, rtol, atol, tape, cap, i0, chunk, pcell,
                                                   st);
    else
        k_chem_call_adjoint<10><<<grid, 32, 0, s>>>(P, U, ubar_out, ubar_in, dt, rtol, atol, tape, cap, i0, chunk,
                                                    pcell, st);
    if (launches) ++*launches;
    return cudaGetLastError();
}

size_t adjoint_bytes_per_cell(int ns, int ncalls, int K, int cap) {
    const int nv = ns + 3, n = ns - 1;
    const int nck = (ncalls + K - 1) / K;
    return sizeof(double) * ((size_t)nck * nv + (size_t)(K + 1) * nv + (size_t)cap * (n + 2)) +
           sizeof(int32_t) * 2 * (size_t)K;
}

cudaError_t launch_chem_adjoint(int ns, const AdjointArgs& a, cudaStream_t s, int64_t* launches) {
    if (a.chunk <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((a.chunk + 31) / 32);
    if (a.backward) {
        if (ns == 9) k_chem_adjoint<9, true><<<grid, 32, 0, s>>>(a);
        else k_chem_adjoint<10, true><<<grid, 32, 0, s>>>(a);
    } else {
        if (ns == 9) k_chem_adjoint<9, false><<<grid, 32, 0, s>>>(a);
        else k_chem_adjoint<10, false><<<grid, 32, 0, s>>>(a);
    }
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace hf
