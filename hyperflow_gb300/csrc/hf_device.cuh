// Device-side thermodynamics, equation of state and HLLC flux for the H2_Li
// mechanism (NS = 9 species of the file, or 10 with the inert AR extension).
//
// Layout: a cell state is NV = NS + 3 doubles in the reference's order
// (rhoY_0..rhoY_{NS-1}, rho*u, rho*v, rho*E), HyperFlow_V3/src/solver.hpp:17-25.
//
// The EOS closure restates what physics.cpp:4-15 gets from Cantera's ideal-gas
// phase: NASA7 polynomials (T <= T_mid uses the low range), e = sum Y_k e_k(T),
// p = rho R T / W, frozen sound speed a = sqrt(cp/cv R T / W).  The UV inversion
// is a Newton solve on T.  It first iterates in FP32 (cheap on this part) from
// the caller's guess, then finishes in FP64 until the correction is below
// 1e-10 T, which leaves T converged to rounding: the FP64 answer does not depend
// on the guess or on the FP32 phase.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mech_h2li.h"

namespace hf {
using namespace hfmech;

constexpr double RU = GAS_CONSTANT;

// Per-species coefficients of e_k(T)*W_k/R = c0 T + c1 T^2 + c2 T^3 + c3 T^4 + c4 T^5 + c5
// with c0 = a0 - 1, c1 = a1/2, c2 = a2/3, c3 = a3/4, c4 = a4/5, c5 = a5.
struct ECoef { double c[2][NS_MAX][6]; };
constexpr ECoef make_ecoef() {
    ECoef e{};
    for (int r = 0; r < 2; ++r)
        for (int k = 0; k < NS_MAX; ++k) {
            const double* a = r == 0 ? NASA_LOW[k] : NASA_HIGH[k];
            e.c[r][k][0] = a[0] - 1.0;
            e.c[r][k][1] = a[1] / 2.0;
            e.c[r][k][2] = a[2] / 3.0;
            e.c[r][k][3] = a[3] / 4.0;
            e.c[r][k][4] = a[4] / 5.0;
            e.c[r][k][5] = a[5];
        }
    return e;
}
__device__ constexpr ECoef D_ECOEF = make_ecoef();
struct InvW { double v[NS_MAX]; };
constexpr InvW make_invw() {
    InvW w{};
    for (int k = 0; k < NS_MAX; ++k) w.v[k] = 1.0 / MW[k];
    return w;
}
__device__ constexpr InvW INVW = make_invw();
struct MolW { double v[NS_MAX]; };
constexpr MolW make_mw() {
    MolW w{};
    for (int k = 0; k < NS_MAX; ++k) w.v[k] = MW[k];
    return w;
}
__device__ constexpr MolW D_MW = make_mw();
struct Nasa { double c[2][NS_MAX][7]; };
constexpr Nasa make_nasa() {
    Nasa n{};
    for (int k = 0; k < NS_MAX; ++k)
        for (int j = 0; j < 7; ++j) { n.c[0][k][j] = NASA_LOW[k][j]; n.c[1][k][j] = NASA_HIGH[k][j]; }
    return n;
}
__device__ constexpr Nasa D_NASA = make_nasa();
constexpr double TMID = 1000.0;  // T_MID is 1000 K for every species of the table

// Mixture polynomial of one NASA range: e(T)/R = sum_j m[j] T^(j+1) + m[5], with
// m[j] = sum_k z_k c_kj and z_k = Y_k / W_k.
template <int NS, int RG>
__device__ __forceinline__ void mix_coef_r(const double* z, double* m) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < NS; ++k) s = fma(z[k], D_ECOEF.c[RG][k][j], s);
        m[j] = s;
    }
}
template <int NS>
__device__ __forceinline__ void mix_coef(const double* z, int range, double* m) {
    if (range == 0) mix_coef_r<NS, 0>(z, m);
    else mix_coef_r<NS, 1>(z, m);
}
template <int NS, int RG>
__device__ __forceinline__ void mix_coef_f(const double* z, float* m) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < NS; ++k) s = fmaf((float)z[k], (float)D_ECOEF.c[RG][k][j], s);
        m[j] = s;
    }
}
// e/R and cv/R from mixture coefficients
__device__ __forceinline__ double poly_e(const double* m, double T) {
    return fma(T, fma(T, fma(T, fma(T, fma(T, m[4], m[3]), m[2]), m[1]), m[0]), m[5]);
}
__device__ __forceinline__ double poly_cv(const double* m, double T) {
    return fma(T, fma(T, fma(T, fma(T, 5.0 * m[4], 4.0 * m[3]), 3.0 * m[2]), 2.0 * m[1]), m[0]);
}
__device__ __forceinline__ float poly_e_f(const float* m, float T) {
    return fmaf(T, fmaf(T, fmaf(T, fmaf(T, fmaf(T, m[4], m[3]), m[2]), m[1]), m[0]), m[5]);
}
__device__ __forceinline__ float poly_cv_f(const float* m, float T) {
    return fmaf(T, fmaf(T, fmaf(T, fmaf(T, 5.0f * m[4], 4.0f * m[3]), 3.0f * m[2]), 2.0f * m[1]), m[0]);
}

// Solves e(T) = e_target for the composition z (z_k = Y_k/W_k).  T holds the
// starting guess on entry and the converged temperature on exit.  m receives the
// FP64 mixture coefficients of the range that T ends in (for cv afterwards).
// Returns false when the iteration does not converge to a finite positive T.
// The FP32 phase pays even from a warm guess (the previous right-hand side's T): it
// leaves one FP64 iteration to do instead of two or three.
template <int NS>
__device__ __forceinline__ bool solve_T(const double* z, double e_target, double& T, double* m) {
    if (!(T > 0.0) || !(T < 1e5)) T = 1000.0;
    // FP32 phase: both ranges, Newton until |dT| <= 1e-5 T.
    {
        float mlo[6], mhi[6];
        mix_coef_f<NS, 0>(z, mlo);
        mix_coef_f<NS, 1>(z, mhi);
        const float et = (float)(e_target * (1.0 / RU));
        float t = (float)T;
        for (int it = 0; it < 40; ++it) {
            const float* mm = t <= 1000.0f ? mlo : mhi;
            float dt = (et - poly_e_f(mm, t)) / poly_cv_f(mm, t);
            dt = fminf(1000.0f, fmaxf(-1000.0f, dt));
            float tn = t + dt;
            if (!(tn > 0.0f)) tn = 0.5f * t;
            t = tn;
            if (!(fabsf(dt) > 1e-5f * t)) break;
        }
        if (t > 0.0f && t < 1e5f) T = (double)t;
    }
    // FP64 phase: stop once the applied correction is below 1e-10 T (quadratic
    // convergence leaves T at rounding level).  Inside the small jump of e(T) at
    // T_mid (no root), two consecutive sub-kelvin flips across T_mid return T_mid.
    const double et = e_target * (1.0 / RU);
    int range = T <= TMID ? 0 : 1;
    mix_coef<NS>(z, range, m);
    int flips = 0;
    for (int it = 0; it < 60; ++it) {
        const int r = T <= TMID ? 0 : 1;
        if (r != range) {
            range = r;
            mix_coef<NS>(z, range, m);
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
            if (rf != range) mix_coef<NS>(z, rf, m);
            return true;
        }
        flips = ((T <= TMID) != (Tn <= TMID) && step < 0.5) ? flips + 1 : 0;
        if (flips >= 2) {
            T = TMID;
            mix_coef<NS>(z, 0, m);
            return true;
        }
        T = Tn;
    }
    return false;
}

struct Props { double p, a, T; };

// physics.cpp:4-15 for a state held in registers.  Returns false when the state
// is inadmissible (non-finite, rho <= 0, a negative partial density, or an EOS
// solve that fails).  T_guess seeds the UV inversion.
template <int NS>
__device__ __forceinline__ bool properties(const double* q, Props& s, double T_guess) {
    bool ok = true;
    double rho = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        rho += q[k];
        ok = ok && (q[k] >= 0.0);
    }
#pragma unroll
    for (int n = NS; n < NS + 3; ++n) ok = ok && isfinite(q[n]);
    ok = ok && isfinite(rho) && (rho > 0.0);
    if (!ok) return false;
    const double ir = 1.0 / rho;
    double z[NS];
    double zs = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        z[k] = q[k] * ir * INVW.v[k];
        zs += z[k];
    }
    const double u = q[NS] * ir, v = q[NS + 1] * ir;
    const double e = q[NS + 2] * ir - 0.5 * (u * u + v * v);
    double T = T_guess, m[6];
    if (!solve_T<NS>(z, e, T, m)) return false;
    const double cvR = poly_cv(m, T);  // cv/R per unit mass (times W units)
    const double cpR = cvR + zs;
    s.T = T;
    s.p = rho * RU * T * zs;
    s.a = sqrt(cpR / cvR * RU * T * zs);
    return s.T > 0.0 && s.p > 0.0 && s.a > 0.0 && isfinite(s.a);
}

// physics.cpp:40-44, one component
__device__ __forceinline__ double minmod(double x, double y) {
    return x * y > 0.0 ? copysign(fmin(fabs(x), fabs(y)), x) : 0.0;
}

// physics.cpp:17-38: multispecies HLLC with Davis speeds in direction n (NS or NS+1).
template <int NS, int N>
__device__ __forceinline__ void hllc(const double* l, const double* r, const Props& pl, const Props& pr,
                                     double* f) {
    constexpr int E = NS + 2;
    double rl = 0.0, rr = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) { rl += l[k]; rr += r[k]; }
    const double ul = l[N] / rl, ur = r[N] / rr;
    const double sl = fmin(ul - pl.a, ur - pr.a), sr = fmax(ul + pl.a, ur + pr.a);
    if (sl >= 0.0 || sr <= 0.0) {
        const bool useL = sl >= 0.0;
        const double* q = useL ? l : r;
        const double v = useL ? ul : ur, p = useL ? pl.p : pr.p;
#pragma unroll
        for (int m = 0; m < NS + 3; ++m) f[m] = v * q[m];
        f[N] += p;
        f[E] += p * v;
        return;
    }
    const double dl = rl * (sl - ul), dr = rr * (sr - ur);
    const double sm = (pr.p - pl.p + dl * ul - dr * ur) / (dl - dr);
    const bool left = sm >= 0.0;
    const double* q = left ? l : r;
    const double v = left ? ul : ur, s = left ? sl : sr, p = left ? pl.p : pr.p, rq = left ? rl : rr;
    const double scale = (s - v) / (s - sm);
    double rs = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) rs += q[k] * scale;
    const double estar = q[E] * scale + rs * (sm - v) * (sm + p / (rq * (s - v)));
#pragma unroll
    for (int m = 0; m < NS + 3; ++m) {
        double st = q[m] * scale;
        if (m == N) st = rs * sm;
        if (m == E) st = estar;
        double fl = v * q[m];
        if (m == N) fl += p;
        if (m == E) fl += p * v;
        f[m] = fl + s * (st - q[m]);
    }
}

}  // namespace hf
