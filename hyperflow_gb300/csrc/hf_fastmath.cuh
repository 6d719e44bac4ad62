// Table-driven FP64 exponential and logarithm for the chemistry kernels, after
// P. T. P. Tang, "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15 (1989) 144-157, and "Table-driven
// implementation of the logarithm function in IEEE floating-point arithmetic",
// ACM TOMS 16 (1990) 378-400, with 64-entry tables (hf_fastmath_tables.h, written by
// gen_fastmath.py).  The kinetics pass evaluates about 30 exponentials per call; on
// this GPU FP64 instructions are the kernel's limit, and these forms take about 10
// (exp), 15 (exp(x) and exp(-x) together) and 15 (log) FP64 instructions, within
// about 1 ulp.  Arguments outside the fast ranges go to the library functions.
#pragma once
#include "hf_fastmath_tables.h"

namespace hf {

// the library functions for the arguments outside the fast ranges (out of line: one
// copy of their code)
static __device__ __noinline__ double fm_exp_lib(double x) { return exp(x); }
static __device__ __noinline__ double fm_log_lib(double x) { return log(x); }

// 2^m * v for v in [0.5, 2.1) and |m| <= 1010: the result stays a normal number
__device__ __forceinline__ double fm_scale(double v, int m) {
    return __hiloint2double(__double2hiint(v) + m * (1 << 20), __double2loint(v));
}

// exp(x), |x| < 700: x = k ln2/64 + r with k = rint(64 x/ln2) and |r| <= ln2/128;
// k = 64 m + j; exp(x) = 2^m 2^(j/64) (1 + p(r)) with p the degree-5 Taylor
// polynomial of exp(r) - 1 (remainder below 4e-17 on that interval).
__device__ __forceinline__ double fexp(double x) {
    if (!(fabs(x) < 700.0)) return fm_exp_lib(x);
    const double SH = 0x1.8p52;  // adding it rounds to an integer held in the low word
    const double t = fma(x, fm::INV_LN2_64, SH);
    const int k = __double2loint(t);
    const double kd = t - SH;
    double r = fma(-kd, fm::LN2_64_HI, x);  // exact: kd * HI has at most 53 bits
    r = fma(-kd, fm::LN2_64_LO, r);
    const double q = fma(fma(fma(r, 1.0 / 120.0, 1.0 / 24.0), r, 1.0 / 6.0), r, 0.5);
    const double p = fma(r * r, q, r);
    const int j = k & 63;
    const double tj = fm::EXP_TAB[j];
    return fm_scale(fma(tj, p, tj), (k - j) / 64);
}

// exp(x) and exp(-x) from one reduction: with E and O the even and odd parts of p,
// exp(x) = 2^m 2^(j/64) (1 + E + O) and exp(-x) = 2^-m 2^(-j/64) (1 + E - O).
__device__ __forceinline__ void fexp_pair(double x, double& ep, double& em) {
    if (!(fabs(x) < 700.0)) {
        ep = fm_exp_lib(x);
        em = fm_exp_lib(-x);
        return;
    }
    const double SH = 0x1.8p52;
    const double t = fma(x, fm::INV_LN2_64, SH);
    const int k = __double2loint(t);
    const double kd = t - SH;
    double r = fma(-kd, fm::LN2_64_HI, x);
    r = fma(-kd, fm::LN2_64_LO, r);
    const double r2 = r * r;
    const double E = r2 * fma(r2, 1.0 / 24.0, 0.5);
    const double O = r * fma(r2, fma(r2, 1.0 / 120.0, 1.0 / 6.0), 1.0);
    const int j = k & 63, m = (k - j) / 64;
    const double tp = fm::EXP_TAB[j], tm = fm::EXPM_TAB[j];
    ep = fm_scale(fma(tp, E + O, tp), m);
    em = fm_scale(fma(tm, E - O, tm), -m);
}

// log(x), x in [2^-1021, 2^1023): x = 2^m y, y in [1, 2); F = 1 + (j + 1/2)/64 with j
// the top 6 fraction bits of y; u = (y - F)/F, |u| <= 1/129;
// log(x) = m ln2 + log(F) + log1p(u), log1p by its degree-7 Taylor polynomial
// (remainder below 2e-18).
__device__ __forceinline__ double flog(double x) {
    if (!(x >= 0x1p-1021 && x < 0x1p1023)) return fm_log_lib(x);
    const int hi = __double2hiint(x);
    const int m = (hi >> 20) - 1023;
    const int j = (hi >> 14) & 63;
    const double y = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, __double2loint(x));
    const double F = fma((double)j, 1.0 / 64.0, 1.0 + 1.0 / 128.0);  // exact
    const double u = (y - F) * fm::LOG_IF[j];                           // y - F is exact
    const double q = fma(fma(fma(fma(fma(u, 1.0 / 7.0, -1.0 / 6.0), u, 0.2), u, -0.25), u, 1.0 / 3.0), u, -0.5);
    const double l1p = fma(u * u, q, u);
    const double md = (double)m;
    return fma(md, fm::LN2_HI, fm::LOG_F[j]) + fma(md, fm::LN2_LO, l1p);
}

}  // namespace hf
