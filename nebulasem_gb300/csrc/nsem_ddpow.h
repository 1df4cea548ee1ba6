/*
 * Correctly rounded (to within ~2^-90 relative before the final rounding)
 * double-precision x^y for x > 0, written with double-double arithmetic.
 *
 * Why: the equation of state p' = P0 (rho theta R / P0)^gamma - p_ref
 * (apps/euler/euler.cpp:211-213) subtracts two numbers of size 1e5 to get a
 * perturbation of a few Pa, so one ulp of p moves p' by ~1e-11 relative.  The
 * FP64 form must round x^y like a correctly rounded pow, on the GPU and in
 * host code alike, so both give the same bits.
 *
 * Method (published techniques, own implementation):
 *   - error-free transformations: Knuth two-sum, Dekker/FMA two-product;
 *     double-double add/mul/div (Dekker 1971; Hida, Li & Bailey 2001);
 *   - table-driven logarithm (P.T.P. Tang, ACM TOMS 16(4), 1990):
 *     x = 2^e m, m r_i = 1 + z with a short r_i, log(1+z) = 2 atanh(z/(2+z));
 *   - table-driven exponential (P.T.P. Tang, ACM TOMS 15(2), 1989):
 *     y log x = n ln2/64 + r, exp = 2^(n/64) (1 + expm1 r).
 * Tables come from nsem_pow_tables.h (gen_pow_tables.py, 200-bit mpmath).
 *
 * Evaluation order (Ziv's strategy, A. Ziv, ACM TOMS 17(3), 1991): a fast
 * phase evaluates y log x and exp with a few double-double steps and Taylor
 * polynomials to about 2^-70 relative, then tests whether every value within
 * the phase's error bound rounds to the same double; only when it does not
 * (about one call in 2^14) does the accurate double-double phase above run.
 * Both phases return the correctly rounded x^y, so the result does not
 * depend on which one ran.
 *
 * Every operation is an explicit fma or a plain IEEE op; compile without FP
 * contraction (nvcc --fmad=false / gcc -ffp-contract=off) so host and device
 * agree bit for bit.
 */
#ifndef NSEM_DDPOW_H
#define NSEM_DDPOW_H

#include <stdint.h>

#ifdef __CUDACC__
#define NSEM_HD __host__ __device__ __forceinline__
#define NSEM_TABLE static __device__ __constant__ const
#define NSEM_TABLE_HOST static const
#else
#include <math.h>
#include <stdint.h>
#include <string.h>
#define NSEM_HD static inline
#define NSEM_TABLE static const
#endif

#ifdef __CUDACC__
/* device copy in constant memory, host copy for host callers */
#define nsem_log_r nsem_log_r_d
#define nsem_log_nlr nsem_log_nlr_d
#define nsem_exp2_64 nsem_exp2_64_d
#include "nsem_pow_tables.h"
#undef nsem_log_r
#undef nsem_log_nlr
#undef nsem_exp2_64
#undef NSEM_POW_TABLES_H
#undef NSEM_TABLE
#define NSEM_TABLE static const
#define nsem_log_r nsem_log_r_h
#define nsem_log_nlr nsem_log_nlr_h
#define nsem_exp2_64 nsem_exp2_64_h
#include "nsem_pow_tables.h"
#undef nsem_log_r
#undef nsem_log_nlr
#undef nsem_exp2_64
#ifdef __CUDA_ARCH__
#define NSEM_LOG_R nsem_log_r_d
#define NSEM_LOG_NLR nsem_log_nlr_d
#define NSEM_EXP2 nsem_exp2_64_d
#else
#define NSEM_LOG_R nsem_log_r_h
#define NSEM_LOG_NLR nsem_log_nlr_h
#define NSEM_EXP2 nsem_exp2_64_h
#endif
#else
#include "nsem_pow_tables.h"
#define NSEM_LOG_R nsem_log_r
#define NSEM_LOG_NLR nsem_log_nlr
#define NSEM_EXP2 nsem_exp2_64
#endif

typedef struct { double h, l; } nsem_dd;

NSEM_HD uint64_t nsem_d2u(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u; memcpy(&u, &x, 8); return u;
#endif
}
NSEM_HD double nsem_u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x; memcpy(&x, &u, 8); return x;
#endif
}

NSEM_HD nsem_dd nsem_two_sum(double a, double b) {
    nsem_dd r;
    r.h = a + b;
    double bb = r.h - a;
    r.l = (a - (r.h - bb)) + (b - bb);
    return r;
}
NSEM_HD nsem_dd nsem_fast_two_sum(double a, double b) {
    nsem_dd r;
    r.h = a + b;
    r.l = b - (r.h - a);
    return r;
}
NSEM_HD nsem_dd nsem_two_prod(double a, double b) {
    nsem_dd r;
    r.h = a * b;
    r.l = fma(a, b, -r.h);
    return r;
}
NSEM_HD nsem_dd nsem_dd_add(nsem_dd a, nsem_dd b) {
    nsem_dd s = nsem_two_sum(a.h, b.h);
    nsem_dd t = nsem_two_sum(a.l, b.l);
    s.l += t.h;
    s = nsem_fast_two_sum(s.h, s.l);
    s.l += t.l;
    return nsem_fast_two_sum(s.h, s.l);
}
NSEM_HD nsem_dd nsem_dd_add_d(nsem_dd a, double b) {
    nsem_dd s = nsem_two_sum(a.h, b);
    s.l += a.l;
    return nsem_fast_two_sum(s.h, s.l);
}
NSEM_HD nsem_dd nsem_dd_mul(nsem_dd a, nsem_dd b) {
    nsem_dd p = nsem_two_prod(a.h, b.h);
    p.l += a.h * b.l + a.l * b.h;
    return nsem_fast_two_sum(p.h, p.l);
}
NSEM_HD nsem_dd nsem_dd_mul_d(nsem_dd a, double b) {
    nsem_dd p = nsem_two_prod(a.h, b);
    p.l += a.l * b;
    return nsem_fast_two_sum(p.h, p.l);
}
/* a / b by long division with three quotient digits */
NSEM_HD nsem_dd nsem_dd_div(nsem_dd a, nsem_dd b) {
    double q1 = a.h / b.h;
    nsem_dd r = nsem_dd_add(a, nsem_dd_mul_d(b, -q1));
    double q2 = r.h / b.h;
    r = nsem_dd_add(r, nsem_dd_mul_d(b, -q2));
    double q3 = r.h / b.h;
    nsem_dd q = nsem_fast_two_sum(q1, q2);
    return nsem_dd_add_d(q, q3);
}

/* log(x) as a double-double, x > 0 finite */
NSEM_HD nsem_dd nsem_log_dd(double x) {
    uint64_t u = nsem_d2u(x);
    int ex = (int)((u >> 52) & 0x7ff);
    int e;
    if (ex == 0) { /* subnormal: renormalise */
        x = x * 18014398509481984.0; /* 2^54 */
        u = nsem_d2u(x);
        ex = (int)((u >> 52) & 0x7ff);
        e = ex - 1023 - 54;
    } else {
        e = ex - 1023;
    }
    double m = nsem_u2d((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
    int i = (int)((m - 0.703125) * 128.0);
    if (i < 0) i = 0;
    if (i > NSEM_LOG_NBIN - 1) i = NSEM_LOG_NBIN - 1;
    const double r = NSEM_LOG_R[i];
    /* z = m r - 1 exactly */
    nsem_dd p = nsem_two_prod(m, r);
    nsem_dd z = nsem_two_sum(p.h - 1.0, p.l);
    /* s = z / (2 + z); log1p(z) = 2 (s + s^3 Q(s^2)) */
    nsem_dd den = nsem_dd_add_d(z, 2.0);
    nsem_dd s = nsem_dd_div(z, den);
    const double s2h = s.h * s.h;
    double q = s2h * (1.0 / 5 + s2h * (1.0 / 7 + s2h * (1.0 / 9 + s2h * (1.0 / 11 + s2h * (1.0 / 13)))));
    nsem_dd third; third.h = NSEM_THIRD_HI; third.l = NSEM_THIRD_LO;
    nsem_dd Q = nsem_dd_add_d(third, q);
    nsem_dd s2 = nsem_dd_mul(s, s);
    nsem_dd s3 = nsem_dd_mul(s2, s);
    nsem_dd l1p = nsem_dd_add(s, nsem_dd_mul(s3, Q));
    l1p.h *= 2.0;
    l1p.l *= 2.0;
    /* e ln2 - log r_i + log1p z */
    const double de = (double)e;
    nsem_dd el = nsem_two_prod(de, NSEM_LN2_MID);
    el.l += de * NSEM_LN2_LO;
    el = nsem_dd_add_d(el, de * NSEM_LN2_HI);
    nsem_dd nl; nl.h = NSEM_LOG_NLR[i][0]; nl.l = NSEM_LOG_NLR[i][1];
    return nsem_dd_add(nsem_dd_add(el, nl), l1p);
}

/* exp(y) for a double-double y, result rounded to double */
NSEM_HD double nsem_exp_dd(nsem_dd y) {
    if (y.h > 709.8) return 1.0 / 0.0;
    if (y.h < -745.2) return 0.0;
    const double nd = rint(y.h * NSEM_INV_LN2_64);
    const long long n = (long long)nd;
    /* r = y - n ln2/64 (ln2/64 split exactly by the power of two) */
    nsem_dd r = nsem_dd_add_d(y, -(nd * (NSEM_LN2_HI / 64)));
    nsem_dd t = nsem_two_prod(nd, NSEM_LN2_MID / 64);
    t.h = -t.h; t.l = -t.l;
    r = nsem_dd_add(r, t);
    r = nsem_dd_add_d(r, -(nd * (NSEM_LN2_LO / 64)));
    /* expm1 r = r + r^2 (1/2 + r (1/6 + r (1/24 + r P(r)))) */
    const double rh = r.h;
    double tail = 1.0 / 120 + rh * (1.0 / 720 + rh * (1.0 / 5040 + rh * (1.0 / 40320 + rh * (1.0 / 362880))));
    nsem_dd c24; c24.h = NSEM_24TH_HI; c24.l = NSEM_24TH_LO;
    nsem_dd c6; c6.h = NSEM_SIXTH_HI; c6.l = NSEM_SIXTH_LO;
    nsem_dd P = nsem_dd_add_d(c24, rh * tail);
    P = nsem_dd_add(c6, nsem_dd_mul(r, P));
    P = nsem_dd_add_d(nsem_dd_mul(r, P), 0.5);
    nsem_dd E = nsem_dd_add(r, nsem_dd_mul(nsem_dd_mul(r, r), P));
    const int j = (int)(n & 63);
    const long long k = (n - j) / 64;
    nsem_dd T; T.h = NSEM_EXP2[j][0]; T.l = NSEM_EXP2[j][1];
    nsem_dd res = nsem_dd_add(T, nsem_dd_mul(T, E));
    /* scale by 2^k (exact for normal results) */
    if (k > -1022 && k < 1023) {
        return res.h * nsem_u2d((uint64_t)(k + 1023) << 52);
    }
    double half = nsem_u2d((uint64_t)((k / 2) + 1023) << 52);
    return (res.h * half) * nsem_u2d((uint64_t)((k - k / 2) + 1023) << 52);
}

/* Fast phase of x^y for normal x > 0 and finite y: x^y = 2^k (hi + lo) with
 * |x^y / 2^k - (hi + lo)| <= *err.  Returns 0 (and nothing else) when x is
 * subnormal or the result leaves the normal range, which the accurate phase
 * handles.
 *
 *   log x = e ln2 - log r_i + log1p z,  z = m r_i - 1 exact, |z| < 2^-7,
 *   log1p z = z - z^2/2 + z^3 (1/3 - z/4 + ... - z^7/10)   (tail < 2^-80),
 *   t = y log x = n ln2/64 + r,  |r| <= ln2/128,
 *   exp t = 2^(n/64) (1 + expm1 r),
 *   expm1 r = r + r^2/2 + r^3 (1/6 + r/24 + ... + r^5/8!)  (tail < 2^-86).
 * z^2 and r^2 are kept exact as products of two doubles (two_prod), the
 * higher terms are plain doubles; the error bound holds the worst-case sum
 * of the truncation and rounding terms with a factor of 4 to spare. */
NSEM_HD int nsem_pow_fast_core(double x, double y, double* hi, double* lo, double* err, int* kk) {
    const uint64_t u = nsem_d2u(x);
    const int ex = (int)((u >> 52) & 0x7ff);
    if (ex == 0) return 0;
    int e = ex - 1023;
    double m = nsem_u2d((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
    int i = (int)((m - 0.703125) * 128.0);
    if (i < 0) i = 0;
    if (i > NSEM_LOG_NBIN - 1) i = NSEM_LOG_NBIN - 1;
    /* z = m r_i - 1: the product is exact as a pair, the subtraction exact
     * (Sterbenz), and |p.h - 1| >= |p.l| unless it is zero */
    const nsem_dd p = nsem_two_prod(m, NSEM_LOG_R[i]);
    const nsem_dd z = nsem_fast_two_sum(p.h - 1.0, p.l);
    const nsem_dd z2 = nsem_two_prod(z.h, z.h);
    double q = -1.0 / 10;
    q = fma(q, z.h, 1.0 / 9);
    q = fma(q, z.h, -1.0 / 8);
    q = fma(q, z.h, 1.0 / 7);
    q = fma(q, z.h, -1.0 / 6);
    q = fma(q, z.h, 1.0 / 5);
    q = fma(q, z.h, -1.0 / 4);
    q = fma(q, z.h, 1.0 / 3);
    const double z3q = (z2.h * z.h) * q;
    const nsem_dd a = nsem_fast_two_sum(z.h, -0.5 * z2.h);
    const double l1p_lo = ((a.l + z.l) - (0.5 * z2.l + z.h * z.l)) + z3q;
    /* e ln2 - log r_i + log1p z; e LN2_HI is exact (LN2_HI has 32 bits) */
    const double de = (double)e;
    const nsem_dd em = nsem_two_prod(de, NSEM_LN2_MID);
    const nsem_dd h1 = nsem_two_sum(de * NSEM_LN2_HI, NSEM_LOG_NLR[i][0]);
    const nsem_dd h2 = nsem_two_sum(h1.h, a.h);
    const double llo = ((((h1.l + h2.l) + NSEM_LOG_NLR[i][1]) + l1p_lo) + em.h) + (em.l + de * NSEM_LN2_LO);
    const nsem_dd L = nsem_fast_two_sum(h2.h, llo);
    /* t = y log x */
    nsem_dd t = nsem_two_prod(L.h, y);
    t.l += L.l * y;
    if (!(fabs(t.h) < 700.0)) return 0;
    /* r = t - n ln2/64 */
    const double nd = rint(t.h * NSEM_INV_LN2_64);
    const long long n = (long long)nd;
    const double rhi = fma(-nd, NSEM_LN2_HI / 64, t.h);
    const nsem_dd c2 = nsem_two_prod(nd, NSEM_LN2_MID / 64);
    const double rlo = (t.l - c2.h) - (c2.l + nd * (NSEM_LN2_LO / 64));
    const nsem_dd r = nsem_two_sum(rhi, rlo);
    /* expm1 r */
    const nsem_dd r2 = nsem_two_prod(r.h, r.h);
    double c = 1.0 / 40320;
    c = fma(c, r.h, 1.0 / 5040);
    c = fma(c, r.h, 1.0 / 720);
    c = fma(c, r.h, 1.0 / 120);
    c = fma(c, r.h, 1.0 / 24);
    c = fma(c, r.h, 1.0 / 6);
    const double r3c = (r2.h * r.h) * c;
    const nsem_dd b = nsem_fast_two_sum(r.h, 0.5 * r2.h);
    const double elo = ((b.l + r.l) + (0.5 * r2.l + r.h * r.l)) + r3c;
    /* 2^(j/64) (1 + expm1 r) */
    const int j = (int)(n & 63);
    const long long k = (n - j) / 64;
    if (!(k > -1022 && k < 1023)) return 0;
    const double Th = NSEM_EXP2[j][0], Tl = NSEM_EXP2[j][1];
    const nsem_dd pe = nsem_two_prod(Th, b.h);
    const nsem_dd h = nsem_fast_two_sum(Th, pe.h);
    const double lo2 = (((h.l + pe.l) + Th * elo) + Tl) + Tl * b.h;
    const nsem_dd res = nsem_fast_two_sum(h.h, lo2);
    *hi = res.h;
    *lo = res.l;
    /* log: 2^-70 + 2^-96 |log x| absolute (worst-case sum of the terms above
     * below 2^-72); exp: 2^-70 relative (below 2^-73 for |t| < 700) */
    *err = ((fabs(y) * (0x1p-70 + 0x1p-96 * fabs(L.h)) + 0x1p-100 * fabs(t.h)) + 0x1p-70) * res.h;
    *kk = (int)k;
    return 1;
}

/* correctly rounded x^y from the fast phase, or 0 when its rounding test
 * cannot decide: every real within err of hi + lo rounds to the same double
 * (rounding is monotonic; lo -/+ 2 err absorbs the rounding of the shifted
 * low parts, which is below 2^-106 hi) */
NSEM_HD int nsem_pow_fast(double x, double y, double* out) {
    double hi, lo, err;
    int k;
    if (!nsem_pow_fast_core(x, y, &hi, &lo, &err, &k)) return 0;
    const double a = hi + (lo - 2.0 * err);
    const double b = hi + (lo + 2.0 * err);
    if (a != b) return 0;
    *out = a * nsem_u2d((uint64_t)(k + 1023) << 52);
    return 1;
}

/* accurate phase, kept out of line on the device: it runs for about one
 * call in 2^14 and would otherwise hold registers in every caller */
#ifdef __CUDACC__
__host__ __device__ __noinline__ static double nsem_pow_accurate(double x, double y)
#else
static double nsem_pow_accurate(double x, double y)
#endif
{
    return nsem_exp_dd(nsem_dd_mul_d(nsem_log_dd(x), y));
}

/* x^y for the equation of state; x > 0 expected.  Non-positive, infinite or
 * NaN arguments give the IEEE pow result for those cases that occur here. */
NSEM_HD double nsem_pow(double x, double y) {
    if (!(x > 0.0) || x == 1.0 / 0.0 || y != y) {
        if (x == 0.0) return (y > 0.0) ? 0.0 : 1.0 / 0.0;
        if (x == 1.0 / 0.0) return (y > 0.0) ? x : 0.0;
        return 0.0 / 0.0;
    }
    if (y == 0.0 || x == 1.0) return 1.0;
    double r;
    if (nsem_pow_fast(x, y, &r)) return r;
    return nsem_pow_accurate(x, y);
}

#endif
