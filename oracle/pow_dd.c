/*
 * Host build of the double-double pow (TEST INFRASTRUCTURE: lets the oracle
 * evaluate the equation of state with a correctly rounded pow, to measure
 * how much of the FP64 parity floor comes from the C library's pow rounding).
 */
#include "nsem_oracle.h"
#include "nsem_ddpow.h"

double nsem_oracle_pow_dd(double x, double y) { return nsem_pow(x, y); }

/* the accurate (double-double) phase alone */
double nsem_oracle_pow_dd_accurate(double x, double y) { return nsem_pow_accurate(x, y); }

/* the fast phase's unrounded result 2^k (hi + lo) and its error bound */
int nsem_oracle_pow_fast_core(double x, double y, double* hi, double* lo, double* err, int* k) {
    return nsem_pow_fast_core(x, y, hi, lo, err, k);
}

/* n pseudo-random x (log-uniform in [xlo, xhi]) for one exponent y: counts
 * the calls the fast phase could not round and the calls whose result
 * differs from the accurate phase (must be zero) */
void nsem_oracle_pow_fast_sweep(int64_t n, uint64_t seed, double xlo, double xhi, double y,
                                int64_t* fallbacks, int64_t* mismatches) {
    int64_t fb = 0, mm = 0;
    const double la = log(xlo), lb = log(xhi);
#pragma omp parallel for reduction(+ : fb, mm) schedule(static)
    for (int64_t i = 0; i < n; i++) {
        /* splitmix64 of (seed, i) */
        uint64_t z = seed + (uint64_t)i * 0x9E3779B97F4A7C15ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z = z ^ (z >> 31);
        const double f = (double)(z >> 11) * 0x1p-53;
        const double x = exp(la + (lb - la) * f);
        double r;
        const int ok = nsem_pow_fast(x, y, &r);
        if (!ok) fb++;
        else if (r != nsem_pow_accurate(x, y)) mm++;
    }
    *fallbacks = fb;
    *mismatches = mm;
}
