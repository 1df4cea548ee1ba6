/*
 * Host build of the double-double pow (TEST INFRASTRUCTURE: lets the oracle
 * evaluate the equation of state with a correctly rounded pow, to measure
 * how much of the FP64 parity floor comes from the C library's pow rounding).
 */
#include "nsem_oracle.h"
#include "nsem_ddpow.h"

double nsem_oracle_pow_dd(double x, double y) { return nsem_pow(x, y); }
