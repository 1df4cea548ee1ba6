/* placeholder replaced below */
#include "nsem_oracle.h"
#include <math.h>
double nsem_oracle_pow_dd(double x, double y) { return pow(x, y); }
