/* Host build of the engine's elementary functions (gp_math.cuh), for the
 * accuracy tests: compiled by tests/test_math.py without floating point
 * contraction, it rounds exactly as the device code. */
#include <stddef.h>

#include "gp_math.cuh"

void math_host_eval(int fn, size_t n, const double * x, double * y)
{
        size_t i;
        for (i = 0; i < n; i++) y[i] = (fn == 0) ? gp_log(x[i]) : gp_exp(x[i]);
}
