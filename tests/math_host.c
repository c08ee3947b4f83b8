/* Host build of the engine's elementary functions and of its single
 * precision screen (gp_math.cuh), for the accuracy tests: compiled by
 * tests/test_math.py without floating point contraction, it rounds exactly
 * as the device code (the screen's single precision logarithm is the C
 * library's on the host, the fast intrinsic on the device). */
#include <stddef.h>

#include "gp_math.cuh"

void math_host_eval(int fn, size_t n, const double * x, double * y)
{
        size_t i;
        for (i = 0; i < n; i++) {
                if (fn == 2)
                        y[i] = gp_neglog_beyond(x[4 * i], x[4 * i + 1],
                            x[4 * i + 2], x[4 * i + 3]);
                else
                        y[i] = (fn == 0) ? gp_log(x[i]) : gp_exp(x[i]);
        }
}
