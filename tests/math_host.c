/* Host build of the engine's elementary functions and of its single
 * precision screen (gp_math.cuh), for the accuracy tests: compiled by
 * tests/test_math.py without floating point contraction, it rounds exactly
 * as the device code (the screen's single precision logarithm is the C
 * library's on the host, the fast intrinsic on the device). */
#include <stddef.h>

#include "gp_libmf.cuh"

/* fn: 0 gp_log, 1 gp_exp, 2 gp_neglog_beyond, 3 gp_libm_logf, 4
 * gp_libm_expf, 5 the C library's logf, 6 its expf (the last four at the
 * single precision value of the argument). */
void math_host_eval(int fn, size_t n, const double * x, double * y)
{
        size_t i;
        for (i = 0; i < n; i++) {
                const float f = (float)x[i];
                if (fn == 3)
                        y[i] = gp_libm_logf(f);
                else if (fn == 4)
                        y[i] = gp_libm_expf(f);
                else if (fn == 5)
                        y[i] = logf(f);
                else if (fn == 6)
                        y[i] = expf(f);
                else if (fn == 2)
                        y[i] = gp_neglog_beyond(x[4 * i], x[4 * i + 1],
                            x[4 * i + 2], x[4 * i + 3]);
                else
                        y[i] = (fn == 0) ? gp_log(x[i]) : gp_exp(x[i]);
        }
}

/* Number of floats with bit patterns in [u0, u1) where gp_libm_logf (fn =
 * 3) or gp_libm_expf (fn = 4) differs from the C library's logf / expf in
 * its bit pattern; the first such argument goes to *first. */
long math_host_libmf_mismatch(int fn, uint32_t u0, uint32_t u1,
    float * first)
{
        long n = 0;
        uint32_t u;
        for (u = u0; u < u1; u++) {
                const float x = gp_libmf_float(u);
                const float a = (fn == 3) ? gp_libm_logf(x) : gp_libm_expf(x);
                const float b = (fn == 3) ? logf(x) : expf(x);
                if (gp_libmf_bits(a) != gp_libmf_bits(b)) {
                        if (n++ == 0) *first = x;
                }
        }
        return n;
}
