/*
 * gp_libmf.cuh -- the single precision logarithm and exponential of the
 * DCS evaluation, returning the same floats as the host C library's logf
 * and expf.
 *
 * dcs_evaluate (pumas.c:11243-11347) interpolates its single precision
 * tables with the C library's logf and expf. A backward DEL multiplies the
 * event weight by DCS values (pumas.c:6036-6093), so a one ulp difference
 * of one of these floats moves the weight by 1e-8 to 1e-7 relative.
 *
 * The engine computes them as the double precision gp_log / gp_exp of
 * gp_math.cuh rounded to single precision, then moves the result by one
 * step of its bit pattern where the C library's result differs. The list
 * of those arguments comes from running the C library of the build host on
 * every float of the DCS domains (gen_libmf_tables.c, which writes
 * gp_libmf_tables.h into the build directory):
 *
 *   logf on [2^-8, 1) (q / K) and on [1, 1.5) (ratios of table energies);
 *   expf on (-64, -2] (logarithms of the tabulated DCS values).
 *
 * Outside those domains the functions return the rounded double precision
 * result. The code compiles as C (host, for the tests) and as CUDA.
 */
#ifndef GP_LIBMF_CUH
#define GP_LIBMF_CUH

#include "gp_math.cuh"
#include "gp_libmf_tables.h"

#if defined(__CUDA_ARCH__)
GP_MATH_HD uint32_t gp_libmf_bits(float x) { return __float_as_uint(x); }
GP_MATH_HD float gp_libmf_float(uint32_t u) { return __uint_as_float(u); }
#else
GP_MATH_HD uint32_t gp_libmf_bits(float x)
{
        uint32_t u;
        memcpy(&u, &x, sizeof(u));
        return u;
}
GP_MATH_HD float gp_libmf_float(uint32_t u)
{
        float x;
        memcpy(&x, &u, sizeof(x));
        return x;
}
#endif

/* y moved by the listed step when the argument bits u (u0 <= u, within the
 * table's domain) are listed: entries of one bucket are sorted by their low
 * 12 bits. */
GP_MATH_HD float gp_libmf_fix(float y, uint32_t u, uint32_t u0,
    const uint32_t * off, const uint16_t * fix)
{
        const uint32_t b = (u - u0) >> GP_LIBMF_SHIFT;
        const uint32_t lo = u & 0xFFFu;
        uint32_t i = GP_MATH_LD(off + b);
        const uint32_t end = GP_MATH_LD(off + b + 1);
        for (; i < end; i++) {
                const uint32_t f = GP_MATH_LD(fix + i);
                const uint32_t fl = f & 0xFFFu;
                if (fl < lo) continue;
                if (fl == lo)
                        return gp_libmf_float(gp_libmf_bits(y) +
                            ((f & 0x8000u) ? 1u : 0xFFFFFFFFu));
                break;
        }
        return y;
}

/* logf of the C library on [2^-8, 1.5), correctly rounded elsewhere. */
GP_MATH_HD float gp_libm_logf(float x)
{
        const float y = (float)gp_log((double)x);
        const uint32_t u = gp_libmf_bits(x);
        if (u - GP_LOGF_U0 < GP_LOGF_U1 - GP_LOGF_U0)
                return gp_libmf_fix(y, u, GP_LOGF_U0, gp_LOGF_off,
                    gp_LOGF_fix);
        if (u - GP_LOGF1_U0 < GP_LOGF1_U1 - GP_LOGF1_U0)
                return gp_libmf_fix(y, u, GP_LOGF1_U0, gp_LOGF1_off,
                    gp_LOGF1_fix);
        return y;
}

/* expf of the C library on (-64, -2], correctly rounded elsewhere. */
GP_MATH_HD float gp_libm_expf(float x)
{
        const float y = (float)gp_exp((double)x);
        const uint32_t u = gp_libmf_bits(x);
        if (u - GP_EXPF_U0 < GP_EXPF_U1 - GP_EXPF_U0)
                return gp_libmf_fix(y, u, GP_EXPF_U0, gp_EXPF_off,
                    gp_EXPF_fix);
        return y;
}

#endif
