/*
 * gp_math.cuh -- double precision elementary functions of the engine.
 *
 * GB300 executes double precision arithmetic at 1/64 of its single
 * precision rate, and the transport spends a large share of its double
 * precision instructions in logarithms (three to four per step: the
 * sampling of DEL and EHS candidates and of the multiple scattering angle,
 * Box-Muller pairs). This file holds a logarithm that needs fewer double
 * precision instructions than a general purpose one, with the same
 * accuracy class (below one ulp).
 *
 * gp_log follows the table-driven method of P. T. P. Tang, "Table-driven
 * implementation of the logarithm function in IEEE floating-point
 * arithmetic", ACM TOMS 16 (1990) 378-400, with a reduction by a short
 * reciprocal instead of a division:
 *
 *   x = 2^k m, 1 <= m < 2;  j = round(128 (m - 1));  F_j = 1 + j / 128
 *   c_j = 1 / F_j rounded to 10 bits, so that r = m c_j - 1 is exact in
 *         one fused multiply-add and |r| < 2^-7.5;
 *   ln x = k ln 2 - ln c_j + ln(1 + r),
 *
 * ln 2 and -ln c_j are pairs of doubles (gp_math_tables.h, generated with
 * 60 digit arithmetic), ln(1 + r) is its Taylor series to r^8 (truncation
 * below 2^-70 r). Non positive, subnormal and non finite arguments go to
 * the library logarithm.
 *
 * The code compiles as C (host) and as CUDA (device): the host build is
 * used by the accuracy tests, whose results hold for the device since both
 * use IEEE fused multiply-adds and roundings.
 */
#ifndef GP_MATH_CUH
#define GP_MATH_CUH

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GP_MATH_HD __host__ __device__ __forceinline__
#ifdef __CUDA_ARCH__
/* Device copy of the tables: global memory through the L1 cache (lanes
 * index different rows, which constant memory would serialise). */
#define GP_MATH_TABLE static __device__ const
#else
#define GP_MATH_TABLE static const
#endif
#else
#define GP_MATH_HD static inline
#define GP_MATH_TABLE static const
#endif

/* Products, sums and differences are written with round-to-nearest
 * intrinsics on the device, so that the compiler never fuses them into
 * multiply-adds: the error-free transformations below need the separate
 * roundings, and every inlined copy of a function must round alike. The
 * host build is compiled without contraction (-ffp-contract=off). */
#if defined(__CUDA_ARCH__)
#include "gp_math_tables.h"
#define GP_MATH_LD(p) __ldg(p)
#define GP_MM(a, b) __dmul_rn((a), (b))
#define GP_MA(a, b) __dadd_rn((a), (b))
#define GP_MS(a, b) __dsub_rn((a), (b))
GP_MATH_HD long long gp_math_bits(double x) { return __double_as_longlong(x); }
GP_MATH_HD double gp_math_double(long long b) { return __longlong_as_double(b); }
#else
#include "gp_math_tables.h"
#define GP_MATH_LD(p) (*(p))
#define GP_MM(a, b) ((a) * (b))
#define GP_MA(a, b) ((a) + (b))
#define GP_MS(a, b) ((a) - (b))
GP_MATH_HD long long gp_math_bits(double x)
{
        long long b;
        memcpy(&b, &x, sizeof(b));
        return b;
}
GP_MATH_HD double gp_math_double(long long b)
{
        double x;
        memcpy(&x, &b, sizeof(x));
        return x;
}
#endif

/* Natural logarithm, below one ulp of error (see the file comment). */
GP_MATH_HD double gp_log(double x)
{
        const unsigned long long ub = (unsigned long long)gp_math_bits(x);
        /* Positive normal finite arguments only; the rest (zero,
         * subnormal, negative, infinite, NaN) to the library. */
        if (ub - 0x0010000000000000ull >= 0x7FE0000000000000ull)
                return log(x);
        const int k = (int)(ub >> 52) - 1023;
        const unsigned long long mb = ub & 0x000FFFFFFFFFFFFFull;
        const int j = (int)((mb + (1ull << 44)) >> 45);
        const double m = gp_math_double(
            (long long)(mb | 0x3FF0000000000000ull));
        const double * t = gp_log_table[j];
        const double r = fma(m, GP_MATH_LD(t), -1.0);
        double q = -0.125;
        q = fma(q, r, 0.14285714285714285);
        q = fma(q, r, -0.16666666666666666);
        q = fma(q, r, 0.2);
        q = fma(q, r, -0.25);
        q = fma(q, r, 0.3333333333333333);
        q = fma(q, r, -0.5);
        const double p = GP_MM(GP_MM(r, r), q);
        /* k ln 2 - ln c_j as hi + e exactly: k LN2_HI is exact and, for
         * k != 0, not smaller than -ln c_j, so that the rounding error e of
         * their sum is exact (Fast2Sum). */
        const double kd = (double)k;
        const double a = GP_MM(kd, GP_LN2_HI);
        const double th = GP_MATH_LD(t + 1);
        const double hi = GP_MA(a, th);
        const double e = GP_MA(GP_MS(a, hi), th);
        const double lo = GP_MA(
            GP_MA(fma(kd, GP_LN2_LO, GP_MATH_LD(t + 2)), e), p);
        return GP_MA(hi, GP_MA(r, lo));
}

/* Exponential, below one ulp of error: the table-driven method of
 * P. T. P. Tang, "Table-driven implementation of the exponential function
 * in IEEE floating-point arithmetic", ACM TOMS 15 (1989) 144-157:
 *
 *   x = (32 m + j) ln 2 / 32 + r, |r| <= ln 2 / 64;
 *   exp x = 2^m 2^(j/32) exp r,
 *
 * with 2^(j/32) as pairs of doubles and exp r - 1 as its Taylor series to
 * r^6 (truncation below 2^-60 r). Arguments outside [-700, 700] and NaN go
 * to the library exponential. */
GP_MATH_HD double gp_exp(double x)
{
        if (!(fabs(x) <= 700.)) return exp(x);
        /* N = round(32 x / ln 2), through the rounding of a large shift. */
        const double shift = 0x1.8p52;
        const double t = fma(x, GP_INV_L32, shift);
        const long long n = gp_math_bits(t) - gp_math_bits(shift);
        const double nd = GP_MS(t, shift);
        const double r = fma(-nd, GP_L32_LO, fma(-nd, GP_L32_HI, x));
        double q = 1.3888888888888889e-03;
        q = fma(q, r, 8.3333333333333332e-03);
        q = fma(q, r, 4.1666666666666664e-02);
        q = fma(q, r, 1.6666666666666666e-01);
        q = fma(q, r, 0.5);
        const double p = fma(GP_MM(r, r), q, r);
        const int j = (int)(n & 31);
        const long long m = n >> 5;
        const double * s2 = gp_exp_table[j];
        const double sh = GP_MATH_LD(s2), sl = GP_MATH_LD(s2 + 1);
        const double v = GP_MA(sh, fma(sh, p, GP_MM(sl, GP_MA(1., p))));
        /* Scale by 2^m in two steps, so that intermediate powers of two
         * stay normal over the whole argument range. */
        const long long m1 = m >> 1, m2 = m - m1;
        const double f1 = gp_math_double((m1 + 1023) << 52);
        const double f2 = gp_math_double((m2 + 1023) << 52);
        return GP_MM(GP_MM(v, f1), f2);
}

/* x rounded toward zero to single precision by integer operations on its
 * bits, for 2^-100 <= x <= 2^100; 0 (no value) outside that range, for
 * negative x and for non finite x. The conversion instructions of the
 * GPU run on its double precision pipe; these shifts do not. */
GP_MATH_HD int gp_math_trunc_float(double x, float * f)
{
        const unsigned long long b = (unsigned long long)gp_math_bits(x);
        /* Biased exponents 923 to 1123, sign bit clear. */
        if ((b >> 52) - 923ull > 200ull) return 0;
        const uint32_t fb = (uint32_t)((b >> 29) - (896ull << 23));
#if defined(__CUDA_ARCH__)
        *f = __uint_as_float(fb);
#else
        memcpy(f, &fb, sizeof(*f));
#endif
        return 1;
}

/* Single precision screen of a thinned interaction candidate: returns 1
 * only when -ln(u) p >= q r (1 + 9.9e-4) holds for the exact values, so
 * that a candidate grammage computed in double precision, -gp_log(u) p or
 * -gp_log(u) / (1 / p), with its errors below 2^-51 relative, is certainly
 * at or beyond q r. Returns 0 when that is not sure, or when an argument
 * is outside [2^-100, 2^100]: the caller then computes the candidate in
 * double precision. The decision is the same as the double precision one
 * whenever it returns 1, so that results do not change.
 *
 * Bounds: each argument truncated to single precision is low by less than
 * 2^-23 relative; the single precision logarithm of u (u in (0, 1]) has an
 * error below 1.3e-5 absolute for u < 0.5 (3 ulp of at most 36.8) and
 * below 4e-7 absolute above; the truncation of u raises -ln by less than
 * 1.2e-7. The lower bound Lf (1 - 1e-4) - 1e-4 covers all three; the
 * factor 1.001 covers the truncation of q and r and four single precision
 * roundings. */
GP_MATH_HD int gp_neglog_beyond(double u, double p, double q, double r)
{
        float uf, pf, qf, rf;
        if (!gp_math_trunc_float(u, &uf) || !gp_math_trunc_float(p, &pf) ||
            !gp_math_trunc_float(q, &qf) || !gp_math_trunc_float(r, &rf))
                return 0;
        if (uf > 1.f) return 0;
#if defined(__CUDA_ARCH__)
        const float L = -__logf(uf);
#else
        const float L = -logf(uf);
#endif
        const float low = L * 0.9999f - 1e-4f;
        if (!(low > 0.f)) return 0;
        return (low * pf >= (qf * rf) * 1.001f) ? 1 : 0;
}

#endif
