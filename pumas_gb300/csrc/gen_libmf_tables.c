/*
 * gen_libmf_tables.c -- writes gp_libmf_tables.h, the corrections that make
 * the engine's single precision logarithm and exponential return the same
 * floats as the host C library's logf and expf.
 *
 * The reference evaluates its single precision DCS tables with the C
 * library's logf and expf (pumas.c:11279, 11320, 11337, 11343). The engine
 * computes these functions as the double precision gp_log / gp_exp of
 * gp_math.cuh rounded to single precision, which is correctly rounded but
 * for rare double roundings. The C library's binary32 routines evaluate a
 * short polynomial in double precision and round it: their results are
 * within one ulp of the correctly rounded ones, and differ from them when
 * the exact value lies close to the midpoint between two floats (about one
 * argument in 1 300 for logf and one in 3 000 for expf).
 *
 * This program runs the host C library on every float of the domains that
 * the DCS evaluation uses and lists the arguments where the two results
 * differ, with the sign of the one ulp step:
 *
 *   logf: x in [2^-8, 1), i.e. q / K from 0.0039 (the tables start at the
 *         physics cutoff, 0.05 by default) to 1 (LOGF), and x in [1, 1.5),
 *         the ratios of consecutive table energies K / K0 and K1 / K0, at
 *         most 1.25 on the reference's energy grids (LOGF1);
 *   expf: x in (-64, -2], the logarithms of the tabulated DCS values (all
 *         the shipped physics have them in [-38, -10]) (EXPF).
 *
 * The list is bucketed by the high bits of the argument: bucket b holds the
 * entries fix[off[b]] .. fix[off[b + 1] - 1], each the low 12 bits of an
 * argument with bit 15 set when the library's result is one step up in the
 * float's bit pattern and clear when it is one step down.
 *
 * pumas_gb300/build.py compiles and runs it on the build host, whose C
 * library is the one the CPU oracles link, and writes the header into the
 * build directory:
 *   gcc -O2 -std=gnu99 -ffp-contract=off -I. gen_libmf_tables.c -o gen -lm
 *   ./gen > gp_libmf_tables.h
 * tests/test_math.py checks the corrected functions against the C library
 * of the host that runs the tests on every float of the three domains, on
 * the host and on the device.
 */
#include <gnu/libc-version.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gp_math.cuh"

#define LOGF_U0 0x3B800000u /* 2^-8 */
#define LOGF_U1 0x3F800000u /* 1 */
#define LOGF1_U0 0x3F800000u /* 1 */
#define LOGF1_U1 0x3FC00000u /* 1.5 */
#define EXPF_U0 0xC0000000u /* -2 */
#define EXPF_U1 0xC2800000u /* -64 */
#define SHIFT 12

static float as_float(uint32_t u)
{
        float f;
        memcpy(&f, &u, 4);
        return f;
}

static uint32_t as_bits(float f)
{
        uint32_t u;
        memcpy(&u, &f, 4);
        return u;
}

static void emit(const char * name, int is_log, uint32_t u0, uint32_t u1)
{
        const uint32_t nb = (u1 - u0) >> SHIFT;
        uint32_t * off = malloc(sizeof(*off) * (nb + 1));
        size_t cap = 1 << 16, n = 0;
        uint16_t * fix = malloc(sizeof(*fix) * cap);
        uint32_t u;
        for (u = u0; u < u1; u++) {
                const uint32_t b = (u - u0) >> SHIFT;
                if (((u - u0) & ((1u << SHIFT) - 1)) == 0) off[b] = n;
                const float x = as_float(u);
                const float lib = is_log ? logf(x) : expf(x);
                const float own = is_log ? (float)gp_log((double)x) :
                                           (float)gp_exp((double)x);
                if (as_bits(lib) == as_bits(own)) continue;
                const int64_t d = (int64_t)as_bits(lib) - as_bits(own);
                if ((d != 1) && (d != -1)) {
                        fprintf(stderr, "%s(%a): results %a and %a are "
                            "more than one step apart\n", name, x, lib, own);
                        exit(1);
                }
                if (n == cap) fix = realloc(fix, sizeof(*fix) * (cap *= 2));
                fix[n++] = (uint16_t)((u & 0xFFF) | ((d > 0) ? 0x8000 : 0));
        }
        off[nb] = n;

        printf("/* %s: %zu corrections over %u buckets. */\n", name, n, nb);
        printf("#define GP_%s_U0 0x%08Xu\n#define GP_%s_U1 0x%08Xu\n", name,
            u0, name, u1);
        printf("GP_MATH_TABLE uint32_t gp_%s_off[%u] = {", name, nb + 1);
        for (u = 0; u <= nb; u++)
                printf("%s%u%s", (u % 10) ? "" : "\n", off[u],
                    (u < nb) ? "," : "");
        printf("};\nGP_MATH_TABLE uint16_t gp_%s_fix[%zu] = {", name,
            n ? n : 1);
        for (u = 0; u < n; u++)
                printf("%s0x%X%s", (u % 12) ? "" : "\n", fix[u],
                    (u + 1 < n) ? "," : "");
        if (n == 0) printf("0");
        printf("};\n\n");
        free(off);
        free(fix);
}

int main(void)
{
        printf("/*\n * gp_libmf_tables.h -- generated by gen_libmf_tables.c "
               "with the C library\n * glibc %s; do not edit.\n *\n"
               " * Corrections from the engine's single precision logarithm "
               "and exponential\n * to the C library's logf and expf, see "
               "gen_libmf_tables.c.\n */\n",
            gnu_get_libc_version());
        printf("#define GP_LIBMF_SHIFT %d\n\n", SHIFT);
        emit("LOGF", 1, LOGF_U0, LOGF_U1);
        emit("LOGF1", 1, LOGF1_U0, LOGF1_U1);
        emit("EXPF", 0, EXPF_U0, EXPF_U1);
        return 0;
}
