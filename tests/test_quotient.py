"""The division-free quotient of the table lookups (gp_quotient in
pumas_gb300/csrc/gp_device.cuh).

A baked table row stores dx = x[i+1] - x[i] and its correctly rounded
reciprocal; a lookup needs t = (v - x[i]) / dx rounded as the reference's
division (table_interpolate_pchip, pumas.c:4146-4157). The device takes
q0 = a (1 / dx), the exact residual r = a - q0 dx by a fused multiply-add
and t = q0 + r (1 / dx) rounded once (Markstein, IBM J. Res. Dev. 34 (1990)
111). The arithmetic is IEEE binary64 on the host as on the device, so the
identity with the division is checked here, in C, on random operands, hard
divisors (mantissas of trailing and leading ones) and quotients in [0, 1) as
the lookups make them.
"""
import os
import subprocess

import pytest

SOURCE = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t next(void)
{
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
}

static double make(int e, uint64_t m)
{
        const uint64_t b = ((uint64_t)(1023 + e) << 52) |
            (m & ((1ull << 52) - 1));
        double d;
        memcpy(&d, &b, 8);
        return d;
}

int main(void)
{
        long n = 0, bad = 0;
        for (int k = 0; k < 4096; k++) {
                uint64_t m = next();
                if (k & 1) m |= (1ull << 52) - (1ull << (k % 52));
                if (k & 2) m = ((1ull << 52) - 1) - (uint64_t)k;
                const double b = make((int)(next() % 81) - 40, m);
                const double rb = 1. / b;
                for (int j = 0; j < 2000; j++) {
                        double a;
                        if (j & 1)
                                a = (double)(next() >> 11) * 0x1p-53 * b;
                        else
                                a = make((int)(next() % 81) - 40, next());
                        const double q0 = a * rb;
                        const double q = fma(fma(-q0, b, a), rb, q0);
                        n++;
                        if (q != a / b) bad++;
                }
        }
        printf("%ld %ld\n", n, bad);
        return 0;
}
"""


def test_quotient_matches_division(tmp_path):
    src = tmp_path / "quotient.c"
    exe = tmp_path / "quotient"
    src.write_text(SOURCE)
    try:
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off",
                               "-o", str(exe), str(src), "-lm"])
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("no C compiler")
    n, bad = map(int, subprocess.check_output([str(exe)]).split())
    assert n == 4096 * 2000
    assert bad == 0
