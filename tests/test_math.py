"""The engine's table-driven logarithm and exponential (gp_math.cuh).

They replace the CUDA library functions in the transport (fewer double
precision instructions on a GPU whose FP64 rate is 1/64 of its FP32 rate).
The host build of the same code is checked against 40 digit values from
mpmath (below one ulp, equal to glibc in nearly all cases); on the GPU the
device results must equal the host build bit for bit.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pumas_gb300", "csrc")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    lib = str(tmp_path_factory.mktemp("math") / "libmath_host.so")
    subprocess.check_call([
        "gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared",
        "-I" + CSRC, "-o", lib, os.path.join(ROOT, "tests", "math_host.c"),
        "-lm"])
    h = ctypes.CDLL(lib)
    h.math_host_eval.argtypes = [ctypes.c_int, ctypes.c_size_t,
                                 ctypes.c_void_p, ctypes.c_void_p]
    h.math_host_eval.restype = None

    def run(fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        h.math_host_eval(fn, len(x), x.ctypes.data, y.ctypes.data)
        return y
    return run


def arguments(fn, n=4000, seed=3):
    rng = np.random.default_rng(seed)
    if fn == 0:
        return np.concatenate([
            rng.random(n) + 2. ** -53,                      # uniform draws
            1. + (rng.random(n) - 0.5) * 1E-06,              # near 1
            np.ldexp(1. + rng.random(n), rng.integers(-1000, 1000, n)),
            np.array([1., 2., 0.5, 1E-300, 1E+300, 1. - 2. ** -53])])
    return np.concatenate([
        -20. * rng.random(n), (rng.random(n) - 0.5) * 1E-06,
        (rng.random(n) - 0.5) * 1400., np.array([0., 1., -1., 700., -700.])])


@pytest.mark.parametrize("fn", [0, 1])
def test_host_accuracy(host, fn):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    x = arguments(fn)
    y = host(fn, x)
    ref = mpmath.log if fn == 0 else mpmath.exp
    worst = 0.
    for xi, yi in zip(x, y):
        e = ref(mpmath.mpf(float(xi)))
        fe = float(e)
        if fe == 0. or not np.isfinite(fe):
            continue
        ulp = float(np.spacing(abs(fe)))
        worst = max(worst, abs(float(mpmath.mpf(float(yi)) - e)) / ulp)
    assert worst < 0.8, worst
    libm = np.log(x) if fn == 0 else np.exp(x)
    assert np.mean(y == libm) > 0.95


def test_special_arguments(host):
    x = np.array([0., -1., np.inf, np.nan, 5E-324])
    with np.errstate(all="ignore"):
        assert np.array_equal(host(0, x), np.log(x), equal_nan=True)
    x = np.array([710., -750., np.inf, -np.inf, np.nan])
    with np.errstate(all="ignore"):
        assert np.array_equal(host(1, x), np.exp(x), equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("fn", [0, 1])
def test_device_equals_host(host, gpu_physics, fn):
    import pumas_gb300 as pg
    lib = pg.library()
    lib.gpumas_math_eval.argtypes = [ctypes.c_int, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p]
    lib.gpumas_math_eval.restype = ctypes.c_int
    x = arguments(fn, n=100000, seed=9)
    y = np.empty_like(x)
    assert lib.gpumas_math_eval(fn, len(x), x.ctypes.data, y.ctypes.data) == 0
    assert np.array_equal(y, host(fn, x))
