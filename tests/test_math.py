"""The engine's table-driven logarithm and exponential, its single
precision screen of thinned candidates (gp_math.cuh), and the single
precision logarithm and exponential of the DCS interpolation, which return
the C library's logf / expf results (gp_libmf.cuh).

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


# Domains of the C library corrections (gen_libmf_tables.c), as float bit
# patterns [u0, u1): logf of q / K, logf of energy ratios, expf of
# logarithms of DCS values.
LIBMF_DOMAINS = [(3, 0x3B800000, 0x3F800000), (3, 0x3F800000, 0x3FC00000),
                 (4, 0xC0000000, 0xC2800000)]


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    from pumas_gb300 import build as engine_build
    engine_build.libmf_tables()
    lib = str(tmp_path_factory.mktemp("math") / "libmath_host.so")
    subprocess.check_call([
        "gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-shared",
        "-I" + CSRC, "-I" + engine_build.BUILD, "-o", lib,
        os.path.join(ROOT, "tests", "math_host.c"), "-lm"])
    h = ctypes.CDLL(lib)
    h.math_host_eval.argtypes = [ctypes.c_int, ctypes.c_size_t,
                                 ctypes.c_void_p, ctypes.c_void_p]
    h.math_host_eval.restype = None
    h.math_host_libmf_mismatch.argtypes = [
        ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
        ctypes.POINTER(ctypes.c_float)]
    h.math_host_libmf_mismatch.restype = ctypes.c_long
    return h


@pytest.fixture(scope="module")
def host(host_lib):
    def run(fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(len(x))
        host_lib.math_host_eval(fn, len(x), x.ctypes.data, y.ctypes.data)
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


def screen_cases(n=20000, seed=5):
    """Quadruples (u, p, q, r) of the thinning screen in its two forms, DEL
    (p = 1: grammage -ln(u) / r against q) and EHS (r = 1: grammage -ln(u) p
    against q), with q placed within 1 % of the boundary -ln(u) p / r, plus
    far cases and arguments outside the screen's range."""
    rng = np.random.default_rng(seed)
    u = np.concatenate([rng.random(n) + 2. ** -53,
                        1. - rng.random(n // 4) * 1E-04,
                        np.full(8, 2. ** -53), np.full(8, 1. - 2. ** -53)])
    m = len(u)
    scale = np.exp(rng.uniform(-30., 30., m))
    delta = np.where(rng.random(m) < 0.8, rng.uniform(-1E-02, 1E-02, m),
                     rng.uniform(-0.9, 5., m))
    L = -np.log(u)
    del_form = rng.random(m) < 0.5
    p = np.where(del_form, 1., scale)
    r = np.where(del_form, scale, 1.)
    q = L * p / r / (1. + delta)
    x = np.stack([u, p, q, r], axis=1)
    bad = np.array([[0.5, 1., 0., 1.], [0.5, 1., -1., 1.],
                    [0.5, 1., 1E-200, 1.], [0.5, 1E+200, 1., 1.],
                    [0.5, 1., np.inf, 1.], [0.5, 1., np.nan, 1.],
                    [1.5, 1., 1E-03, 1.], [1E-300, 1., 1., 1.]])
    return np.ascontiguousarray(np.concatenate([x, bad]))


def screen_exact(host, x):
    """Whether the double precision candidate, computed as the transport
    does with gp_log, is at or beyond q."""
    L = -host(0, x[:, 0])
    dbl = np.where(x[:, 1] == 1., L / x[:, 3], L * x[:, 1])
    return dbl >= x[:, 2]


def test_screen_is_conservative(host):
    """The screen never rules out a candidate that the double precision
    comparison keeps, and rules out nearly every in-range candidate that is
    more than 1 % beyond."""
    x = screen_cases()
    s = host(2, x) == 1.
    exact = screen_exact(host, x)
    assert not np.any(s & ~exact)
    n = len(x) - 8
    L = -np.log(x[:n, 0])
    far = (L * x[:n, 1] >= 1.01 * x[:n, 2] * x[:n, 3]) & (L > 1E-02)
    assert np.mean(s[:n][far]) > 0.999
    assert not np.any(s[n:])


@pytest.mark.gpu
def test_device_screen(host, gpu_physics):
    import pumas_gb300 as pg
    lib = pg.library()
    lib.gpumas_math_eval.argtypes = [ctypes.c_int, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p]
    lib.gpumas_math_eval.restype = ctypes.c_int
    x = screen_cases(n=200000, seed=11)
    y = np.empty(len(x))
    assert lib.gpumas_math_eval(2, len(x), x.ctypes.data, y.ctypes.data) == 0
    s = y == 1.
    assert not np.any(s & ~screen_exact(host, x))
    assert np.mean(s == (host(2, x) == 1.)) > 0.999


@pytest.mark.parametrize("fn,u0,u1", LIBMF_DOMAINS)
def test_libmf_equals_c_library(host_lib, fn, u0, u1):
    """On every float of each DCS domain, the corrected single precision
    logarithm / exponential returns the bit pattern of this host's C
    library logf / expf (the functions the reference calls in dcs_evaluate,
    pumas.c:11279-11343)."""
    first = ctypes.c_float(0.)
    n = host_lib.math_host_libmf_mismatch(fn, u0, u1, ctypes.byref(first))
    assert n == 0, "%d mismatches, first at %r" % (n, first.value)


def libmf_arguments(seed=13, n=400000):
    """Float arguments of the DCS domains: random bit patterns, the first
    and last float of every correction bucket, and a few values outside the
    domains; returned as doubles with the function index."""
    rng = np.random.default_rng(seed)
    out = []
    for fn, u0, u1 in LIBMF_DOMAINS:
        u = np.concatenate([
            rng.integers(u0, u1, n, dtype=np.uint64),
            np.arange(u0, u1, 4096, dtype=np.uint64),
            np.arange(u0 + 4095, u1, 4096, dtype=np.uint64)])
        x = u.astype(np.uint32).view(np.float32).astype(np.float64)
        out.append((fn, x))
    out.append((3, np.array([1E-05, 0.001, 1.5, 3., 1E+06])))
    out.append((4, np.array([-1., -0.5, -70., -100., 0., 1.])))
    return out


def libmf_inside(fn, x):
    """Whether float arguments x lie in one of fn's correction domains."""
    u = x.astype(np.float32).view(np.uint32).astype(np.int64)
    inside = np.zeros(len(x), bool)
    for f, u0, u1 in LIBMF_DOMAINS:
        if f == fn:
            inside |= (u >= u0) & (u < u1)
    return inside


def test_libmf_host_arguments(host):
    """The sampled arguments of the device test give the C library's
    results on the host too (a sanity check of the argument generator)."""
    for fn, x in libmf_arguments(n=20000):
        inside = libmf_inside(fn, x)
        y = host(fn, x)
        ref = host(fn + 2, x)
        assert np.array_equal(y[inside], ref[inside])


@pytest.mark.gpu
def test_device_libmf_equals_c_library(host, gpu_physics):
    """On the device, the single precision logarithm and exponential of the
    DCS interpolation return this host's C library logf / expf results on
    the sampled arguments of the DCS domains, and equal the host build of
    the same code everywhere."""
    import pumas_gb300 as pg
    lib = pg.library()
    lib.gpumas_math_eval.argtypes = [ctypes.c_int, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p]
    lib.gpumas_math_eval.restype = ctypes.c_int
    for fn, x in libmf_arguments():
        y = np.empty_like(x)
        assert lib.gpumas_math_eval(fn, len(x), x.ctypes.data,
                                    y.ctypes.data) == 0
        assert np.array_equal(y, host(fn, x))
        inside = libmf_inside(fn, x)
        assert np.array_equal(y[inside], host(fn + 2, x)[inside])
