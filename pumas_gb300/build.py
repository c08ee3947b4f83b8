"""Build recipe of libgpumas.so, the GB300 transport engine.

The CUDA sources under csrc/ are compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel and linked into
``pumas_gb300/_build/libgpumas.so``, inside the source tree. Host and
device code are compiled without floating point contraction
(``-ffp-contract=off``, ``--fmad=false``): every product and sum is rounded
on its own, as in the reference's C code, so that the transport reproduces
the reference's roundings; fused multiply-adds appear only where the code
asks for one (``fma``), in its own math functions and division steps.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgpumas.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["gp_physics.cu", "gp_transport.cu", "gp_batch.cu", "gp_errors.cu",
           "gp_tabulate.cu"]
# Per file flags (none at present).
FILE_FLAGS = {}
HEADERS = ["gp_internal.h", "gp_device.cuh", "gp_math.cuh",
           "gp_math_tables.h", "gp_models.cuh", "gp_io.cuh", "gp_context.h",
           "gp_libmf.cuh", "gen_libmf_tables.c"]
# Generated into the build directory by gen_libmf_tables.c from the build
# host's C library (the one the CPU oracles link).
LIBMF_TABLES = os.path.join(BUILD, "gp_libmf_tables.h")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
    "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
    "-ffp-contract=off",
    "-I" + INCLUDE, "-I" + CSRC, "-I" + BUILD,
]


def _nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.exists(p) or p == "nvcc"):
            return p
    return "nvcc"


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in _sources() + HEADERS] + [
        os.path.join(INCLUDE, h) for h in ("gpumas.h", "gpumas_geometry.h")
    ] + [LIBMF_TABLES]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def libmf_tables(force=False):
    """Write gp_libmf_tables.h: the arguments where the build host's C
    library logf / expf differ from the engine's correctly rounded single
    precision results, over the domains of the DCS evaluation."""
    src = os.path.join(CSRC, "gen_libmf_tables.c")
    if (not force and os.path.exists(LIBMF_TABLES) and
            os.path.getmtime(LIBMF_TABLES) >= max(
                os.path.getmtime(src),
                os.path.getmtime(os.path.join(CSRC, "gp_math.cuh")),
                os.path.getmtime(os.path.join(CSRC, "gp_math_tables.h")))):
        return LIBMF_TABLES
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "gen_libmf_tables")
    subprocess.check_call([
        os.environ.get("CC", "gcc"), "-O2", "-std=gnu99",
        "-ffp-contract=off", "-I" + CSRC, "-o", exe, src, "-lm"])
    tmp = LIBMF_TABLES + ".tmp"
    with open(tmp, "w") as f:
        subprocess.check_call([exe], stdout=f)
    os.replace(tmp, LIBMF_TABLES)
    return LIBMF_TABLES


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link libgpumas.so if any source changed."""
    libmf_tables()
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + FILE_FLAGS.get(src, []) + list(
            extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=len(_sources())) as pool:
        objs = list(pool.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
           "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
