"""Build recipe of libgpumas.so, the GB300 transport engine.

The CUDA sources under csrc/ are compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel and linked into
``pumas_gb300/_build/libgpumas.so``, inside the source tree. Host code is
compiled without floating point contraction so that constants evaluated on
the host match the reference's on every host architecture.
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

SOURCES = ["gp_physics.cu", "gp_transport.cu", "gp_batch.cu"]
HEADERS = ["gp_internal.h", "gp_device.cuh", "gp_math.cuh",
           "gp_math_tables.h", "gp_models.cuh", "gp_io.cuh", "gp_context.h"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
    "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I" + INCLUDE, "-I" + CSRC,
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
        os.path.join(INCLUDE, h) for h in ("gpumas.h", "gpumas_geometry.h")]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link libgpumas.so if any source changed."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + list(extra_flags) + [
            "-c", os.path.join(CSRC, src), "-o", obj]
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
