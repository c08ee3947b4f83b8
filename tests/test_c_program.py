"""A C99 program built against include/gpumas.h (tests/straight_gpumas.c),
shaped like the reference's examples/pumas/straight.c:133-179.

CPU: it compiles with gcc -std=c99 -Wall against the header alone and links
against libgpumas.so. GPU: it runs, and its final states match the C
restatement oracle on the same initial states within 1e-9.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, compare

SOURCE = os.path.join(ROOT, "tests", "straight_gpumas.c")


def build_program(tmp):
    from pumas_gb300 import build
    lib = build.build()
    exe = os.path.join(str(tmp), "straight_gpumas")
    cuda_lib = "/usr/local/cuda/lib64"
    subprocess.check_call([
        os.environ.get("CC", "gcc"), "-std=c99", "-Wall", "-Werror", "-O2",
        "-I" + os.path.join(ROOT, "include"), "-o", exe, SOURCE,
        "-L" + os.path.dirname(lib), "-lgpumas",
        "-Wl,-rpath," + os.path.dirname(lib), "-L" + cuda_lib,
        "-Wl,-rpath," + cuda_lib, "-lm"])
    return exe


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no gcc")
def test_c_program_builds(tmp_path):
    exe = build_program(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_c_program_matches_oracle(tmp_path, port):
    import oracle
    import pumas_gb300 as pg
    exe = build_program(tmp_path)
    dump = tmp_path / "muon.pumas"
    dump.write_bytes(pg.default_dump())
    out = tmp_path / "out.bin"
    n = 4000
    args = [exe, str(dump), str(out), "300", "30", "1", "1000", str(n)]
    run = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    assert run.stdout.startswith("mean weight")
    raw = out.read_bytes()
    ns, nr = pg.STATE_DTYPE.itemsize, pg.RESULT_DTYPE.itemsize
    assert len(raw) == n * (2 * ns + nr)
    s0 = np.frombuffer(raw[:n * ns], dtype=pg.STATE_DTYPE)
    s1 = np.frombuffer(raw[n * ns:2 * n * ns], dtype=pg.STATE_DTYPE)
    r1 = np.frombuffer(raw[2 * n * ns:], dtype=pg.RESULT_DTYPE)
    assert np.all(r1["status"] == 0)
    rock = port.material_index("StandardRock")
    geo = oracle.make_geometry(0, [(rock, 0.)], uniform_medium=0)
    cfg = oracle.Config(energy_loss=2, decay=0, direction=1, scattering=-1,
                        event=2, limit_distance=300., accuracy=1E-02,
                        seed=20240607)
    s2, r2 = port.transport(cfg, geo, s0, 0, port.max_threads())
    _, close = compare(s1, r1, s2, r2, 1E-09)
    assert close.mean() >= 0.999, "%d / %d outside 1e-9" % (
        (~close).sum(), n)
