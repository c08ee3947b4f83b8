"""The frame recorder (pumas_recorder, pumas.h:378-458) on the GPU engine.

The fixtures tests/golden/frames_*.npz hold the frames recorded by the
unmodified reference's own recorder (tests/golden/make_golden.py frames).
Recording must not change the transport; the GPU recorder must produce the
same frames: same number per event, same event flags and media, states
within the parity tolerance.
"""
import glob
import os

import numpy as np
import pytest

from cases import CASES
from conftest import GOLDEN, compare, gpu_context, gpu_geometry

FILES = sorted(glob.glob(os.path.join(GOLDEN, "frames_*.npz")))


def case_of(path):
    base = os.path.basename(path)[len("frames_"):-len(".npz")]
    name, period = base.rsplit("_p", 1)
    return name, int(period)


@pytest.mark.parametrize("path", FILES, ids=lambda p: case_of(p)[0])
def test_reference_frames_are_consistent(path):
    """Recording does not change the reference's transport, and the frames
    start with PUMAS_EVENT_START and end with PUMAS_EVENT_STOP."""
    name, period = case_of(path)
    rec = np.load(path)
    gold = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = len(rec["initial"])
    assert np.array_equal(rec["initial"], gold["initial"][:n])
    assert rec["final"].tobytes() == gold["final"][:n].tobytes()
    frames, length = rec["frames"], rec["length"]
    start, stop = 4096, 8192
    for k in range(n):
        assert length[k] >= 1
        assert frames[k, 0]["event"] & start
        if length[k] <= frames.shape[1]:
            last = frames[k, length[k] - 1]
            assert last["event"] & stop
            assert last["state"].tobytes() == rec["final"][k].tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=lambda p: case_of(p)[0])
def test_gpu_frames_match_reference(gpu_physics, path):
    name, period = case_of(path)
    rec = np.load(path)
    case = CASES[name]
    geo = gpu_geometry(gpu_physics, case["geometry"])
    ctx = gpu_context(gpu_physics, case["config"], case["seed"], geo)
    s0 = rec["initial"]
    max_frames = rec["frames"].shape[1]
    s, r, frames, length = ctx.transport_record(s0, 0, period, max_frames)
    # The transported states are those of a transport without recording.
    s2, r2 = ctx.transport(s0, 0)
    assert s.tobytes() == s2.tobytes() and r.tobytes() == r2.tobytes()
    _, close = compare(s, r, rec["final"], rec["results"], 1E-09)
    good = 0
    for k in np.nonzero(close)[0]:
        m = min(int(length[k]), max_frames)
        if length[k] != rec["length"][k]:
            continue
        a, b = frames[k, :m], rec["frames"][k, :m]
        if not (np.array_equal(a["event"], b["event"]) and
                np.array_equal(a["medium"], b["medium"])):
            continue
        sa, sb = a["state"], b["state"]
        ok = True
        for f in ("energy", "distance", "grammage", "time"):
            ok &= np.all(np.abs(sa[f] - sb[f]) <=
                         1E-09 * np.maximum(np.abs(sb[f]), 1.))
        for f in ("position", "direction"):
            ok &= np.all(np.abs(sa[f] - sb[f]) <= 1E-09 * np.maximum(
                np.abs(sb[f]).max(), 1.))
        ok &= np.all(np.abs(sa["weight"] - sb["weight"]) <=
                     1E-09 * np.abs(sb["weight"]))
        good += int(ok)
    n = len(s0)
    assert good >= n - max(1, n // 20), "%d / %d events" % (good, n)
