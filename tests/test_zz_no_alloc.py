"""The allocation free transport entry point (GPU).

Some callers cannot allocate device memory while they transport -- a host
whose allocator owns the GPU memory, a plugin whose framework forbids
allocation on its hot path. gpumas_context_transport_device_static serves
them: its slot pool is a static device array of the library instead of a
cudaMalloc'ed one, reserved on a device when a physics is loaded there.
This checks, through the C ABI, that it gives the same results as
gpumas_context_transport_device, bit for bit, on two calls in a row (the
second call reuses the array the first one left behind) and with the
default (largest) pool, and that pool sizes above the static maximum or not
a multiple of 128 are refused.

Collected last on purpose (file name), so that a run stopping at the first
failure has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1E-09


def _columns(torch, states):
    dev = torch.device("cuda", 0)
    cols = {}
    for f in ("charge", "energy", "distance", "grammage", "time", "weight"):
        cols[f] = torch.from_numpy(np.ascontiguousarray(states[f])).to(dev)
    for k in range(3):
        cols["p%d" % k] = torch.from_numpy(
            np.ascontiguousarray(states["position"][:, k])).to(dev)
        cols["d%d" % k] = torch.from_numpy(
            np.ascontiguousarray(states["direction"][:, k])).to(dev)
    cols["decayed"] = torch.from_numpy(
        np.ascontiguousarray(states["decayed"])).to(dev)
    import pumas_gb300 as pg
    cols["result"] = torch.zeros((len(states), pg.RESULT_DTYPE.itemsize),
                                 dtype=torch.uint8,
                                 device=dev)
    return cols


def _soa(pg, cols):
    c = pg._Soa()
    for f in ("charge", "energy", "distance", "grammage", "time", "weight",
              "decayed"):
        setattr(c, f, cols[f].data_ptr())
    for k in range(3):
        c.position[k] = cols["p%d" % k].data_ptr()
        c.direction[k] = cols["d%d" % k].data_ptr()
    c.result = cols["result"].data_ptr()
    return c


def _host(pg, cols):
    out = {k: v.cpu().numpy() for k, v in cols.items() if k != "result"}
    out["result"] = np.frombuffer(cols["result"].cpu().numpy().tobytes(),
                                  dtype=pg.RESULT_DTYPE)
    return out


def test_static_pool_matches_device_entry_point(gpu_physics):
    torch = pytest.importorskip("torch")
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W

    lib = pg.library()
    fn = lib.gpumas_context_transport_device_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(pg._Context), ctypes.c_size_t,
                   ctypes.POINTER(pg._Soa), ctypes.c_uint64, ctypes.c_int,
                   ctypes.c_void_p]

    ctx = pg.Context(gpu_physics)
    W.rock_slab_config(ctx)
    ctx.seed = 17
    ctx.set_geometry(W.rock_slab_geometry(gpu_physics))
    ctx.tuning(engine=pg.ENGINE_POOL, pool_slots=4096, max_inner=2)

    n = 6000
    for call, slots in enumerate((2048, 2048, 0)):
        first = 1000 + call * n
        s0 = W.rock_slab(n, seed=17, first_event=first)
        a_cols = _columns(torch, s0)
        b_cols = _columns(torch, s0)
        rc = ctx.transport_device(n, {
            "charge": a_cols["charge"].data_ptr(),
            "energy": a_cols["energy"].data_ptr(),
            "distance": a_cols["distance"].data_ptr(),
            "grammage": a_cols["grammage"].data_ptr(),
            "time": a_cols["time"].data_ptr(),
            "weight": a_cols["weight"].data_ptr(),
            "decayed": a_cols["decayed"].data_ptr(),
            "position": [a_cols["p%d" % k].data_ptr() for k in range(3)],
            "direction": [a_cols["d%d" % k].data_ptr() for k in range(3)],
            "result": a_cols["result"].data_ptr()}, first)
        assert rc == 0
        torch.cuda.synchronize()
        soa = _soa(pg, b_cols)
        rc = fn(ctx._ptr, n, ctypes.byref(soa), first, slots, None)
        assert rc == 0
        torch.cuda.synchronize()
        a, b = _host(pg, a_cols), _host(pg, b_cols)
        for k in a:
            if k == "result":
                continue
            x, y = a[k], b[k]
            assert np.all(np.abs(x - y) <= RTOL * np.maximum(np.abs(x), 1.)), k
            # The same kernels run the same events: bit for bit.
            assert x.tobytes() == y.tobytes(), k
        ra, rb = a["result"], b["result"]
        for f in ("event", "medium_in", "medium_out", "status", "steps",
                  "draws"):
            assert np.array_equal(ra[f], rb[f]), f
        assert np.all(rb["status"] == 0)

    # Pool sizes above the static maximum, or not a multiple of 128, are
    # refused.
    soa = _soa(pg, _columns(torch, W.rock_slab(128, seed=1)))
    for slots in (2 * pg_static_slots(), pg_static_slots() + 128, 200, -128):
        assert fn(ctx._ptr, 128, ctypes.byref(soa), 0, slots,
                  None) == pg.RETURN_VALUE_ERROR


def pg_static_slots():
    import os
    import re
    from conftest import ROOT
    text = open(os.path.join(ROOT, "include", "gpumas.h")).read()
    return int(re.search(r"#define GPUMAS_STATIC_SLOTS (\d+)", text).group(1))


def test_static_pool_runs_locals(gpu_physics):
    """Media with local properties through the static pool: every event as
    on the one thread per event kernel, bit for bit."""
    torch = pytest.importorskip("torch")
    import pumas_gb300 as pg
    from cases import CASES, make_states
    from conftest import gpu_context, gpu_geometry

    lib = pg.library()
    fn = lib.gpumas_context_transport_device_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(pg._Context), ctypes.c_size_t,
                   ctypes.POINTER(pg._Soa), ctypes.c_uint64, ctypes.c_int,
                   ctypes.c_void_p]
    case = CASES["atmosphere_forward"]
    geo = gpu_geometry(gpu_physics, case["geometry"])
    ctx = gpu_context(gpu_physics, case["config"], case["seed"], geo)
    s0 = make_states("atmosphere_forward", n=300, first_event=11)
    ctx.tuning(engine=pg.ENGINE_PLAIN)
    a, ra = ctx.transport(s0, 11)
    ctx.tuning(engine=pg.ENGINE_POOL, max_inner=2)
    cols = _columns(torch, s0)
    soa = _soa(pg, cols)
    assert fn(ctx._ptr, len(s0), ctypes.byref(soa), 11, 2048, None) == 0
    torch.cuda.synchronize()
    b = _host(pg, cols)
    assert a["energy"].tobytes() == b["energy"].tobytes()
    assert a["time"].tobytes() == b["time"].tobytes()
    assert a["position"][:, 2].tobytes() == b["p2"].tobytes()
    assert a["direction"][:, 0].tobytes() == b["d0"].tobytes()
    assert ra.tobytes() == b["result"].tobytes()
