"""Media with local properties (struct gpumas_locals): density profiles and
magnetic fields, the device form of the reference's `pumas_locals_cb`
(pumas.h:324-349, transport_set_locals pumas.c:5528-5552, the magnetic
steps of pumas.c:6352-6382, 6833-6911).

Parity with the reference runs through the golden cases with locals of
tests/cases.py in test_gpu_parity.py: the stepping cases atmosphere_* and
iron_field, and the closed form CSDA deflection (transport_csda_deflect,
pumas.c:4968-5171) of rock_csda_field*, water_csda_field_backward. This
file covers the descriptor's layout, its checks and the entry points that
do not take locals.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from cases import AIR_LOCALS, CASES
from conftest import gpu_context, gpu_geometry

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

LAYOUT_C = r"""
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include "gpumas_geometry.h"
int main(void)
{
        printf("%zu %zu %zu %zu %zu\n", sizeof(struct gpumas_locals),
            offsetof(struct gpumas_locals, magnet),
            offsetof(struct gpumas_locals, lambda),
            sizeof(struct gpumas_geometry),
            offsetof(struct gpumas_geometry, locals));
        return 0;
}
"""


def test_layout_of_mirrors(tmp_path):
    """The ctypes mirrors (product and oracle) have the C layout."""
    import oracle
    import pumas_gb300 as pg
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C)
    exe = str(tmp_path / "layout")
    subprocess.check_call(["gcc", "-std=c99", "-I" + os.path.join(
        ROOT, "include"), "-o", exe, str(src), "-lm"])
    c = [int(v) for v in subprocess.check_output([exe]).split()]
    for L, G in ((pg._Locals, pg._Geometry), (oracle.Locals,
                                             oracle.Geometry)):
        assert ctypes.sizeof(L) == c[0]
        assert L.magnet.offset == c[1]
        assert L.lambda_.offset == c[2]
        assert ctypes.sizeof(G) == c[3]
        assert G.locals.offset == c[4]


def _atmosphere(physics, **changes):
    spec = dict(CASES["atmosphere_forward"]["geometry"])
    air = dict(AIR_LOCALS, **changes)
    spec["locals"] = [dict(), air]
    return gpu_geometry(physics, spec)


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [dict(model=7), dict(lambda_=0.),
                                 dict(rho0=-1.), dict(eps=0.),
                                 dict(magnet=(np.inf, 0., 0.))])
def test_bad_locals_are_refused(gpu_physics, bad):
    import pumas_gb300 as pg
    ctx = pg.Context(gpu_physics)
    with pytest.raises(pg.PumasError) as e:
        ctx.set_geometry(_atmosphere(gpu_physics, **bad))
    assert e.value.code == pg.RETURN_VALUE_ERROR


@pytest.mark.gpu
def test_pool_entry_points_refuse_locals(gpu_physics):
    """The slot pool engine and the static entry point run uniform media
    only; a context with locals runs through gpumas_context_transport."""
    import pumas_gb300 as pg
    case = CASES["atmosphere_forward"]
    geo = gpu_geometry(gpu_physics, case["geometry"])
    ctx = gpu_context(gpu_physics, case["config"], case["seed"], geo)
    eng = pg.Engine(gpu_physics, pool_slots=4096)
    from cases import make_states
    s0 = make_states("atmosphere_forward", n=8)
    with pytest.raises(pg.PumasError) as e:
        eng.submit_host(ctx, s0)
    assert e.value.code == pg.RETURN_VALUE_ERROR
    lib = pg.library()
    fn = lib.gpumas_context_transport_device_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(pg._Context), ctypes.c_size_t,
                   ctypes.POINTER(pg._Soa), ctypes.c_uint64, ctypes.c_int,
                   ctypes.c_void_p]
    soa = pg._Soa()
    assert fn(ctx._ptr, 8, ctypes.byref(soa), 0, 0, None) == \
        pg.RETURN_VALUE_ERROR

    # A pool tuning does not move a context with locals off its kernel.
    a, ra = ctx.transport(s0)
    ctx.tuning(engine=pg.ENGINE_POOL, pool_slots=4096, max_inner=2)
    b, rb = ctx.transport(s0)
    assert ctx.stats()["launches"] == 1
    assert np.array_equal(a, b) and np.array_equal(ra, rb)
