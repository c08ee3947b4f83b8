"""Media with local properties (struct gpumas_locals): density profiles and
magnetic fields, the device form of the reference's `pumas_locals_cb`
(pumas.h:324-349, transport_set_locals pumas.c:5528-5552, the magnetic
steps of pumas.c:6352-6382, 6833-6911).

Parity with the reference runs through the golden cases with locals of
tests/cases.py in test_gpu_parity.py: the stepping cases atmosphere_* and
iron_field, and the closed form CSDA deflection (transport_csda_deflect,
pumas.c:4968-5171) of rock_csda_field*, water_csda_field_backward. This
file covers the descriptor's layout, its checks, and the slot pool engine
against the one thread per event kernel on media with locals.
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
@pytest.mark.parametrize("name", ["atmosphere_forward", "atmosphere_backward",
                                  "iron_field"])
def test_pool_engine_runs_locals(gpu_physics, name):
    """Media with local properties also run on the slot pool engine: the
    context's transport with the pool tuning, and the engine's job queue
    with a job of uniform media beside, give every event of the one thread
    per event kernel bit for bit."""
    import pumas_gb300 as pg
    from cases import make_states
    case = CASES[name]
    geo = gpu_geometry(gpu_physics, case["geometry"])
    ctx = gpu_context(gpu_physics, case["config"], case["seed"], geo)
    s0 = make_states(name, n=400, first_event=3)
    ctx.tuning(engine=pg.ENGINE_PLAIN)
    a, ra = ctx.transport(s0, 3)
    assert ctx.stats()["launches"] == 1
    ctx.tuning(engine=pg.ENGINE_POOL, pool_slots=4096, max_inner=2,
               batch=4)
    b, rb = ctx.transport(s0, 3)
    assert ctx.stats()["launches"] > 1
    assert a.tobytes() == b.tobytes()
    assert ra.tobytes() == rb.tobytes()

    rock = CASES["rock_slab"]
    ctx2 = gpu_context(gpu_physics, rock["config"], rock["seed"],
                       gpu_geometry(gpu_physics, rock["geometry"]))
    s2 = make_states("rock_slab", n=300)
    ctx2.tuning(engine=pg.ENGINE_PLAIN)
    c, rc = ctx2.transport(s2, 0)
    eng = pg.Engine(gpu_physics, pool_slots=4096, max_inner=2, batch=4,
                    state_budget=1 << 28)
    t2 = eng.submit_host(ctx2, s2, 0)
    t1 = eng.submit_host(ctx, s0, 3)
    done = set()
    for _ in range(100000):
        got, pending = eng.step()
        done.update(got)
        if {t1, t2} <= done:
            break
    assert {t1, t2} <= done
    d, rd = eng.result(t1)
    assert a.tobytes() == d.tobytes() and ra.tobytes() == rd.tobytes()
    d, rd = eng.result(t2)
    assert c.tobytes() == d.tobytes() and rc.tobytes() == rd.tobytes()
