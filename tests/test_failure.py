"""Failure detection on the device (GPU): rejection samplings whose trial
cap runs out.

The reference's rejection loops have no bound (pumas.c:5839, 6115, 6126,
6241, 6918, 6973, 11208). On the device each one stops after the context's
`max_trials` trials (gpumas_context_trials_set) and its event ends with
GPUMAS_RETURN_INTERNAL_ERROR. With a cap of one or two trials many events
need more; this checks, for both engines, that those events report the
error, that every other event is bit for bit the one of an uncapped run,
and that the call returns promptly. No GPU fault, trap or endless loop is
involved: the cap is an ordinary loop bound.
"""
import time

import numpy as np
import pytest

from cases import CASES, make_states
from conftest import gpu_context, gpu_geometry

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["rock_slab", "stack_backward_straggled"])
@pytest.mark.parametrize("engine", [1, 2])
@pytest.mark.parametrize("cap", [1, 2])
def test_trial_cap_runs_out(gpu_physics, name, engine, cap):
    import pumas_gb300 as pg
    case = CASES[name]
    s0 = make_states(name, n=2000, first_event=300)
    geo = gpu_geometry(gpu_physics, case["geometry"])
    out = []
    for trials in (0, cap):
        ctx = gpu_context(gpu_physics, case["config"], case["seed"], geo)
        ctx.tuning(engine=engine, pool_slots=1024, max_inner=4, batch=4)
        ctx.max_trials = trials
        assert ctx.max_trials == (100000 if trials == 0 else cap)
        t0 = time.perf_counter()
        out.append(ctx.transport(s0, 300))
        out[-1] += (time.perf_counter() - t0,)
    (a, ra, _), (b, rb, dt) = out
    assert np.all(ra["status"] == 0)
    failed = rb["status"] != 0
    assert failed.any(), "no rejection needed more than %d trials" % cap
    assert np.all(rb["status"][failed] == pg.RETURN_INTERNAL_ERROR)
    ok = ~failed
    assert ok.any()
    assert a[ok].tobytes() == b[ok].tobytes()
    assert ra[ok].tobytes() == rb[ok].tobytes()
    assert dt < 30., dt


def test_trial_cap_values(gpu_physics):
    import pumas_gb300 as pg
    ctx = pg.Context(gpu_physics)
    assert ctx.max_trials == 100000
    ctx.max_trials = 7
    assert ctx.max_trials == 7
    ctx.max_trials = 0
    assert ctx.max_trials == 100000
    with pytest.raises(pg.PumasError) as err:
        ctx.max_trials = -1
    assert err.value.code == pg.RETURN_VALUE_ERROR
