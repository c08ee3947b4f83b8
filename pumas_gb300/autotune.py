"""Autotuner of the slot pool engine.

The engine has three parameters that change its speed but never its
results (an event's random stream depends only on its context seed and
event id):

* ``pool_slots``: events in flight (resident slots, refilled from the
  event queue as events finish);
* ``max_inner``: continuous steps a slot makes per visit before it yields
  its lane (events per lane and visit);
* ``batch``: pool iterations per CUDA graph launch, i.e. how often the host
  checks for completed jobs and admits new ones (the refill / compaction
  period seen from the host);
* ``tail``: the drain threshold, in active slots, below which the last
  events run to their end in one launch instead of being regrouped by step
  kind (-1: one slot per resident thread, 0: never).

``tune`` times an engine run of a sample workload for each point of a grid
and keeps the fastest; the result is stored as JSON and read back by
``load`` for engines created later. Timings are wall clock around a whole
run, after one untimed run per engine (graph capture, pool allocation).
"""
import itertools
import json
import os
import time

DEFAULT_GRID = {
    "pool_slots": [524288, 1048576, 2097152],
    "max_inner": [4, 8, 16],
    "batch": [8, 16],
    "tail": [0, -1],
}

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PATH = os.path.join(HERE, "data", "_build", "tuning.json")


def tune(physics, make_run, grid=None, repeats=1, log=None):
    """Time ``make_run(engine)`` (a callable that runs a sample workload on
    the given engine and returns when it is done) for every point of
    ``grid`` and return the fastest point as a dict, with the timings of
    all points under ``"trials"``."""
    from . import Engine
    grid = dict(DEFAULT_GRID, **(grid or {}))
    keys = ("pool_slots", "max_inner", "batch", "tail")
    trials = []
    for values in itertools.product(*(grid[k] for k in keys)):
        point = dict(zip(keys, values))
        eng = Engine(physics, **point)
        make_run(eng)
        best = None
        for _ in range(repeats):
            t = time.perf_counter()
            make_run(eng)
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        del eng
        trials.append(dict(point, seconds=best))
        if log is not None:
            log(trials[-1])
    top = min(trials, key=lambda t: t["seconds"])
    out = {k: top[k] for k in keys}
    out["seconds"] = top["seconds"]
    out["trials"] = trials
    return out


def save(result, path=DEFAULT_PATH):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(result, f, indent=1)


def load(path=DEFAULT_PATH):
    """Tuned engine parameters (pool_slots, max_inner, batch, tail), or an
    empty dict when no tuning was stored."""
    try:
        with open(path) as f:
            r = json.load(f)
    except (OSError, ValueError):
        return {}
    return {k: int(r[k]) for k in ("pool_slots", "max_inner", "batch",
                                   "tail") if k in r}
