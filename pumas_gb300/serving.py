"""Continuous-batching request server over the transport engine.

A request is a transport job whose initial states are in host memory: the
events of a slab-stack job, or a muography flux query over a set of
directions through the resident terrain. Physics tables, geometries and
contexts stay resident on the device. The server runs one engine
(gpumas_engine) and loops over three things:

* admit: queued requests enter the running engine in arrival order as long
  as the device state budget has room (gpumas_engine_submit_host refuses a
  request that does not fit; it waits for running requests to free memory);
* step: one CUDA graph batch of pool iterations, in which the events of
  every admitted request share the slot pool;
* complete: requests whose last event finished have their states and
  results copied back to host memory and are returned with their latency
  (arrival to results in host memory).

A request's results do not depend on what else runs: event k of a request
uses the random stream (context seed, first_event + k).

`plain_serve` is the baseline: one request at a time, each with one plain
one-thread-per-event launch through its context.
"""
import collections
import time

import numpy as np

from . import (ENGINE_PLAIN, MODE_BACKWARD, Context, Engine, PumasError,
               STATE_DTYPE, RESULT_DTYPE)
from . import workloads as W


class Request:
    """A transport request: a context (settings, geometry, seed) and the
    pumas_state records of its events, with event ids from first_event."""

    __slots__ = ("context", "states", "first_event", "kind", "arrival",
                 "admitted", "completed", "final", "results", "ticket")

    def __init__(self, context, states, first_event, kind=""):
        self.context = context
        self.states = states
        self.first_event = first_event
        self.kind = kind
        self.arrival = self.admitted = self.completed = None
        self.final = self.results = self.ticket = None

    @property
    def n(self):
        return len(self.states)

    @property
    def latency(self):
        return self.completed - self.arrival


class Server:
    """Continuous batching of transport requests on one GPU."""

    def __init__(self, physics, state_budget=40 << 30, max_jobs=1 << 20,
                 pool_slots=65536, max_inner=8, batch=4):
        self.engine = Engine(physics, pool_slots=pool_slots,
                             max_inner=max_inner, batch=batch,
                             max_jobs=max_jobs, state_budget=state_budget)
        self.queue = collections.deque()
        self.running = {}
        self.completed = 0

    def submit(self, request, now=None):
        """Queue a request (arrival time `now`, default: the clock)."""
        request.arrival = time.perf_counter() if now is None else now
        self.queue.append(request)

    def _admit(self):
        while self.queue:
            r = self.queue[0]
            t = self.engine.submit_host(r.context, r.states, r.first_event)
            if t is None:
                break
            r.ticket = t
            r.admitted = time.perf_counter()
            self.running[t] = r
            self.queue.popleft()

    def poll(self):
        """Admit what fits, run one batch, return the completed requests."""
        self._admit()
        done, _ = self.engine.step()
        now = time.perf_counter()
        out = []
        for t in done:
            r = self.running.pop(t)
            r.final, r.results = self.engine.result(t)
            r.completed = now
            out.append(r)
        self.completed += len(out)
        # Memory freed by completions admits queued requests at once.
        if out:
            self._admit()
        return out

    @property
    def idle(self):
        return not self.queue and not self.running


def serve_open_loop(server, requests, arrivals):
    """Offer `requests` at times `arrivals` (s from now) and serve them all.
    Returns the wall time from the first arrival to the last completion."""
    order = np.argsort(arrivals)
    t0 = time.perf_counter()
    k = 0
    n = len(requests)
    while k < n or not server.idle:
        now = time.perf_counter() - t0
        while k < n and arrivals[order[k]] <= now:
            server.submit(requests[order[k]], t0 + arrivals[order[k]])
            k += 1
        if server.idle:
            if k < n:
                time.sleep(max(0., min(1E-04, arrivals[order[k]] - now)))
            continue
        server.poll()
    return time.perf_counter() - t0


def plain_serve(requests, arrivals):
    """Baseline: requests in arrival order, one at a time, each through a
    plain one-thread-per-event launch of its context (synchronous
    gpumas_context_transport). Returns the wall time."""
    order = np.argsort(arrivals)
    t0 = time.perf_counter()
    for k in order:
        r = requests[k]
        now = time.perf_counter() - t0
        if arrivals[k] > now:
            time.sleep(arrivals[k] - now)
        r.arrival = t0 + arrivals[k]
        r.context.tuning(engine=ENGINE_PLAIN)
        r.final, r.results = r.context.transport(r.states, r.first_event)
        r.completed = time.perf_counter()
    return time.perf_counter() - t0


# ---------------------------------------------------------------------------
# Request mix of the serving workload.
# ---------------------------------------------------------------------------
class RequestMix:
    """Request generator: with probability 0.7 a slab-stack job drawn from
    a resident set of job geometries (events log-uniform in [1e2, 1e6]),
    otherwise a terrain flux query over 1-256 random directions with
    1e3-1e5 events each (log-uniform); event counts are multiplied by
    `scale` (at least 1 event). Request i uses event ids from i << 32."""

    def __init__(self, physics, seed=11, n_templates=256, scale=1E-03,
                 terrain_n=512):
        self.physics = physics
        self.seed = seed
        self.scale = scale
        self.templates = []
        for k, job in enumerate(W.slab_jobs(n_templates, seed=seed)):
            c = Context(physics)
            W.apply_config(c, W.slab_job_config(job))
            c.seed = seed * 7919 + k
            c.set_geometry(W.slab_job_geometry(physics, job))
            self.templates.append((job, c))
        self.terrain = Context(physics)
        W.apply_config(self.terrain, W.config_dict("terrain"))
        self.terrain.seed = seed
        self.heights = W.terrain_heights(n=terrain_n)
        self.terrain.set_geometry(W.terrain_geometry(physics, n=terrain_n))

    def make(self, i):
        """Request number i (deterministic in (seed, i))."""
        idx = np.array([i], dtype=np.uint64)
        u = [float(W.uniform(self.seed, 4, idx, k)[0]) for k in range(5)]
        first = int(i) << 32
        if u[0] < 0.7:
            job, c = self.templates[min(int(u[1] * len(self.templates)),
                                        len(self.templates) - 1)]
            n = max(1, int(round(self.scale * 100. * 1E+04 ** u[2])))
            j = dict(job, n=n, first_event=first)
            return Request(c, W.slab_job_states(j, seed=self.seed), first,
                           "job")
        nd = 1 + min(int(256 * u[1]), 255)
        per = max(1, int(round(self.scale * 1E+03 * 100. ** u[2])))
        ev = np.arange(nd, dtype=np.uint64) + np.uint64(first)
        zen = np.radians(85.) * W.uniform(self.seed, 4, ev, 5)
        azi = 2. * np.pi * W.uniform(self.seed, 4, ev, 6)
        s, _ = W.terrain(per, seed=self.seed, first_event=first,
                         directions=(zen, azi), heights=self.heights)
        return Request(self.terrain, s, first, "flux")


def agreement(a, ra, b, rb, rtol=1E-09):
    """Per event agreement of two transports of the same events: (bit
    identical, within rtol relative on energy, distance, grammage, time,
    weight, position and direction with identical end events, media and
    status). Scalars are compared relative to their magnitude, the position
    and direction vectors relative to their norm (a near zero transverse
    component is not held to rtol of itself)."""
    same = (a == b) & (ra == rb)
    close = np.ones(len(a), bool)
    for f in ("energy", "distance", "grammage", "time", "weight"):
        x, y = a[f], b[f]
        scale = np.maximum(np.maximum(np.abs(x), np.abs(y)), 1E-300)
        close &= np.abs(x - y) <= rtol * scale
    for f in ("position", "direction"):
        x, y = a[f], b[f]
        scale = np.maximum(np.maximum(np.linalg.norm(x, axis=1),
                                      np.linalg.norm(y, axis=1)), 1E-300)
        close &= np.linalg.norm(x - y, axis=1) <= rtol * scale
    for f in ("event", "medium_in", "medium_out", "status"):
        close &= ra[f] == rb[f]
    return same, close


def percentiles(values):
    v = np.asarray(values, dtype=np.float64)
    if len(v) == 0:
        return {"p50": None, "p95": None, "p99": None}
    return {"p50": float(np.percentile(v, 50)),
            "p95": float(np.percentile(v, 95)),
            "p99": float(np.percentile(v, 99))}


def sweep(physics, rates, seconds=2.0, scale=1E-03, seed=7,
          pool_slots=1 << 20, max_inner=8, batch=8, plain_max=300,
          stop_after=2):
    """Serving sweep: Poisson arrivals at each rate (requests/s, in
    increasing order) for `seconds`, continuous batching against the plain
    one-launch-per-request baseline (on at most plain_max requests of each
    rate), p50/p95/p99 latency in ms. Returns the sweep and the highest
    sustained rate (served throughput at least 90 % of the offered rate)
    with its p99. After `stop_after` rates in a row that are not sustained
    the server is saturated: the higher rates are listed as skipped (their
    backlog would only grow)."""
    mix = RequestMix(physics, seed=seed, scale=scale)
    server = Server(physics, pool_slots=pool_slots, max_inner=max_inner,
                    batch=batch)
    # Warm-up: a few requests through both paths.
    warm = [mix.make(10 ** 9 + i) for i in range(20)]
    serve_open_loop(server, warm, np.zeros(len(warm)))
    plain_serve([mix.make(10 ** 9 + i) for i in range(5)], np.zeros(5))
    out = []
    best = None
    base = 0
    missed = 0
    for rate in rates:
        if stop_after and missed >= stop_after:
            out.append({"rate": rate, "skipped": "saturated at lower rates"})
            continue
        n = max(1, int(round(rate * seconds)))
        gaps = -np.log(W.uniform(seed, 5, np.arange(
            base, base + n, dtype=np.uint64), 0)) / rate
        arrivals = np.cumsum(gaps) - gaps[0]
        reqs = [mix.make(base + i) for i in range(n)]
        events = sum(r.n for r in reqs)
        wall = serve_open_loop(server, reqs, arrivals)
        lat = [1E+03 * r.latency for r in reqs]
        errors = sum(int(np.count_nonzero(r.results["status"]))
                     for r in reqs)
        entry = {"rate": rate, "requests": n, "events": events,
                 "wall_s": wall, "throughput_rps": n / wall,
                 "events_per_s": events / wall,
                 "latency_ms": percentiles(lat), "event_errors": errors,
                 "sustained": bool(n / wall >= 0.9 * rate)}
        missed = 0 if entry["sustained"] else missed + 1
        # The plain baseline on the same arrivals (bounded: the first
        # plain_max requests; none with plain_max = 0).
        m = min(n, plain_max)
        if m == 0:
            out.append(entry)
            if entry["sustained"]:
                best = entry
            base += n
            continue
        preqs = [mix.make(base + i) for i in range(m)]
        pwall = plain_serve(preqs, arrivals[:m])
        n_ev = n_same = n_close = 0
        for a, b in zip(reqs[:m], preqs):
            same, close = agreement(a.final, a.results, b.final, b.results)
            n_ev += len(same)
            n_same += int(same.sum())
            n_close += int(close.sum())
        entry["plain"] = {"requests": m, "wall_s": pwall,
                          "throughput_rps": m / pwall,
                          "events_per_s": sum(r.n for r in preqs) / pwall,
                          "latency_ms": percentiles(
                              [1E+03 * r.latency for r in preqs]),
                          "events_compared": n_ev,
                          "bit_identical_events": n_same,
                          "events_within_1e-9": n_close}
        out.append(entry)
        if entry["sustained"]:
            best = entry
        base += n
    return {"sweep": out,
            "highest_sustained_rate": best["rate"] if best else None,
            "p99_ms_at_highest_sustained": (best["latency_ms"]["p99"]
                                            if best else None),
            "throughput_rps_at_highest_sustained": (
                best["throughput_rps"] if best else None),
            "engine": server.engine.stats(),
            "config": {"event_scale": scale, "seconds_per_rate": seconds,
                       "state_budget_gb": 40, "pool_slots": pool_slots,
                       "batch": batch, "max_inner": max_inner,
                       "mix": "70 % slab-stack jobs, 30 % terrain flux "
                              "queries (1-256 directions)"}}


def bench(args, rank, world, local):
    """Serving sweep over args.rates as its own bench line."""
    import json

    import pumas_gb300 as pg
    physics = pg.Physics()
    rates = [float(x) for x in args.rates.split(",")]
    r = sweep(physics, rates, args.serve_seconds, args.serve_scale,
              args.seed, args.pool_slots or (1 << 20), args.max_inner or 8,
              args.batch or 8, plain_max=args.serve_plain)
    if rank != 0:
        return
    top = None
    for e in r["sweep"]:
        if e["rate"] == r["highest_sustained_rate"] and "skipped" not in e:
            top = e
    top = top or r["sweep"][0]
    line = {"metric": "requests/s at p99 latency", "value":
            top["throughput_rps"], "unit": "requests/s", "n_gpus": world,
            "steps": len(rates), "warmup": 1,
            "ms_per_step": 1E+03 * top["wall_s"],
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(r["config"], workload="serve: Poisson arrivals, "
                           "70 %% slab-stack jobs, 30 %% terrain flux "
                           "queries (1-256 directions), events x %g"
                           % args.serve_scale)}
    line.update({k: v for k, v in r.items() if k != "config"})
    print(json.dumps(line), flush=True)
