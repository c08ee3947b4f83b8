"""Batched jobs and continuous batching on the GPU engine (gpumas_engine).

Many independent transport jobs (different geometries, directions, limits,
seeds and event counts) run in one slot pool. Each job's results must equal
those of the same job transported alone through its context: an event's
random stream depends only on (context seed, event id) and its operations
do not depend on what runs beside it. The runs below are bit for bit equal;
the serving mix is checked at 1e-9 with at least 99.9 % of events bit for
bit (an event whose phases ran in different kernels can differ by an ulp
where the compiler fused multiply-adds differently). The jobs of the batched
slab-stack workload are also checked against the CPU oracle at 1e-9.
"""
import numpy as np
import pytest

from conftest import compare

pytestmark = pytest.mark.gpu


def to_device(states):
    """Device structure of arrays of pumas_state records (torch tensors)."""
    import torch
    import pumas_gb300 as pg
    dev = torch.device("cuda", 0)
    cols = {}
    for f in ("charge", "energy", "distance", "grammage", "time", "weight"):
        cols[f] = torch.from_numpy(np.ascontiguousarray(states[f])).to(dev)
    for k in range(3):
        cols["position%d" % k] = torch.from_numpy(
            np.ascontiguousarray(states["position"][:, k])).to(dev)
        cols["direction%d" % k] = torch.from_numpy(
            np.ascontiguousarray(states["direction"][:, k])).to(dev)
    cols["decayed"] = torch.from_numpy(
        np.ascontiguousarray(states["decayed"])).to(dev)
    cols["result"] = torch.zeros((len(states), pg.RESULT_DTYPE.itemsize),
                                 dtype=torch.uint8,
                                 device=dev)
    soa = {f: cols[f].data_ptr() for f in
           ("charge", "energy", "distance", "grammage", "time", "weight",
            "decayed", "result")}
    soa["position"] = [cols["position%d" % k].data_ptr() for k in range(3)]
    soa["direction"] = [cols["direction%d" % k].data_ptr() for k in range(3)]
    return cols, soa


def from_device(cols, n):
    import pumas_gb300 as pg
    s = np.zeros(n, dtype=pg.STATE_DTYPE)
    for f in ("charge", "energy", "distance", "grammage", "time", "weight",
              "decayed"):
        s[f] = cols[f].cpu().numpy()
    for k in range(3):
        s["position"][:, k] = cols["position%d" % k].cpu().numpy()
        s["direction"][:, k] = cols["direction%d" % k].cpu().numpy()
    r = np.frombuffer(cols["result"].cpu().numpy().tobytes(),
                      dtype=pg.RESULT_DTYPE)
    return s, r


def make_jobs(physics, n_jobs, scale, seed=5):
    """Contexts, geometries and initial states of slab-stack jobs."""
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    out = []
    for k, job in enumerate(W.slab_jobs(n_jobs, seed=seed,
                                        event_scale=scale)):
        ctx = pg.Context(physics)
        W.apply_config(ctx, W.slab_job_config(job))
        ctx.seed = 1000 + k
        ctx.set_geometry(W.slab_job_geometry(physics, job))
        out.append((job, ctx, W.slab_job_states(job, seed=seed)))
    return out


def test_engine_run_matches_context_transport(gpu_physics):
    """One run of 24 uneven jobs (forward and backward, 1 to 8 slabs of
    rock, water and iron) plus a terrain job: every job bit-identical to its
    own context transport."""
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    jobs = make_jobs(gpu_physics, 24, 0.003)
    ctx = pg.Context(gpu_physics)
    W.apply_config(ctx, W.config_dict("terrain"))
    ctx.seed = 99
    ctx.set_geometry(W.terrain_geometry(gpu_physics, n=128))
    hs = W.terrain_heights(n=128)
    s_t, _ = W.terrain(40, seed=4, directions=W.terrain_directions(4, 8),
                       heights=hs)
    jobs.append((dict(first_event=7 << 40), ctx, s_t))
    eng = pg.Engine(gpu_physics, pool_slots=4096, max_inner=4, batch=6)
    dev = []
    for job, c, s0 in jobs:
        cols, soa = to_device(s0)
        dev.append((cols, soa))
    eng.run([(c, len(s0), soa, job["first_event"])
             for (job, c, s0), (cols, soa) in zip(jobs, dev)])
    for (job, c, s0), (cols, soa) in zip(jobs, dev):
        a, ra = from_device(cols, len(s0))
        b, rb = c.transport(s0, job["first_event"])
        assert a.tobytes() == b.tobytes()
        assert ra.tobytes() == rb.tobytes()
        assert np.all(ra["status"] == 0)
    st = eng.stats()
    assert st["events"] == sum(len(s0) for _, _, s0 in jobs)
    assert st["launches"] > 0 and st["kernel_ms"] > 0.


def test_engine_continuous_batching(gpu_physics):
    """Jobs submitted from host memory while others run, under a small
    state budget: submissions beyond the budget are refused until running
    jobs complete; each result equals the job run alone."""
    import pumas_gb300 as pg
    jobs = make_jobs(gpu_physics, 16, 0.002, seed=8)
    per_event = pg.STATE_DTYPE.itemsize + pg.RESULT_DTYPE.itemsize
    largest = max(len(s0) for _, _, s0 in jobs)
    budget = 3 * (largest * per_event + 512)
    eng = pg.Engine(gpu_physics, pool_slots=2048, max_inner=2, batch=2,
                    max_jobs=8, state_budget=budget)
    queue = list(range(len(jobs)))
    tickets, refused, done = {}, 0, {}
    for it in range(100000):
        while queue:
            k = queue[0]
            job, c, s0 = jobs[k]
            t = eng.submit_host(c, s0, job["first_event"])
            if t is None:
                refused += 1
                break
            tickets[t] = k
            queue.pop(0)
        finished, pending = eng.step()
        for t in finished:
            done[tickets[t]] = eng.result(t)
        if not queue and pending == 0:
            break
    assert len(done) == len(jobs)
    assert refused > 0
    assert eng.stats()["budget_used"] == 0
    for k, (job, c, s0) in enumerate(jobs):
        a, ra = done[k]
        b, rb = c.transport(s0, job["first_event"])
        assert a.tobytes() == b.tobytes()
        assert ra.tobytes() == rb.tobytes()


def test_engine_jobs_match_oracle(gpu_physics, port):
    """Slab-stack jobs through the engine against the CPU oracle: at least
    99.9 % of events within 1e-9."""
    import oracle
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    jobs = make_jobs(gpu_physics, 12, 0.004, seed=11)
    eng = pg.Engine(gpu_physics, pool_slots=8192)
    dev = [to_device(s0) for _, _, s0 in jobs]
    eng.run([(c, len(s0), soa, job["first_event"])
             for (job, c, s0), (cols, soa) in zip(jobs, dev)])
    good = total = 0
    for (job, c, s0), (cols, soa) in zip(jobs, dev):
        a, ra = from_device(cols, len(s0))
        mats = [port.material_index(m) for m in job["materials"]]
        geo = oracle.make_geometry(
            1, [(m, 0.) for m in mats], slab_z=job["slab_z"],
            slab_medium=list(range(len(mats))))
        cfg = oracle.Config(seed=c.seed, **W.slab_job_config(job))
        b, rb = port.transport(cfg, geo, s0, job["first_event"], 0)
        _, close = compare(a, ra, b, rb, 1E-09)
        good += int(close.sum())
        total += len(close)
    assert good >= 0.999 * total, "%d / %d" % (good, total)


def test_engine_rejects_bad_jobs(gpu_physics):
    import pumas_gb300 as pg
    eng = pg.Engine(gpu_physics, pool_slots=256, max_jobs=2)
    ctx = pg.Context(gpu_physics)
    with pytest.raises(pg.PumasError) as err:
        eng.submit_host(ctx, pg.new_states(4))       # no geometry
    assert err.value.code == pg.RETURN_MEDIUM_ERROR
    ctx.set_geometry(pg.Geometry.slabs(
        [0., 10.], [gpu_physics.material_index("Water")]))
    ctx.accuracy = 2.
    with pytest.raises(pg.PumasError) as err:
        eng.submit_host(ctx, pg.new_states(4))
    assert err.value.code == pg.RETURN_ACCURACY_ERROR
    ctx.accuracy = 1E-02
    assert eng.submit_host(ctx, pg.new_states(4)) is None   # no budget
    # Empty jobs complete at the next step without device work.
    t = eng.submit(ctx, 0, {k: 0 for k in (
        "charge", "energy", "distance", "grammage", "time", "weight",
        "decayed", "position", "direction")} | {"position": [0] * 3,
                                                "direction": [0] * 3})
    done, pending = eng.step()
    assert done == [t] and pending == 0


def test_serving_results_same_alone_and_in_mix(gpu_physics):
    """Requests of the serving mix (slab-stack jobs and terrain flux
    queries) served together with continuous batching under a small state
    budget give, request by request, the results of the request run
    alone."""
    from pumas_gb300 import serving
    mix = serving.RequestMix(gpu_physics, seed=3, n_templates=8,
                             scale=2E-04, terrain_n=128)
    reqs = [mix.make(i) for i in range(40)]
    assert {r.kind for r in reqs} == {"job", "flux"}
    per_event = 136
    server = serving.Server(gpu_physics,
                            state_budget=4 * per_event * max(
                                r.n for r in reqs) + 4096,
                            max_jobs=64, pool_slots=4096, batch=2)
    arrivals = np.linspace(0., 0.05, len(reqs))
    serving.serve_open_loop(server, reqs, arrivals)
    assert server.completed == len(reqs)
    n = n_same = 0
    for r in reqs:
        assert r.latency > 0.
        a, ra = r.context.transport(r.states, r.first_event)
        same, close = serving.agreement(r.final, r.results, a, ra)
        assert close.all()
        n += len(same)
        n_same += int(same.sum())
    # Same draws and operations: all but a few events bit for bit (an ulp
    # where multiply-adds were fused differently in different kernels).
    assert n_same >= 0.999 * n
