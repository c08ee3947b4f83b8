"""Host logic without a GPU: the workload generators, the serving
agreement and percentile helpers, the autotuner's selection and storage,
and the bench's rank helpers."""
import numpy as np
import pytest

from pumas_gb300 import workloads as W


def test_slab_jobs_follow_their_specification():
    jobs = W.slab_jobs(512, seed=5)
    again = W.slab_jobs(512, seed=5)
    assert all(np.array_equal(a["slab_z"], b["slab_z"]) and a["n"] == b["n"]
               for a, b in zip(jobs, again))
    for j, job in enumerate(jobs):
        ns = len(job["materials"])
        assert 1 <= ns <= 8 and len(job["slab_z"]) == ns + 1
        thick = np.diff(job["slab_z"])
        assert np.all(thick >= 1.) and np.all(thick <= 2000.)
        assert set(job["materials"]) <= set(W.JOB_MATERIALS)
        assert 100 <= job["n"] <= 1E+06
        assert 1. <= job["emin"] <= 100.
        assert job["emax"] == pytest.approx(1E+03 * job["emin"])
        assert job["first_event"] == j << 32
        cfg = W.slab_job_config(job)
        assert cfg["limit_energy"] == (1. if job["direction"] == 0 else 1E+07)
    # Both directions and all materials occur.
    assert {j["direction"] for j in jobs} == {0, 1}
    assert {m for j in jobs for m in j["materials"]} == set(W.JOB_MATERIALS)
    # Scaled event counts: round(x) against round(100 x), x >= 1.
    scaled = W.slab_jobs(512, seed=5, event_scale=1E-02)
    assert all(abs(100 * s["n"] - j["n"]) <= 51
               for s, j in zip(scaled, jobs))


def test_slab_job_states():
    job = dict(W.slab_jobs(4, seed=5)[1], n=1000)
    s = W.slab_job_states(job, seed=5)
    assert len(s) == 1000
    assert np.all((s["energy"] >= job["emin"]) & (s["energy"] <= job["emax"]))
    assert np.allclose(np.linalg.norm(s["direction"], axis=1), 1.)
    assert np.all(s["position"][:, 2] == 0.)
    assert np.array_equal(s, W.slab_job_states(job, seed=5))


def test_terrain_states_and_flux():
    zen, azi = W.terrain_directions(4, 8)
    assert len(zen) == 32 and np.all(zen < np.radians(85.))
    heights = W.terrain_heights(n=64)
    s, d = W.terrain(3, seed=2, directions=(zen, azi), heights=heights)
    assert len(s) == 96 and np.array_equal(np.bincount(d), np.full(32, 3))
    assert np.allclose(np.linalg.norm(s["direction"], axis=1), 1.)
    # Momenta point down: the muons come from the sky.
    assert np.all(s["direction"][:, 2] < 0.)
    # The detector sits under the surface at the grid centre.
    h, x0, y0 = heights
    zs = W.surface_height(h, x0, y0, W.TERRAIN_CELL, 0., 0.)
    assert np.all(s["position"][:, 2] < zs)
    # Flux: only events that left through the top count.
    from pumas_gb300 import EVENT_MEDIUM, RESULT_DTYPE
    r = np.zeros(len(s), dtype=RESULT_DTYPE)
    r["event"] = EVENT_MEDIUM
    r["medium_out"] = -1
    r["medium_out"][d == 0] = 0
    f = W.terrain_flux(s, r, d, 32)
    assert f[0] == 0. and np.all(f[1:] > 0.)


def test_serving_agreement_and_percentiles():
    from pumas_gb300 import RESULT_DTYPE, new_states
    from pumas_gb300.serving import agreement, percentiles
    a = new_states(8)
    a["energy"] = np.linspace(1., 8., 8)
    ra = np.zeros(8, dtype=RESULT_DTYPE)
    b, rb = a.copy(), ra.copy()
    same, close = agreement(a, ra, b, rb)
    assert same.all() and close.all()
    b["energy"][1] *= 1. + 1E-12      # an ulp-scale difference: close
    b["energy"][2] *= 1. + 1E-06      # a real difference
    rb["event"][3] = 1                # another end event
    # Vectors are compared relative to their norm: a last bits difference
    # of a near zero transverse component is close, a real deflection not.
    a["position"][4] = b["position"][4] = (1E-08, 0., 1E+05)
    b["position"][4, 0] = 2E-08
    a["direction"][5] = b["direction"][5] = (0., 0., 1.)
    b["direction"][5, 0] = 1E-06
    same, close = agreement(a, ra, b, rb)
    assert list(np.where(~same)[0]) == [1, 2, 3, 4, 5]
    assert list(np.where(~close)[0]) == [2, 3, 5]
    p = percentiles(np.arange(1., 101.))
    assert p["p50"] == pytest.approx(50.5) and p["p99"] == pytest.approx(
        99.01)
    assert percentiles([])["p99"] is None


def test_autotune_picks_the_fastest_point(monkeypatch, tmp_path):
    """The tuner times every grid point and keeps the fastest; the stored
    result reads back as engine parameters."""
    import pumas_gb300
    from pumas_gb300 import autotune

    class FakeEngine:
        def __init__(self, physics, **point):
            self.point = point

    clock = {"t": 0.}
    monkeypatch.setattr(pumas_gb300, "Engine", FakeEngine)
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: clock["t"])

    def run(engine):
        p = engine.point
        # A made-up cost with its minimum at (1048576, 8, 16, 0).
        clock["t"] += (abs(p["pool_slots"] - 1048576) / 1E+06 +
                       abs(p["max_inner"] - 8) + abs(p["batch"] - 16) +
                       (0.5 if p["tail"] else 0.) + 1.)

    best = autotune.tune(None, run)
    assert (best["pool_slots"], best["max_inner"], best["batch"],
            best["tail"]) == (1048576, 8, 16, 0)
    g = autotune.DEFAULT_GRID
    assert len(best["trials"]) == (len(g["pool_slots"]) * len(g["max_inner"]) *
                                   len(g["batch"]) * len(g["tail"]))
    path = tmp_path / "tuning.json"
    autotune.save(best, str(path))
    assert autotune.load(str(path)) == dict(
        pool_slots=1048576, max_inner=8, batch=16, tail=0)
    assert autotune.load(str(tmp_path / "missing.json")) == {}


def test_bench_rank_helpers():
    import bench
    assert bench.rank_first_event(0) == 0
    assert bench.rank_first_event(3) == 3 * 10 ** 12


def test_atmosphere_workload_on_the_oracle():
    """The atmosphere workload of the bench, through the CPU oracle: every
    event ends cleanly, some reach the rock, and the CPU baseline helper
    reports a rate."""
    import bench
    import oracle
    import pumas_gb300 as pg
    s0 = W.atmosphere(64, seed=7)
    assert np.all(s0["direction"][:, 2] <= -0.2)
    oracle.build_port()
    port = oracle.Port(pg.default_dump())
    spec = W.atmosphere_spec()
    media = [(port.material_index(m), d) for m, d in spec["media"]]
    geo = oracle.make_geometry(spec["kind"], media, **{
        k: v for k, v in spec.items() if k not in ("kind", "media")})
    cfg = oracle.Config(seed=7, **W.config_dict("atmosphere"))
    s1, r1 = port.transport(cfg, geo, s0, 0, 1)
    assert np.all(r1["status"] == 0)
    assert np.any(r1["medium_out"] == 0) or np.any(s1["position"][:, 2] < 0.)
    assert np.mean(r1["steps"]) > 10.
    cpu = bench.port_baseline("atmosphere", s0, W.config_dict("atmosphere"),
                              spec, 7, 0, "64 events")
    assert cpu["value"] > 0. and cpu["kind"] == "port"


def test_cpu_baseline_explains_itself():
    """The CPU baseline of the bench line reports the host's cores, the
    OpenMP threads, the one thread rate, the thread scaling and the rate
    with the Coulomb functions in double, on the same events."""
    import bench
    cpu = bench.cpu_baseline(400, 7)
    for key in ("value", "cores", "nproc", "omp_max_threads", "one_thread",
                "thread_scaling", "one_thread_coulomb_double"):
        assert key in cpu, key
    assert cpu["kind"] == "port" and cpu["value"] > 0.
    assert cpu["one_thread_coulomb_double"]["same_steps"]


def test_atmosphere_geometry_descriptor():
    """The bench's device geometry: the ctypes descriptor carries the
    locals of both media."""
    g = W.atmosphere_geometry({"StandardRock": 0, "Air": 2})
    c = g.c
    assert c.kind == 1 and c.n_slabs == 2 and c.n_media == 2
    assert [c.slab_z[i] for i in range(3)] == list(W.ATMOSPHERE_Z)
    assert (c.media[0].material, c.media[1].material) == (0, 2)
    air, rock = c.locals[1], c.locals[0]
    assert rock.model == 0 and list(rock.magnet) == [0., 0., 0.]
    assert air.model == 1 and air.rho0 == 1.205 and air.lambda_ == 12E+03
    assert list(air.axis) == [0., 0., 1.] and air.eps == 5E-02
    assert list(air.magnet) == [0., 2E-05, -4E-05]
