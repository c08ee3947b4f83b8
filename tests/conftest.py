"""Shared fixtures: physics dump, CPU oracles and the GPU engine."""
import gzip
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


# Parity fractions reported by the GPU tests: name -> (events within
# tolerance, events). Printed at the end of the run.
PARITY_REPORT = {}


def pytest_terminal_summary(terminalreporter):
    if not PARITY_REPORT:
        return
    tr = terminalreporter
    tr.section("parity: events within 1e-9 on every field (weight included), "
               "or table entries bit for bit")
    good = total = 0
    for name in sorted(PARITY_REPORT):
        g, n = PARITY_REPORT[name]
        good += g
        total += n
        tr.write_line("%-40s %8d / %-8d %.5f" % (name, g, n, g / max(n, 1)))
    tr.write_line("%-40s %8d / %-8d %.5f" % ("all", good, total,
                                            good / max(total, 1)))


@pytest.fixture(scope="session")
def dump():
    import pumas_gb300
    return pumas_gb300.default_dump()


@pytest.fixture(scope="session")
def port(dump):
    import oracle
    oracle.build_port()
    return oracle.Port(dump)


@pytest.fixture(scope="session")
def reference(dump, tmp_path_factory):
    import oracle
    try:
        if not oracle.reference_available():
            if not oracle.build_reference():
                pytest.skip("reference sources not available")
    except Exception as exc:
        pytest.skip("reference not buildable: %s" % exc)
    path = tmp_path_factory.mktemp("phys") / "muon.pumas"
    path.write_bytes(dump)
    return oracle.Reference(str(path))


@pytest.fixture(scope="session")
def gpu_physics(dump):
    import pumas_gb300
    pumas_gb300.library(build=True)
    return pumas_gb300.Physics(dump)


@pytest.fixture(scope="session")
def tau_dump():
    import pumas_gb300
    return pumas_gb300.default_dump("tau")


@pytest.fixture(scope="session")
def oracle_cache():
    """Oracles of physics other than the default muon one, by (kind,
    physics), each in its own copy of the library (the physics is a global
    of the library)."""
    return {}


@pytest.fixture(scope="session")
def gpu_tau_physics(gpu_physics, tau_dump):
    import pumas_gb300
    return pumas_gb300.Physics(tau_dump)


def case_oracle(request, name, kind):
    """The oracle (`port` or `reference`) with a case's physics."""
    import oracle
    from cases import particle, physics_dump
    p = particle(name)
    base = request.getfixturevalue(kind)
    if p == "muon":
        return base
    cache = request.getfixturevalue("oracle_cache")
    if (kind, p) not in cache:
        dump = physics_dump(p)
        if kind == "port":
            cache[kind, p] = oracle.Port(dump, private=True)
        else:
            path = request.getfixturevalue("tmp_path_factory").mktemp(
                "phys") / (p + ".pumas")
            path.write_bytes(dump)
            cache[kind, p] = oracle.Reference(str(path), private=True)
    return cache[kind, p]


@pytest.fixture(scope="session")
def gpu_physics_cache():
    """GPU physics of the cases with non-default DCS models, by name."""
    return {}


def case_physics(request, name):
    """The GPU physics of a case."""
    from cases import particle, physics_dump
    p = particle(name)
    if p in ("muon", "tau"):
        return request.getfixturevalue(
            "gpu_physics" if p == "muon" else "gpu_%s_physics" % p)
    request.getfixturevalue("gpu_physics")
    cache = request.getfixturevalue("gpu_physics_cache")
    if p not in cache:
        import pumas_gb300
        cache[p] = pumas_gb300.Physics(physics_dump(p))
    return cache[p]


def oracle_geometry(orc, spec):
    import oracle
    media = [(orc.material_index(m), d) for m, d in spec["media"]]
    kw = {k: v for k, v in spec.items() if k not in ("kind", "media")}
    return oracle.make_geometry(spec["kind"], media, **kw)


def gpu_geometry(physics, spec):
    import pumas_gb300 as pg
    media = [(physics.material_index(m), d) for m, d in spec["media"]]
    loc = spec.get("locals")
    if spec["kind"] == pg.GEOMETRY_UNIFORM:
        return pg.Geometry(pg.GEOMETRY_UNIFORM, media, locals=loc, medium=0)
    if spec["kind"] == pg.GEOMETRY_SLABS:
        return pg.Geometry(pg.GEOMETRY_SLABS, media, locals=loc,
                           z=spec["slab_z"], slab_media=spec["slab_media"])
    return pg.Geometry(pg.GEOMETRY_HEIGHTMAP, media,
                       heights=spec["hm_z"], x0=spec["hm_x0"],
                       y0=spec["hm_y0"], dx=spec["hm_dx"], dy=spec["hm_dy"],
                       below=spec["hm_below"], above=spec["hm_above"],
                       ztop=spec["hm_ztop"])


def oracle_config(cfg, seed):
    import oracle
    return oracle.Config(seed=seed, **cfg)


def gpu_context(physics, cfg, seed, geometry):
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    ctx = pg.Context(physics)
    W.apply_config(ctx, cfg)
    ctx.seed = seed
    ctx.set_geometry(geometry)
    return ctx


FIELDS = ("energy", "distance", "grammage", "time", "weight")


def compare(a, ra, b, rb, rtol=1E-09):
    """Per event agreement of two transports: (bit-identical mask,
    within-tolerance mask). Tolerance is relative with an absolute floor of
    rtol for quantities near zero, on energy, distance, grammage, time,
    weight, position and direction, plus equal end events and media."""
    same = np.ones(len(a), bool)
    close = np.ones(len(a), bool)
    for f in FIELDS + ("position", "direction"):
        x, y = a[f], b[f]
        if x.ndim == 1:
            x, y = x[:, None], y[:, None]
        same &= np.all(x == y, axis=1)
        scale = np.maximum(np.maximum(np.abs(x), np.abs(y)), 1.)
        if f in ("position", "direction"):
            scale = np.maximum(scale, np.max(np.abs(x), axis=1,
                                             keepdims=True))
        close &= np.all(np.abs(x - y) <= rtol * scale, axis=1)
    for f in ("event", "medium_out", "status"):
        same &= ra[f] == rb[f]
        close &= ra[f] == rb[f]
    same &= a["decayed"] == b["decayed"]
    close &= a["decayed"] == b["decayed"]
    return same, close
