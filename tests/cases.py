"""Parity cases shared by the golden fixture generator and the tests.

Each case is a transport configuration (the public pumas_context settings),
a geometry made of named materials and a generator of initial states. The
same case runs on the reference (to make the golden fixtures), on the C
restatement oracle and on the GPU engine.
"""
import numpy as np

from pumas_gb300 import workloads as W
from pumas_gb300 import STATE_DTYPE

FWD, BWD = 0, 1
CSDA, MIXED, STRAGGLED, DISABLED = 0, 1, 2, -1
WEIGHTED, RANDOMISED = 0, 1
LIMIT_ENERGY, LIMIT_DISTANCE, LIMIT_GRAMMAGE, LIMIT_TIME = 1, 2, 4, 8


def _cfg(energy_loss, scattering, direction, decay=WEIGHTED, event=0,
         **limits):
    c = dict(energy_loss=energy_loss, scattering=scattering,
             direction=direction, decay=decay, event=event,
             limit_energy=0., limit_distance=0., limit_grammage=0.,
             limit_time=0., accuracy=1E-02)
    c.update(limits)
    return c


def _states(n, seed, first, emin, emax, z0=0., uz=1., alt=True):
    ev = np.arange(first, first + n, dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.) if alt else -1.
    s["energy"] = emin * (emax / emin) ** W.uniform(seed, 1, ev, 0)
    s["weight"] = 1.
    s["position"][:, 2] = z0
    s["direction"][:, 2] = uz
    return s


STACK = dict(kind=1, media=[("StandardRock", 0.), ("Water", 0.),
                            ("Iron", 0.), ("Air", 0.), ("StandardRock", 2000.)],
             slab_z=[0., 10., 30., 31., 200., 400.],
             slab_media=[0, 1, 2, 3, 4])
ROCK_SLAB = dict(kind=1, media=[("StandardRock", 0.)], slab_z=[0., 1000.],
                 slab_media=[0])
ROCK = dict(kind=0, media=[("StandardRock", 0.)])
WATER = dict(kind=0, media=[("Water", 0.)])

CASES = {
    # Plain forward CSDA in infinite rock (pumas.c:4777-4949).
    "plain_csda": dict(
        config=_cfg(CSDA, DISABLED, FWD, decay=DISABLED, event=LIMIT_ENERGY,
                    limit_energy=1.),
        geometry=ROCK, n=2000, seed=1,
        states=lambda n, s, f: W.plain_csda(n, s, f)),
    # Forward straggled + mixed scattering through 1 km of rock.
    "rock_slab": dict(
        config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY,
                    limit_energy=1.),
        geometry=ROCK_SLAB, n=300, seed=7,
        states=lambda n, s, f: W.rock_slab(n, s, f)),
    # Backward straggled + mixed, up through the rock slab.
    "rock_slab_backward": dict(
        config=_cfg(STRAGGLED, MIXED, BWD),
        geometry=ROCK_SLAB, n=200, seed=9,
        states=lambda n, s, f: _states(n, s, f, 10., 1E+04, z0=999.999)),
    # Forward mixed (no straggling): DEL and EHS pre-sampled as limits.
    "stack_forward_mixed": dict(
        config=_cfg(MIXED, MIXED, FWD, event=LIMIT_ENERGY, limit_energy=1.),
        geometry=STACK, n=200, seed=11,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04)),
    # Forward straggled through the multi-material stack.
    "stack_forward_straggled": dict(
        config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY,
                    limit_energy=1.),
        geometry=STACK, n=200, seed=12,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04)),
    # Backward mixed and straggled through the stack.
    "stack_backward_mixed": dict(
        config=_cfg(MIXED, MIXED, BWD),
        geometry=STACK, n=200, seed=13,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04, z0=399.99)),
    "stack_backward_straggled": dict(
        config=_cfg(STRAGGLED, MIXED, BWD),
        geometry=STACK, n=200, seed=14,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04, z0=399.99)),
    # Randomised decay, CSDA stepping without scattering.
    "stack_csda_randomised": dict(
        config=_cfg(CSDA, DISABLED, FWD, decay=RANDOMISED,
                    event=LIMIT_ENERGY, limit_energy=1.),
        geometry=STACK, n=300, seed=15,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+03)),
    # External limits in water (pumas.c:5250-5259, 6389-6397, 6713-6809).
    "water_distance_limit": dict(
        config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY |
                    LIMIT_DISTANCE, limit_energy=1., limit_distance=50.),
        geometry=WATER, n=200, seed=16,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+03)),
    "water_grammage_limit": dict(
        config=_cfg(MIXED, MIXED, FWD, event=LIMIT_GRAMMAGE,
                    limit_grammage=3E+05),
        geometry=WATER, n=200, seed=17,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04)),
    "water_time_limit": dict(
        config=_cfg(CSDA, MIXED, FWD, event=LIMIT_TIME, limit_time=1E+02),
        geometry=WATER, n=200, seed=18,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+03)),
    # CSDA in infinite rock, backward, grammage limit.
    "rock_csda_backward": dict(
        config=_cfg(CSDA, DISABLED, BWD, event=LIMIT_GRAMMAGE,
                    limit_grammage=1E+05),
        geometry=ROCK, n=500, seed=19,
        states=lambda n, s, f: _states(n, s, f, 1., 1E+04)),
}


def _terrain_states(n, seed, first):
    """Muons at a detector 20 m under the centre of the small terrain, from
    directions drawn uniformly in zenith [0, 85] deg and azimuth, kinetic
    energy log-uniform in [1 GeV, 100 TeV], weight 1 / pdf."""
    h = TERRAIN["hm_z"]
    ev = np.arange(first, first + n, dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.)
    lr = np.log(1E+05)
    k = np.exp(lr * W.uniform(seed, 1, ev, 0))
    s["energy"] = k
    s["weight"] = k * lr
    zen = np.radians(85.) * W.uniform(seed, 1, ev, 1)
    azi = 2. * np.pi * W.uniform(seed, 1, ev, 2)
    z0 = W.surface_height(h, TERRAIN["hm_x0"], TERRAIN["hm_y0"],
                          TERRAIN["hm_dx"], 0., 0.) - 20.
    s["position"][:, 2] = z0
    st = np.sin(zen)
    s["direction"][:, 0] = -st * np.cos(azi)
    s["direction"][:, 1] = -st * np.sin(azi)
    s["direction"][:, 2] = -np.cos(zen)
    return s


# A 64 x 64 node cut of the terrain workload's construction (10 m cells).
TERRAIN = W.terrain_spec(seed=3, n=64)

CASES["terrain_backward"] = dict(
    config=_cfg(STRAGGLED, MIXED, BWD),
    geometry=TERRAIN, n=200, seed=21,
    states=lambda n, s, f: _terrain_states(n, s, f))


# Media with local properties (struct gpumas_locals): the reference's
# exponential atmosphere with the geomagnetic field of
# examples/pumas/geometry.c:76-97, over 200 m of rock, and a magnetised iron
# slab (1.5 T, a muon spectrometer's magnet).
AIR_LOCALS = dict(model=1, rho0=1.205, axis=(0., 0., 1.), h0=0.,
                  lambda_=12E+03, eps=5E-02, magnet=(0., 2E-05, -4E-05))
ATMOSPHERE = dict(kind=1, media=[("StandardRock", 0.), ("Air", 0.)],
                  slab_z=[-200., 0., 20000.], slab_media=[0, 1],
                  locals=[dict(), AIR_LOCALS])
IRON_FIELD = dict(kind=1, media=[("Iron", 0.)], slab_z=[0., 20.],
                  slab_media=[0], locals=[dict(magnet=(1.5, 0., 0.))])


def _sky_states(n, seed, first, emin, emax, z0, cos_min=0.2):
    """Muons with momenta pointing down, at zenith angles of cosine in
    [cos_min, 1] and uniform azimuth."""
    s = _states(n, seed, first, emin, emax, z0=z0)
    ev = np.arange(first, first + n, dtype=np.uint64)
    c = cos_min + (1. - cos_min) * W.uniform(seed, 1, ev, 1)
    phi = 2. * np.pi * W.uniform(seed, 1, ev, 2)
    st = np.sqrt(1. - c * c)
    s["direction"][:, 0] = st * np.cos(phi)
    s["direction"][:, 1] = st * np.sin(phi)
    s["direction"][:, 2] = -c
    return s


CASES["atmosphere_forward"] = dict(
    config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY, limit_energy=1.),
    geometry=ATMOSPHERE, n=100, seed=31,
    states=lambda n, s, f: _sky_states(n, s, f, 1., 1E+03, 15000.))
CASES["atmosphere_backward"] = dict(
    config=_cfg(STRAGGLED, MIXED, BWD, event=LIMIT_ENERGY,
                limit_energy=1E+05),
    geometry=ATMOSPHERE, n=100, seed=32,
    states=lambda n, s, f: _sky_states(n, s, f, 1., 1E+02, -199.))
CASES["atmosphere_csda"] = dict(
    config=_cfg(CSDA, DISABLED, FWD, decay=DISABLED, event=LIMIT_ENERGY,
                limit_energy=1.),
    geometry=ATMOSPHERE, n=100, seed=33,
    states=lambda n, s, f: _sky_states(n, s, f, 1., 1E+03, 15000.))
CASES["iron_field"] = dict(
    config=_cfg(STRAGGLED, MIXED, FWD),
    geometry=IRON_FIELD, n=200, seed=34,
    states=lambda n, s, f: _states(n, s, f, 1., 1E+02))


# Deterministic CSDA in uniform media with a field: the reference's closed
# form deflection (transport_csda_deflect, pumas.c:4968-5075).
CASES["rock_csda_field"] = dict(
    config=_cfg(CSDA, DISABLED, FWD, decay=DISABLED, event=LIMIT_ENERGY,
                limit_energy=1.),
    geometry=dict(kind=0, media=[("StandardRock", 0.)],
                  locals=[dict(magnet=(0., 5E-03, 0.))]),
    n=200, seed=35,
    states=lambda n, s, f: _states(n, s, f, 1., 1E+04))
# Short tracks: the small rotation branch of the closed form.
CASES["rock_csda_field_distance"] = dict(
    config=_cfg(CSDA, DISABLED, FWD, decay=DISABLED, event=LIMIT_DISTANCE,
                limit_distance=20.),
    geometry=CASES["rock_csda_field"]["geometry"], n=200, seed=37,
    states=lambda n, s, f: _states(n, s, f, 10., 1E+04))
CASES["water_csda_field_backward"] = dict(
    config=_cfg(CSDA, DISABLED, BWD, decay=DISABLED, event=LIMIT_ENERGY,
                limit_energy=1E+04),
    geometry=dict(kind=0, media=[("Water", 0.)],
                  locals=[dict(magnet=(2E-04, 0., 1E-04))]),
    n=200, seed=36,
    states=lambda n, s, f: _states(n, s, f, 1., 1E+02))


# Taus (physics made by pumas_physics_create for PUMAS_PARTICLE_TAU): the
# randomised decay of forward taus through the multi-material stack, with
# straggling, and in rock in closed form CSDA; weighted backward transport
# over 20 m of rock.
CASES["tau_stack_forward"] = dict(
    physics="tau",
    config=_cfg(STRAGGLED, MIXED, FWD, decay=RANDOMISED),
    geometry=STACK, n=200, seed=41,
    states=lambda n, s, f: _states(n, s, f, 1E+05, 1E+08))
CASES["tau_rock_csda_randomised"] = dict(
    physics="tau",
    config=_cfg(CSDA, DISABLED, FWD, decay=RANDOMISED),
    geometry=ROCK, n=200, seed=42,
    states=lambda n, s, f: _states(n, s, f, 1E+02, 1E+06))
CASES["tau_rock_backward"] = dict(
    physics="tau",
    config=_cfg(STRAGGLED, MIXED, BWD, event=LIMIT_DISTANCE,
                limit_distance=20.),
    geometry=ROCK_SLAB, n=200, seed=43,
    states=lambda n, s, f: _states(n, s, f, 1E+04, 1E+06, z0=999.999))


# Non-default DCS models (pumas.h:742-771): KKP bremsstrahlung and pair
# production with BM photonuclear; ABB bremsstrahlung with BBKS
# photonuclear; BBKS for taus.
CASES["models_kkp_rock_slab"] = dict(
    physics="muon_kkp",
    config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY, limit_energy=1.),
    geometry=ROCK_SLAB, n=200, seed=51,
    states=lambda n, s, f: W.rock_slab(n, s, f))
CASES["models_kkp_stack_backward"] = dict(
    physics="muon_kkp",
    config=_cfg(STRAGGLED, MIXED, BWD),
    geometry=STACK, n=150, seed=52,
    states=lambda n, s, f: _states(n, s, f, 1., 1E+04, z0=399.999))
CASES["models_abb_stack_forward"] = dict(
    physics="muon_abb",
    config=_cfg(STRAGGLED, MIXED, FWD, event=LIMIT_ENERGY, limit_energy=1.),
    geometry=STACK, n=200, seed=53,
    states=lambda n, s, f: _states(n, s, f, 1., 1E+04))
CASES["models_bbks_tau_stack"] = dict(
    physics="tau_bbks",
    config=_cfg(STRAGGLED, MIXED, FWD, decay=RANDOMISED),
    geometry=STACK, n=200, seed=54,
    states=lambda n, s, f: _states(n, s, f, 1E+05, 1E+08))


def particle(name):
    """Physics of a case: "muon" (default), "tau", or a physics with
    non-default DCS models ("muon_kkp", "muon_abb", "tau_bbks")."""
    return CASES[name].get("physics", "muon")


# Physics with non-default DCS models: their GPU golden cases run in
# tests/test_zy_models.py, after the other GPU tests.
MODEL_PHYSICS = ("muon_kkp", "muon_abb", "tau_bbks")


def has_models(name):
    return particle(name) in MODEL_PHYSICS


def physics_dump(name):
    """Bytes of a physics dump: the shipped muon and tau dumps, or the test
    fixtures with non-default DCS models (tests/golden/physics_*.pumas.gz,
    made by tests/golden/make_golden.py physics)."""
    import gzip
    import os
    from pumas_gb300 import default_dump
    if name in ("muon", "tau"):
        return default_dump(name)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                        "physics_%s.pumas.gz" % name)
    with gzip.open(path, "rb") as f:
        return f.read()


def has_locals(name):
    """Whether a case's media have local properties (density profiles,
    magnetic fields)."""
    return CASES[name]["geometry"].get("locals") is not None


def make_states(name, n=None, first_event=0):
    c = CASES[name]
    return c["states"](c["n"] if n is None else n, c["seed"], first_event)


def material_indices(index_of, geometry):
    return [(index_of(m), d) for m, d in geometry["media"]]


# Events transported over several calls (the carry of gpumas_result): the
# two-regime loop of examples/pumas/geometry.c:269-312. Backward muons from a
# detector at the bottom of a rock layer under the atmosphere: below 100 GeV
# a detailed simulation (straggled energy loss, mixed scattering, energy
# limit 100 GeV), above it a fast one (mixed energy loss, no scattering, up
# to 1000 times the largest detector energy); the loop ends when the muon
# leaves the geometry or reaches that energy. Each call continues the
# random stream and Box-Muller cache of the event's previous call, as one
# reference context per event does.
FLT_EPSILON = 1.1920928955078125E-07
CHAIN = dict(
    geometry=dict(kind=1, media=[("StandardRock", 0.), ("Air", 0.)],
                  slab_z=[0., 90., 10000.], slab_media=[0, 1]),
    n=200, seed=61, first_event=4000, energy_min=1., energy_max=1E+03)
CHAIN_THRESHOLD = CHAIN["energy_max"] * 1E+03
CHAIN_LOW = _cfg(STRAGGLED, MIXED, BWD, event=LIMIT_ENERGY,
                 limit_energy=1E+02)
CHAIN_HIGH = _cfg(MIXED, DISABLED, BWD, event=LIMIT_ENERGY,
                  limit_energy=CHAIN_THRESHOLD)


def chain_states(n=None, seed=None, first=None):
    """Detector muons as examples/pumas/geometry.c:227-253 draws them: energy
    log-uniform with weight kf ln(Emax / Emin) times 2 for the charge, random
    charge, direction at an elevation drawn here uniformly in [5, 90] deg."""
    c = CHAIN
    n = c["n"] if n is None else n
    seed = c["seed"] if seed is None else seed
    first = c["first_event"] if first is None else first
    ev = np.arange(first, first + n, dtype=np.uint64)
    rk = np.log(c["energy_max"] / c["energy_min"])
    kf = c["energy_min"] * np.exp(rk * W.uniform(seed, 1, ev, 0))
    # Energies within FLT_EPSILON below 100 GeV would take the fast regime
    # at once in the loop of the example; keep them out of the sample.
    kf = np.where(np.abs(kf - 1E+02) < 1E-05, 1.01E+02, kf)
    elev = np.radians(5. + 85. * W.uniform(seed, 1, ev, 1))
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(W.uniform(seed, 1, ev, 2) > 0.5, 1., -1.)
    s["energy"] = kf
    s["weight"] = kf * rk * 2.
    cos_theta = np.cos(0.5 * np.pi - elev)
    s["direction"][:, 0] = -np.sqrt(1. - cos_theta * cos_theta)
    s["direction"][:, 2] = -cos_theta
    return s


def run_chain(transport, states, max_calls=16):
    """Run the loop of examples/pumas/geometry.c:269-312 over a batch.

    `transport(config, states, results)` transports every event of the
    batch with a carrying context of settings `config` and returns the new
    (states, results). The loop calls the detailed and the fast settings in
    turn on the whole batch. In a call whose regime does not apply to an
    event, the event returns at once without a random draw: above the
    energy limit of a backward transport (transport_limit,
    pumas.c:5576-5596) or outside the geometry (pumas.c:3187-3195). So each
    event sees the same sequence of effective calls as in the example's
    per-event loop. Returns (states, results, calls)."""
    from pumas_gb300 import RESULT_DTYPE
    s = np.array(states, copy=True)
    r = np.zeros(len(s), dtype=RESULT_DTYPE)
    calls = 0
    while calls < max_calls:
        for cfg in (CHAIN_LOW, CHAIN_HIGH):
            s, r = transport(cfg, s, r)
            calls += 1
        out = (r["event"] == 16) & (r["medium_out"] == -1)
        done = out | (s["energy"] >= CHAIN_THRESHOLD - FLT_EPSILON)
        if np.all(done):
            break
    return s, r, calls
