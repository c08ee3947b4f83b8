"""Synthetic transport workloads (initial states and geometries).

Initial states are sampled from draws of the Philox-4x32-10 stream in
domain 1 (the transport itself uses domain 0), keyed by (seed, event id),
so that any subset of events can be regenerated independently:

* ``plain_csda``: mu- at the origin along +z in infinite StandardRock,
  kinetic energy log-uniform in [10 GeV, 10 TeV], CSDA energy loss, no
  scattering, no decay, stop at 1 GeV.
* ``rock_slab``: mu+ (odd event id) / mu- (even) entering a 1 km StandardRock
  slab at z = 0 along +z, vacuum outside, kinetic energy log-uniform in
  [10 GeV, 100 TeV], straggled loss, mixed scattering, weighted decay, stop
  at 1 GeV or on exit.
* ``terrain``: backward transport from a detector under a synthetic
  heightmap, see ``terrain_geometry``.
* ``slab_jobs``: batched uneven jobs of slab stacks, see ``slab_jobs``.
"""
import numpy as np

from . import (MODE_BACKWARD, MODE_CSDA, MODE_DISABLED, MODE_FORWARD,
               MODE_MIXED, MODE_STRAGGLED, MODE_WEIGHTED, EVENT_LIMIT_ENERGY,
               EVENT_NONE, STATE_DTYPE, Geometry)

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox-4x32-10 over uint64 arrays holding 32 bit words."""
    c0, c1, c2, c3 = [np.asarray(c, dtype=np.uint64) & MASK
                      for c in (c0, c1, c2, c3)]
    k0 = np.uint64(k0) & MASK
    k1 = np.uint64(k1) & MASK
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0), lo1, (hi0 ^ c3 ^ k1), lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def uniform(seed, domain, events, n):
    """Draw n (scalar) of the streams of `events` in `domain`."""
    events = np.asarray(events, dtype=np.uint64)
    block = np.full(events.shape, n >> 1, dtype=np.uint64)
    x0, x1, x2, x3 = philox4x32_10(
        block, np.full(events.shape, domain, dtype=np.uint64),
        events & MASK, events >> np.uint64(32), seed & 0xFFFFFFFF,
        (seed >> 32) & 0xFFFFFFFF)
    w = (x3 << np.uint64(32)) | x2 if (n & 1) else (x1 << np.uint64(32)) | x0
    return ((w >> np.uint64(12)).astype(np.float64) + 0.5) * 2.0 ** -52


def _log_uniform(seed, events, draw, lo, hi):
    return lo * (hi / lo) ** uniform(seed, 1, events, draw)


def plain_csda(n, seed=1, first_event=0):
    """Initial states of the plain CSDA workload (infinite rock)."""
    ev = np.arange(first_event, first_event + n, dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = -1.
    s["energy"] = _log_uniform(seed, ev, 0, 10., 1E+04)
    s["weight"] = 1.
    s["direction"][:, 2] = 1.
    return s


def plain_csda_config(ctx):
    ctx.mode.energy_loss = MODE_CSDA
    ctx.mode.scattering = MODE_DISABLED
    ctx.mode.decay = MODE_DISABLED
    ctx.mode.direction = MODE_FORWARD
    ctx.event = EVENT_LIMIT_ENERGY
    ctx.limit.energy = 1.


def rock_slab(n, seed=1, first_event=0):
    """Initial states of the 1 km rock slab workload."""
    ev = np.arange(first_event, first_event + n, dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.)
    s["energy"] = _log_uniform(seed, ev, 0, 10., 1E+05)
    s["weight"] = 1.
    s["direction"][:, 2] = 1.
    return s


def rock_slab_config(ctx):
    ctx.mode.energy_loss = MODE_STRAGGLED
    ctx.mode.scattering = MODE_MIXED
    ctx.mode.decay = MODE_WEIGHTED
    ctx.mode.direction = MODE_FORWARD
    ctx.event = EVENT_LIMIT_ENERGY
    ctx.limit.energy = 1.


def rock_slab_geometry(physics_or_index):
    rock = _material(physics_or_index, "StandardRock")
    return Geometry.slabs([0., 1000.], [rock])


def _material(physics_or_index, name):
    if isinstance(physics_or_index, dict):
        return physics_or_index[name]
    return physics_or_index.material_index(name)


def config_dict(kind):
    """The context settings of a workload as a plain dict (for oracles)."""
    if kind == "plain_csda":
        return dict(energy_loss=MODE_CSDA, decay=-1, direction=MODE_FORWARD,
                    scattering=MODE_DISABLED, event=EVENT_LIMIT_ENERGY,
                    limit_energy=1., accuracy=1E-02)
    if kind == "rock_slab":
        return dict(energy_loss=MODE_STRAGGLED, decay=MODE_WEIGHTED,
                    direction=MODE_FORWARD, scattering=MODE_MIXED,
                    event=EVENT_LIMIT_ENERGY, limit_energy=1.,
                    accuracy=1E-02)
    if kind == "terrain":
        return dict(energy_loss=MODE_STRAGGLED, decay=MODE_WEIGHTED,
                    direction=MODE_BACKWARD, scattering=MODE_MIXED,
                    event=EVENT_NONE, limit_energy=0., accuracy=1E-02)
    raise KeyError(kind)


def apply_config(ctx, cfg):
    ctx.mode.energy_loss = cfg["energy_loss"]
    ctx.mode.decay = cfg["decay"]
    ctx.mode.direction = cfg["direction"]
    ctx.mode.scattering = cfg["scattering"]
    ctx.event = cfg["event"]
    ctx.limit.energy = cfg.get("limit_energy", 0.)
    ctx.limit.distance = cfg.get("limit_distance", 0.)
    ctx.limit.grammage = cfg.get("limit_grammage", 0.)
    ctx.limit.time = cfg.get("limit_time", 0.)
    ctx.accuracy = cfg.get("accuracy", 1E-02)
