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
* ``atmosphere``: muons from the sky through an exponential atmosphere with
  the geomagnetic field into rock, see ``atmosphere_geometry``.
"""
import numpy as np

from . import (MODE_BACKWARD, MODE_CSDA, MODE_DISABLED, MODE_FORWARD,
               MODE_MIXED, MODE_STRAGGLED, MODE_WEIGHTED, EVENT_LIMIT_ENERGY,
               EVENT_NONE, STATE_DTYPE, DENSITY_EXPONENTIAL, Geometry)

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


# The exponential atmosphere of the reference's examples/pumas/geometry.c
# (76-97): 1.205 kg/m^3 at sea level, 12 km scale height, geomagnetic field
# (0, 20, -40) uT, over 200 m of rock, up to 20 km.
ATMOSPHERE_LOCALS = dict(model=DENSITY_EXPONENTIAL, rho0=1.205,
                         axis=(0., 0., 1.), h0=0., lambda_=12E+03,
                         eps=5E-02, magnet=(0., 2E-05, -4E-05))
ATMOSPHERE_Z = (-200., 0., 20E+03)


def atmosphere_geometry(physics_or_index):
    """Two slabs: StandardRock (uniform) under the atmosphere (Air with the
    exponential density and the field)."""
    rock = _material(physics_or_index, "StandardRock")
    air = _material(physics_or_index, "Air")
    return Geometry.slabs(list(ATMOSPHERE_Z), [rock, air],
                          locals=[dict(), dict(ATMOSPHERE_LOCALS)])


def atmosphere_spec():
    """The atmosphere geometry as a plain dict (for oracles and tests)."""
    return dict(kind=1, media=[("StandardRock", 0.), ("Air", 0.)],
                slab_z=list(ATMOSPHERE_Z), slab_media=[0, 1],
                locals=[dict(), dict(ATMOSPHERE_LOCALS)])


def atmosphere(n, seed=1, first_event=0, emin=1., emax=1E+03, z0=15E+03):
    """Initial states of the atmosphere workload: mu+ / mu- by event id
    parity at altitude z0 with momenta pointing down, zenith angle cosine
    uniform in [0.2, 1], uniform azimuth, kinetic energy log-uniform in
    [emin, emax]."""
    ev = np.arange(first_event, first_event + n, dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.)
    s["energy"] = _log_uniform(seed, ev, 0, emin, emax)
    s["weight"] = 1.
    s["position"][:, 2] = z0
    c = 0.2 + 0.8 * uniform(seed, 1, ev, 1)
    phi = 2. * np.pi * uniform(seed, 1, ev, 2)
    st = np.sqrt(1. - c * c)
    s["direction"][:, 0] = st * np.cos(phi)
    s["direction"][:, 1] = st * np.sin(phi)
    s["direction"][:, 2] = -c
    return s


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
    if kind == "atmosphere":
        return dict(energy_loss=MODE_STRAGGLED, decay=MODE_WEIGHTED,
                    direction=MODE_FORWARD, scattering=MODE_MIXED,
                    event=EVENT_LIMIT_ENERGY, limit_energy=1.,
                    accuracy=1E-02)
    if kind == "terrain":
        # Backward transport stops on leaving the geometry (z = 3 km) or,
        # for near horizontal tracks through kilometres of rock, when the
        # energy reaches the top of the tables (1e8 GeV): beyond it the
        # muon flux weight is negligible and the reference's hard elastic
        # scatter sampling (pumas.c:5839-5864) practically never accepts.
        return dict(energy_loss=MODE_STRAGGLED, decay=MODE_WEIGHTED,
                    direction=MODE_BACKWARD, scattering=MODE_MIXED,
                    event=EVENT_LIMIT_ENERGY, limit_energy=TERRAIN_EMAX,
                    accuracy=1E-02)
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


# ---------------------------------------------------------------------------
# Backward muography over a synthetic terrain.
# ---------------------------------------------------------------------------
TERRAIN_N = 512          # nodes per side
TERRAIN_CELL = 10.       # m
TERRAIN_PEAK = 800.      # m, height of the Gaussian hill
TERRAIN_SIGMA = 1500.    # m
TERRAIN_NOISE = 5.       # m, i.i.d. Gaussian noise before smoothing
TERRAIN_ZTOP = 3000.     # m, end of the transport (no medium above)
TERRAIN_DEPTH = 20.      # m, detector depth below the surface
TERRAIN_EMAX = 1E+08     # GeV, backward energy limit (top of the tables)
FLUX_NORM = 0.14         # GeV^-1 cm^-2 s^-1 sr^-1 at 1 GeV
FLUX_INDEX = 2.7


def _normal(seed, domain, events, draw):
    """Standard normal deviates from two uniforms (Box-Muller)."""
    u1 = uniform(seed, domain, events, 2 * draw)
    u2 = uniform(seed, domain, events, 2 * draw + 1)
    return np.sqrt(-2. * np.log(u1)) * np.cos(2. * np.pi * u2)


def terrain_heights(seed=3, n=TERRAIN_N, cell=TERRAIN_CELL):
    """Heightmap of the terrain workload: a Gaussian hill (peak 800 m,
    sigma 1.5 km) centred on the grid, plus i.i.d. N(0, 5 m) noise from the
    Philox stream of (seed, domain 3, node index), smoothed by a 3 x 3 box
    (edge nodes averaged over their in-grid neighbours). Returns (heights
    [n, n] indexed [y, x], x0, y0)."""
    x0 = -0.5 * (n - 1) * cell
    x = x0 + cell * np.arange(n)
    xx, yy = np.meshgrid(x, x)
    hill = TERRAIN_PEAK * np.exp(-(xx ** 2 + yy ** 2) /
                                 (2. * TERRAIN_SIGMA ** 2))
    nodes = np.arange(n * n, dtype=np.uint64)
    noise = TERRAIN_NOISE * _normal(seed, 3, nodes, 0).reshape(n, n)
    z = hill + noise
    acc = np.zeros_like(z)
    cnt = np.zeros_like(z)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            ys = slice(max(dy, 0), n + min(dy, 0))
            yd = slice(max(-dy, 0), n + min(-dy, 0))
            xs = slice(max(dx, 0), n + min(dx, 0))
            xd = slice(max(-dx, 0), n + min(-dx, 0))
            acc[yd, xd] += z[ys, xs]
            cnt[yd, xd] += 1.
    return acc / cnt, x0, x0


def terrain_geometry(physics_or_index, seed=3, n=TERRAIN_N):
    """Heightmap geometry: StandardRock below the surface, Air above, no
    medium above 3 km."""
    h, x0, y0 = terrain_heights(seed, n)
    rock = _material(physics_or_index, "StandardRock")
    air = _material(physics_or_index, "Air")
    return Geometry.heightmap(h, x0, y0, TERRAIN_CELL, TERRAIN_CELL,
                              (rock, 0.), (air, 0.), TERRAIN_ZTOP)


def terrain_spec(seed=3, n=TERRAIN_N):
    """The terrain geometry as a plain dict (for oracles and tests)."""
    h, x0, y0 = terrain_heights(seed, n)
    return dict(kind=2, media=[("StandardRock", 0.), ("Air", 0.)],
                hm_z=h, hm_x0=x0, hm_y0=y0, hm_dx=TERRAIN_CELL,
                hm_dy=TERRAIN_CELL, hm_below=0, hm_above=1,
                hm_ztop=TERRAIN_ZTOP)


def surface_height(h, x0, y0, cell, x, y):
    """Bilinear surface height (the rule of gpumas_geometry.h)."""
    fx, fy = (x - x0) / cell, (y - y0) / cell
    i, j = int(fx), int(fy)
    s, r = fx - i, fy - j
    a = h[j, i] + s * (h[j, i + 1] - h[j, i])
    b = h[j + 1, i] + s * (h[j + 1, i + 1] - h[j + 1, i])
    return a + r * (b - a)


def terrain_directions(n_zenith=32, n_azimuth=64, zmax=85.):
    """Bin centres of the direction grid: (zenith, azimuth) in radians,
    zenith bins over [0, zmax] deg, azimuth bins over [0, 360] deg."""
    dz = zmax / n_zenith
    za = np.radians(dz * (np.arange(n_zenith) + 0.5))
    az = np.radians(360. / n_azimuth * (np.arange(n_azimuth) + 0.5))
    zz, aa = np.meshgrid(za, az, indexing="ij")
    return zz.ravel(), aa.ravel()


def terrain(n_per_direction, seed=1, first_event=0, directions=None,
            heights=None, emin=1., emax=1E+05):
    """Initial states of the terrain workload: for each direction of the
    grid, n_per_direction muons at the detector (20 m below the surface at
    the grid centre) with momentum pointing down along the direction (they
    come from the sky), kinetic energy log-uniform in [emin, emax], weight
    1 / pdf(K), mu+ / mu- by event id parity. Event ids run direction by
    direction from first_event. Returns (states, direction index)."""
    if heights is None:
        heights = terrain_heights()
    h, x0, y0 = heights
    if directions is None:
        directions = terrain_directions()
    zen, azi = directions
    nd = len(zen)
    n = nd * n_per_direction
    ev = np.arange(first_event, first_event + n, dtype=np.uint64)
    d = np.repeat(np.arange(nd), n_per_direction)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.)
    u = uniform(seed, 1, ev, 0)
    lr = np.log(emax / emin)
    k = emin * np.exp(lr * u)
    s["energy"] = k
    s["weight"] = k * lr
    zd = surface_height(h, x0, y0, TERRAIN_CELL, 0., 0.) - TERRAIN_DEPTH
    s["position"][:, 2] = zd
    st = np.sin(zen[d])
    s["direction"][:, 0] = -st * np.cos(azi[d])
    s["direction"][:, 1] = -st * np.sin(azi[d])
    s["direction"][:, 2] = -np.cos(zen[d])
    return s, d


def terrain_flux(final, results, direction_index, n_directions):
    """Muon flux per direction (per cm^2 s sr) from backward transported
    events: mean over events of weight x 0.14 E^-2.7 cos(theta), with E the
    total energy and theta the zenith angle at the end point, for events
    that reached the top of the geometry."""
    from . import EVENT_MEDIUM
    e_total = final["energy"] + 0.10565839
    cos_t = np.clip(-final["direction"][:, 2], 0., 1.)
    ok = (results["event"] == EVENT_MEDIUM) & (results["medium_out"] == -1)
    w = np.where(ok, final["weight"] * FLUX_NORM *
                 e_total ** -FLUX_INDEX * cos_t, 0.)
    tot = np.bincount(direction_index, weights=w, minlength=n_directions)
    cnt = np.bincount(direction_index, minlength=n_directions)
    return tot / np.maximum(cnt, 1)


# ---------------------------------------------------------------------------
# Batched uneven jobs: slab stacks of rock, water and iron.
# ---------------------------------------------------------------------------
JOB_MATERIALS = ("StandardRock", "Water", "Iron")


def slab_jobs(n_jobs=8192, seed=5, event_scale=1.):
    """Job descriptions of the batched workload, drawn from the Philox
    stream of (seed, domain 2, job index):

    * 1 to 8 slabs stacked from z = 0 up, each of StandardRock, Water or
      Iron (uniform) with a thickness log-uniform in [1 m, 2 km];
    * events log-uniform in [1e2, 1e6] (times event_scale, at least 1);
    * Emin log-uniform in [1, 100] GeV, Emax = 1000 Emin;
    * forward or backward with probability 1/2. Forward muons start at
      z = 0 going up and stop on exit or at 1 GeV; backward ones are
      detected at z = 0 coming down and are transported back up to the
      exit or to 1e7 GeV.

    Straggled energy loss, mixed scattering, weighted decay. Returns a list
    of dicts (slab boundaries, material names, n, emin, emax, direction,
    first_event = job index x 2^32)."""
    jobs = []
    idx = np.arange(n_jobs, dtype=np.uint64)
    u = [uniform(seed, 2, idx, k) for k in range(6 + 16)]
    for j in range(n_jobs):
        ns = 1 + min(int(8 * u[0][j]), 7)
        mats = [JOB_MATERIALS[min(int(3 * u[6 + 2 * k][j]), 2)]
                for k in range(ns)]
        thick = [2000. ** u[7 + 2 * k][j] for k in range(ns)]
        z = np.concatenate([[0.], np.cumsum(thick)])
        n = max(1, int(round(event_scale * 100. * 1E+04 ** u[1][j])))
        emin = 100. ** u[2][j]
        jobs.append(dict(slab_z=z, materials=mats, n=n, emin=emin,
                         emax=1E+03 * emin,
                         direction=MODE_FORWARD if u[3][j] < 0.5 else
                         MODE_BACKWARD,
                         first_event=int(j) << 32))
    return jobs


def slab_job_config(job):
    c = dict(energy_loss=MODE_STRAGGLED, decay=MODE_WEIGHTED,
             direction=job["direction"], scattering=MODE_MIXED,
             event=EVENT_LIMIT_ENERGY, accuracy=1E-02)
    c["limit_energy"] = 1. if job["direction"] == MODE_FORWARD else 1E+07
    return c


def slab_job_geometry(physics, job):
    mats = [physics.material_index(m) for m in job["materials"]]
    return Geometry.slabs(list(job["slab_z"]), mats)


def slab_job_states(job, seed=5):
    """Initial states of a job: kinetic energy log-uniform in
    [emin, emax] (Philox domain 1 of the event ids), at z = 0, going up
    (forward) or coming down (backward), mu+ / mu- by event id parity."""
    n = job["n"]
    ev = np.arange(job["first_event"], job["first_event"] + n,
                   dtype=np.uint64)
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["charge"] = np.where(ev % 2 == 1, 1., -1.)
    s["energy"] = _log_uniform(seed, ev, 0, job["emin"], job["emax"])
    s["weight"] = 1.
    s["direction"][:, 2] = 1. if job["direction"] == MODE_FORWARD else -1.
    return s
