"""pumas_gb300 -- GB300 engine for the PUMAS muon transport hot path.

Python mirror of the reference's transport API (include/pumas.h) over the C
ABI of libgpumas.so (include/gpumas.h):

* ``Physics``: the physics tables, loaded from a ``pumas_physics_dump``
  stream as produced by the reference's ``pumas_physics_create`` (the
  package ships one for the materials of data/materials.xml);
* ``Context``: the ``pumas_context`` settings (``mode.energy_loss``,
  ``mode.decay``, ``mode.direction``, ``mode.scattering``, ``event``,
  ``limit.*``, ``accuracy``) plus a geometry descriptor and a Philox seed in
  place of the medium and random callbacks;
* ``Context.transport(states)``: ``pumas_context_transport`` over an array
  of ``pumas_state`` records, on the GPU.

There is no CPU fallback: if the CUDA library is not built or no device is
usable, the calls raise.
"""
import ctypes
import gzip
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(HERE, "data")
DEFAULT_DUMP = os.path.join(DATA, "muon.pumas.gz")
TAU_DUMP = os.path.join(DATA, "tau.pumas.gz")
PARTICLE_MUON, PARTICLE_TAU = 0, 1

# enum pumas_mode / pumas_event / pumas_return values (pumas.h:90-196).
MODE_DISABLED, MODE_CSDA, MODE_MIXED, MODE_STRAGGLED = -1, 0, 1, 2
MODE_WEIGHTED, MODE_RANDOMISED = 0, 1
MODE_FORWARD, MODE_BACKWARD = 0, 1
EVENT_NONE, EVENT_LIMIT_ENERGY, EVENT_LIMIT_DISTANCE = 0, 1, 2
EVENT_LIMIT_GRAMMAGE, EVENT_LIMIT_TIME, EVENT_LIMIT = 4, 8, 15
EVENT_MEDIUM = 16
EVENT_VERTEX_BREMSSTRAHLUNG, EVENT_VERTEX_PAIR_CREATION = 32, 64
EVENT_VERTEX_PHOTONUCLEAR, EVENT_VERTEX_DELTA_RAY = 128, 256
EVENT_VERTEX_DEL, EVENT_VERTEX_COULOMB, EVENT_VERTEX_DECAY = 480, 512, 1024
EVENT_VERTEX, EVENT_WEIGHT = 2016, 2048
RETURN_SUCCESS, RETURN_ACCURACY_ERROR, RETURN_DECAY_ERROR = 0, 1, 3
RETURN_DENSITY_ERROR, RETURN_DIRECTION_ERROR = 4, 5
RETURN_INDEX_ERROR, RETURN_PHYSICS_ERROR, RETURN_INTERNAL_ERROR = 7, 8, 9
RETURN_FORMAT_ERROR, RETURN_MEDIUM_ERROR, RETURN_MEMORY_ERROR = 11, 12, 13
RETURN_MODEL_ERROR, RETURN_MISSING_LIMIT = 14, 15
RETURN_UNKNOWN_MATERIAL, RETURN_UNKNOWN_PARTICLE = 22, 23
RETURN_RAISE_ERROR, RETURN_VALUE_ERROR = 18, 24
RETURN_DEVICE_ERROR = 64

GEOMETRY_UNIFORM, GEOMETRY_SLABS, GEOMETRY_HEIGHTMAP = 0, 1, 2
DENSITY_UNIFORM, DENSITY_EXPONENTIAL = 0, 1

# struct pumas_state (pumas.h:289-309), padded to 8 bytes.
STATE_DTYPE = np.dtype([
    ("charge", "f8"), ("energy", "f8"), ("distance", "f8"),
    ("grammage", "f8"), ("time", "f8"), ("weight", "f8"),
    ("position", "f8", 3), ("direction", "f8", 3), ("decayed", "i4"),
    ("pad", "i4")])
RESULT_DTYPE = np.dtype([
    ("event", "i4"), ("medium_in", "i4"), ("medium_out", "i4"),
    ("status", "i4"), ("steps", "i4"), ("randn_done", "i4"),
    ("draws", "u8"), ("randn_next", "f8")])
# struct gpumas_frame: a recorded state, its medium index and event flags.
FRAME_DTYPE = np.dtype([("state", STATE_DTYPE), ("medium", "i4"),
                        ("event", "i4")])
EVENT_START, EVENT_STOP = 4096, 8192


class PumasError(RuntimeError):
    """A non-success return code of the engine."""

    def __init__(self, code, where=""):
        self.code = code
        super().__init__("%s: return code %d" % (where, code))


class _Medium(ctypes.Structure):
    _fields_ = [("material", ctypes.c_int), ("density", ctypes.c_double)]


class _Locals(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("rho0", ctypes.c_double),
                ("axis", ctypes.c_double * 3), ("h0", ctypes.c_double),
                ("lambda_", ctypes.c_double), ("eps", ctypes.c_double),
                ("magnet", ctypes.c_double * 3)]


class _Geometry(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("n_media", ctypes.c_int),
        ("media", ctypes.POINTER(_Medium)),
        ("uniform_medium", ctypes.c_int),
        ("n_slabs", ctypes.c_int),
        ("slab_z", ctypes.POINTER(ctypes.c_double)),
        ("slab_medium", ctypes.POINTER(ctypes.c_int)),
        ("hm_nx", ctypes.c_int), ("hm_ny", ctypes.c_int),
        ("hm_x0", ctypes.c_double), ("hm_y0", ctypes.c_double),
        ("hm_dx", ctypes.c_double), ("hm_dy", ctypes.c_double),
        ("hm_z", ctypes.POINTER(ctypes.c_double)),
        ("hm_below", ctypes.c_int), ("hm_above", ctypes.c_int),
        ("hm_ztop", ctypes.c_double),
        ("locals", ctypes.POINTER(_Locals))]


class _Mode(ctypes.Structure):
    _fields_ = [("energy_loss", ctypes.c_int), ("decay", ctypes.c_int),
                ("direction", ctypes.c_int), ("scattering", ctypes.c_int)]


class _Limit(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("distance", ctypes.c_double),
                ("grammage", ctypes.c_double), ("time", ctypes.c_double)]


class _Context(ctypes.Structure):
    _fields_ = [("mode", _Mode), ("event", ctypes.c_int), ("limit", _Limit),
                ("accuracy", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("user_data", ctypes.c_void_p)]


class _Recorder(ctypes.Structure):
    _fields_ = [("period", ctypes.c_int), ("max_frames", ctypes.c_int),
                ("frames", ctypes.c_void_p), ("length", ctypes.c_void_p)]


class _Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int), ("kernel_ms", ctypes.c_double)]


class _Tuning(ctypes.Structure):
    _fields_ = [("engine", ctypes.c_int), ("pool_slots", ctypes.c_int),
                ("max_inner", ctypes.c_int), ("batch", ctypes.c_int),
                ("tail", ctypes.c_int)]


ENGINE_AUTO, ENGINE_PLAIN, ENGINE_POOL = 0, 1, 2


class _Soa(ctypes.Structure):
    _fields_ = [
        ("charge", ctypes.c_void_p), ("energy", ctypes.c_void_p),
        ("distance", ctypes.c_void_p), ("grammage", ctypes.c_void_p),
        ("time", ctypes.c_void_p), ("weight", ctypes.c_void_p),
        ("position", ctypes.c_void_p * 3),
        ("direction", ctypes.c_void_p * 3),
        ("decayed", ctypes.c_void_p), ("result", ctypes.c_void_p)]


class _Job(ctypes.Structure):
    _fields_ = [("context", ctypes.c_void_p), ("n", ctypes.c_size_t),
                ("events", _Soa), ("first_event", ctypes.c_uint64)]


class _EngineStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_longlong),
                ("batches", ctypes.c_longlong),
                ("kernel_ms", ctypes.c_double),
                ("events", ctypes.c_longlong),
                ("budget_used", ctypes.c_size_t)]


_lib = None


def library(build=False):
    """The loaded libgpumas.so (built first if `build`)."""
    global _lib
    if _lib is None:
        if build:
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(
                "libgpumas.so is not built (pumas_gb300.build.build())")
        lib = ctypes.CDLL(_build.LIB)
        vp, sz, i, d = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, \
            ctypes.c_double
        u64 = ctypes.c_uint64
        pp = ctypes.POINTER(ctypes.c_void_p)
        lib.gpumas_physics_load.argtypes = [pp, ctypes.c_char_p, sz]
        lib.gpumas_physics_upload.argtypes = [pp, vp]
        lib.gpumas_physics_destroy.argtypes = [pp]
        lib.gpumas_physics_destroy.restype = None
        lib.gpumas_physics_material_index.argtypes = [
            vp, ctypes.c_char_p, ctypes.POINTER(i)]
        lib.gpumas_physics_info.argtypes = [
            vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(d),
            ctypes.POINTER(d)]
        lib.gpumas_physics_particle.argtypes = [
            vp, ctypes.POINTER(i), ctypes.POINTER(d), ctypes.POINTER(d)]
        lib.gpumas_context_create.argtypes = [
            ctypes.POINTER(ctypes.POINTER(_Context)), vp, i]
        lib.gpumas_context_destroy.argtypes = [
            ctypes.POINTER(ctypes.POINTER(_Context))]
        lib.gpumas_context_destroy.restype = None
        lib.gpumas_context_geometry_set.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(_Geometry)]
        lib.gpumas_context_transport.argtypes = [
            ctypes.POINTER(_Context), sz, vp, vp, u64]
        lib.gpumas_context_transport_device.argtypes = [
            ctypes.POINTER(_Context), sz, ctypes.POINTER(_Soa), u64, vp]
        lib.gpumas_context_stats.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(_Stats)]
        lib.gpumas_context_tuning_set.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(_Tuning)]
        lib.gpumas_context_tuning_get.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(_Tuning)]
        lib.gpumas_context_trials_set.argtypes = [ctypes.POINTER(_Context), i]
        lib.gpumas_context_carry_set.argtypes = [ctypes.POINTER(_Context), i]
        lib.gpumas_context_carry_get.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(i)]
        lib.gpumas_context_trials_get.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(i)]
        lib.gpumas_engine_create.argtypes = [
            pp, vp, ctypes.POINTER(_Tuning), i, sz]
        lib.gpumas_engine_destroy.argtypes = [pp]
        lib.gpumas_engine_destroy.restype = None
        lib.gpumas_engine_submit.argtypes = [
            vp, ctypes.POINTER(_Job), ctypes.POINTER(i)]
        lib.gpumas_engine_submit_host.argtypes = [
            vp, ctypes.POINTER(_Context), sz, vp, vp, u64, ctypes.POINTER(i)]
        lib.gpumas_engine_step.argtypes = [
            vp, i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]
        lib.gpumas_engine_run.argtypes = [vp, sz, ctypes.POINTER(_Job)]
        lib.gpumas_engine_stats.argtypes = [
            vp, ctypes.POINTER(_EngineStats)]
        lib.gpumas_context_recorder_set.argtypes = [
            ctypes.POINTER(_Context), ctypes.POINTER(_Recorder)]
        lib.gpumas_bench_dfma.argtypes = [ctypes.POINTER(ctypes.c_double)]
        lib.gpumas_random_fill.argtypes = [
            u64, ctypes.c_uint32, u64, u64, sz, vp]
        for f in ("gpumas_physics_load", "gpumas_physics_upload",
                  "gpumas_physics_material_index", "gpumas_physics_info",
                  "gpumas_physics_particle",
                  "gpumas_context_create", "gpumas_context_geometry_set",
                  "gpumas_context_transport",
                  "gpumas_context_transport_device", "gpumas_context_stats",
                  "gpumas_context_tuning_set", "gpumas_context_tuning_get",
                  "gpumas_context_trials_set", "gpumas_context_trials_get",
                  "gpumas_context_carry_set", "gpumas_context_carry_get",
                  "gpumas_bench_dfma", "gpumas_random_fill",
                  "gpumas_engine_create", "gpumas_engine_submit",
                  "gpumas_engine_submit_host", "gpumas_engine_step",
                  "gpumas_engine_run", "gpumas_engine_stats",
                  "gpumas_context_recorder_set"):
            getattr(lib, f).restype = i
        _lib = lib
    return _lib


def _check(rc, where):
    if rc != RETURN_SUCCESS:
        raise PumasError(rc, where)


def default_dump(particle="muon"):
    """Bytes of a shipped physics dump (StandardRock, Water, Air, Iron) for
    muons or taus, made by the reference's pumas_physics_create."""
    path = {"muon": DEFAULT_DUMP, "tau": TAU_DUMP}[particle]
    with gzip.open(path, "rb") as f:
        return f.read()


class Physics:
    """Device physics tables (pumas_physics)."""

    def __init__(self, dump=None):
        if dump is None:
            dump = default_dump()
        lib = library()
        self._lib = lib
        self._ptr = ctypes.c_void_p()
        _check(lib.gpumas_physics_load(ctypes.byref(self._ptr), dump,
                                       len(dump)), "gpumas_physics_load")
        self._fill(dump[8:])

    def _fill(self, blob):
        """Sizes and particle of the loaded physics; `blob` starts with the
        struct's header."""
        lib = self._lib
        nm, ne = ctypes.c_int(), ctypes.c_int()
        cut, mass = ctypes.c_double(), ctypes.c_double()
        lib.gpumas_physics_info(self._ptr, ctypes.byref(nm), ctypes.byref(ne),
                                ctypes.byref(cut), ctypes.byref(mass))
        self.n_materials, self.n_elements = nm.value, ne.value
        # Grid sizes from the struct's header (read as gpumas_physics_load
        # does): the energy rows and the DCS sampling points.
        hdr = np.frombuffer(blob, dtype=np.int32, count=11)
        self.n_energies, self.n_table_dcs = int(hdr[1]), int(hdr[9])
        self.cutoff, self.mass = cut.value, mass.value
        part, ctau = ctypes.c_int(), ctypes.c_double()
        _check(lib.gpumas_physics_particle(self._ptr, ctypes.byref(part),
                                           ctypes.byref(ctau), None),
               "gpumas_physics_particle")
        self.particle, self.ctau = part.value, ctau.value

    @classmethod
    def upload(cls, address):
        """Physics from a live struct pumas_physics at a host address
        (gpumas_physics_upload)."""
        self = cls.__new__(cls)
        lib = library()
        self._lib = lib
        self._ptr = ctypes.c_void_p()
        _check(lib.gpumas_physics_upload(ctypes.byref(self._ptr),
                                         ctypes.c_void_p(address)),
               "gpumas_physics_upload")
        size = int(np.frombuffer((ctypes.c_char * 4).from_address(address),
                                 dtype=np.int32)[0])
        self._fill((ctypes.c_char * size).from_address(address).raw)
        return self

    def tabulate(self):
        """Tabulate on the device the per element DEL tables of this
        physics (gpumas_physics_tabulate): CSn and CSn_dK [4, n_elements,
        n_energies], DCS tables [3, n_elements, n_energies, n_table_dcs, 2],
        envelope exponents [3, n_elements, n_energies], and the device time
        in ms."""
        ne = self.n_energies
        nx = self.n_table_dcs
        nel = self.n_elements
        csn = np.zeros((4, nel, ne))
        dk = np.zeros((4, nel, ne))
        dcs = np.zeros((3, nel, ne, nx, 2), dtype=np.float32)
        alpha = np.zeros((3, nel, ne), dtype=np.float32)
        ms = ctypes.c_float(0.)
        f = self._lib.gpumas_physics_tabulate
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.POINTER(ctypes.c_float)]
        _check(f(self._ptr, csn.ctypes.data, dk.ctypes.data, dcs.ctypes.data,
                 alpha.ctypes.data, ctypes.byref(ms)),
               "gpumas_physics_tabulate")
        return {"csn": csn, "csn_dk": dk, "dcs": dcs, "alpha": alpha,
                "ms": ms.value}

    def material_index(self, name):
        idx = ctypes.c_int(-1)
        _check(self._lib.gpumas_physics_material_index(
            self._ptr, name.encode(), ctypes.byref(idx)),
            "gpumas_physics_material_index")
        return idx.value

    def __del__(self):
        if getattr(self, "_ptr", None):
            self._lib.gpumas_physics_destroy(ctypes.byref(self._ptr))


class Geometry:
    """A geometry descriptor (include/gpumas_geometry.h).

    `media` is a list of (material index, density in kg/m^3 or 0 for the
    material's default). `locals`, if given, holds one dict per medium
    (struct gpumas_locals): ``model`` (DENSITY_UNIFORM or
    DENSITY_EXPONENTIAL), ``rho0``, ``axis``, ``h0``, ``lambda_``, ``eps``
    for the density profile rho0 exp(-(axis . r - h0) / lambda_), and
    ``magnet``, a uniform field in T."""

    def __init__(self, kind, media, locals=None, **kw):
        self._keep = []
        g = _Geometry()
        g.kind = kind
        m = (_Medium * len(media))(*[_Medium(int(a), float(b))
                                     for a, b in media])
        self._keep.append(m)
        g.n_media, g.media = len(media), m
        g.uniform_medium = int(kw.get("medium", 0))
        if kind == GEOMETRY_SLABS:
            z = np.ascontiguousarray(kw["z"], dtype=np.float64)
            sm = np.ascontiguousarray(kw["slab_media"], dtype=np.int32)
            self._keep += [z, sm]
            g.n_slabs = len(sm)
            g.slab_z = z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            g.slab_medium = sm.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        elif kind == GEOMETRY_HEIGHTMAP:
            hz = np.ascontiguousarray(kw["heights"], dtype=np.float64)
            self._keep.append(hz)
            g.hm_ny, g.hm_nx = hz.shape
            g.hm_x0, g.hm_y0 = kw["x0"], kw["y0"]
            g.hm_dx, g.hm_dy = kw["dx"], kw["dy"]
            g.hm_z = hz.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            g.hm_below, g.hm_above = kw["below"], kw["above"]
            g.hm_ztop = kw["ztop"]
        if locals is not None:
            if len(locals) != len(media):
                raise ValueError("one locals entry per medium")
            arr = (_Locals * len(media))()
            for a, d in zip(arr, locals):
                a.model = int(d.get("model", DENSITY_UNIFORM))
                a.rho0 = float(d.get("rho0", 0.))
                a.axis[:] = [float(v) for v in d.get("axis", (0., 0., 1.))]
                a.h0 = float(d.get("h0", 0.))
                a.lambda_ = float(d.get("lambda_", 0.))
                a.eps = float(d.get("eps", 0.))
                a.magnet[:] = [float(v) for v in d.get("magnet", (0., 0., 0.))]
            self._keep.append(arr)
            g.locals = arr
        self.c = g

    @classmethod
    def uniform(cls, material, density=0.):
        return cls(GEOMETRY_UNIFORM, [(material, density)], medium=0)

    @classmethod
    def slabs(cls, z, materials, densities=None, locals=None):
        densities = densities or [0.] * len(materials)
        media = list(zip(materials, densities))
        return cls(GEOMETRY_SLABS, media, locals=locals, z=z,
                   slab_media=list(range(len(materials))))

    @classmethod
    def heightmap(cls, heights, x0, y0, dx, dy, below, above, ztop):
        media = [below, above]
        return cls(GEOMETRY_HEIGHTMAP, media, heights=heights, x0=x0, y0=y0,
                   dx=dx, dy=dy, below=0, above=1, ztop=ztop)


def new_states(n):
    """A zeroed array of pumas_state records with unit weight."""
    s = np.zeros(n, dtype=STATE_DTYPE)
    s["weight"] = 1.
    return s


class Context:
    """A simulation context (pumas_context) on the GPU."""

    def __init__(self, physics):
        self.physics = physics
        self._lib = physics._lib
        self._ptr = ctypes.POINTER(_Context)()
        _check(self._lib.gpumas_context_create(
            ctypes.byref(self._ptr), physics._ptr, 0),
            "gpumas_context_create")
        self._c = self._ptr.contents
        self.mode = self._c.mode
        self.limit = self._c.limit
        self.geometry = None

    event = property(lambda self: self._c.event,
                     lambda self, v: setattr(self._c, "event", int(v)))
    accuracy = property(lambda self: self._c.accuracy,
                        lambda self, v: setattr(self._c, "accuracy",
                                                float(v)))
    seed = property(lambda self: self._c.seed,
                    lambda self, v: setattr(self._c, "seed", int(v)))

    def random_seed_set(self, seed=None):
        """Set the random stream's key (pumas_context_random_seed_set); with
        None, a key drawn from the OS random stream. Returns the key."""
        lib = self._lib
        f = lib.gpumas_context_random_seed_set
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(_Context),
                      ctypes.POINTER(ctypes.c_uint64)]
        key = None if seed is None else ctypes.byref(ctypes.c_uint64(seed))
        _check(f(self._ptr, key), "gpumas_context_random_seed_set")
        return self.seed

    def set_geometry(self, geometry):
        _check(self._lib.gpumas_context_geometry_set(
            self._ptr, ctypes.byref(geometry.c)),
            "gpumas_context_geometry_set")
        self.geometry = geometry

    def transport(self, states, first_event=0, check=False, results=None):
        """Transport a copy of `states`; returns (states, results). With
        `check`, a non-success per event return code raises. With `carry`
        set, each event continues the random state of `results` (those of
        its previous call; zeros for a first call)."""
        s = np.array(states, dtype=STATE_DTYPE, copy=True, order="C")
        if results is None:
            r = np.zeros(len(s), dtype=RESULT_DTYPE)
        else:
            r = np.array(results, dtype=RESULT_DTYPE, copy=True, order="C")
        rc = self._lib.gpumas_context_transport(
            self._ptr, len(s), s.ctypes.data, r.ctypes.data, first_event)
        if rc != RETURN_SUCCESS and (check or rc >= RETURN_DEVICE_ERROR or
                                     not np.any(r["status"] == rc)):
            raise PumasError(rc, "gpumas_context_transport")
        return s, r

    def transport_record(self, states, first_event=0, period=1,
                         max_frames=64):
        """Transport a copy of `states` with the device frame recorder
        (pumas_recorder: `period` 1 records every step, <= 0 only starts,
        stops, DELs and medium changes). Returns (states, results, frames
        [n, max_frames] of FRAME_DTYPE, frame counts); an event with more
        than max_frames frames keeps its first max_frames ones."""
        import torch
        n = len(states)
        dev = torch.device("cuda", torch.cuda.current_device())
        frames = torch.zeros((max(n, 1), max_frames * FRAME_DTYPE.itemsize),
                             dtype=torch.uint8, device=dev)
        length = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
        rec = _Recorder(period, max_frames, frames.data_ptr(),
                        length.data_ptr())
        _check(self._lib.gpumas_context_recorder_set(self._ptr,
                                                     ctypes.byref(rec)),
               "gpumas_context_recorder_set")
        try:
            s, r = self.transport(states, first_event)
        finally:
            self._lib.gpumas_context_recorder_set(self._ptr, None)
        f = np.frombuffer(frames.cpu().numpy().tobytes(),
                          dtype=FRAME_DTYPE).reshape(max(n, 1), max_frames)
        return s, r, f[:n], length.cpu().numpy()[:n]

    def transport_raw(self, n, states_ptr, results_ptr, first_event=0):
        """Transport n states at a host address (in place)."""
        return self._lib.gpumas_context_transport(
            self._ptr, n, states_ptr, results_ptr, first_event)

    def transport_device(self, n, soa, first_event=0, stream=None):
        """Transport n events of a device SoA (dict of device pointers)."""
        c = _soa(soa)
        return self._lib.gpumas_context_transport_device(
            self._ptr, n, ctypes.byref(c), first_event, stream)

    def tuning(self, engine=0, pool_slots=0, max_inner=0, batch=0, tail=0):
        """Set engine parameters (zero keeps a value); returns the current
        ones as a dict."""
        t = _Tuning(engine, pool_slots, max_inner, batch, tail)
        _check(self._lib.gpumas_context_tuning_set(self._ptr,
                                                   ctypes.byref(t)),
               "gpumas_context_tuning_set")
        self._lib.gpumas_context_tuning_get(self._ptr, ctypes.byref(t))
        return {"engine": t.engine, "pool_slots": t.pool_slots,
                "max_inner": t.max_inner, "batch": t.batch, "tail": t.tail}

    @property
    def carry(self):
        """Whether transport calls continue each event's random stream and
        Box-Muller cache from its results (gpumas_context_carry_set)."""
        c = ctypes.c_int()
        _check(self._lib.gpumas_context_carry_get(self._ptr, ctypes.byref(c)),
               "gpumas_context_carry_get")
        return bool(c.value)

    @carry.setter
    def carry(self, on):
        _check(self._lib.gpumas_context_carry_set(self._ptr, int(bool(on))),
               "gpumas_context_carry_set")

    @property
    def max_trials(self):
        """Trials of a rejection sampling before an event fails with
        RETURN_INTERNAL_ERROR (gpumas_context_trials_set)."""
        n = ctypes.c_int()
        _check(self._lib.gpumas_context_trials_get(self._ptr,
                                                   ctypes.byref(n)),
               "gpumas_context_trials_get")
        return n.value

    @max_trials.setter
    def max_trials(self, n):
        _check(self._lib.gpumas_context_trials_set(self._ptr, int(n)),
               "gpumas_context_trials_set")

    def stats(self):
        st = _Stats()
        self._lib.gpumas_context_stats(self._ptr, ctypes.byref(st))
        return {"launches": st.launches, "kernel_ms": st.kernel_ms}

    def __del__(self):
        if getattr(self, "_ptr", None):
            self._lib.gpumas_context_destroy(ctypes.byref(self._ptr))


def _soa(soa):
    """A gpumas_soa from a dict of device pointers (position and direction
    as 3-lists, result optional)."""
    c = _Soa()
    for k in ("charge", "energy", "distance", "grammage", "time", "weight",
              "decayed"):
        setattr(c, k, soa[k])
    for k in range(3):
        c.position[k] = soa["position"][k]
        c.direction[k] = soa["direction"][k]
    c.result = soa.get("result", None)
    return c


class Engine:
    """A persistent transport engine (gpumas_engine): many jobs of different
    contexts in one slot pool, submitted at once (``run``) or while others
    run (``submit`` / ``submit_host`` then ``step``)."""

    def __init__(self, physics, pool_slots=0, max_inner=0, batch=0,
                 max_jobs=0, state_budget=0, tail=0):
        self.physics = physics
        self._lib = physics._lib
        self._ptr = ctypes.c_void_p()
        t = _Tuning(ENGINE_POOL, pool_slots, max_inner, batch, tail)
        _check(self._lib.gpumas_engine_create(
            ctypes.byref(self._ptr), physics._ptr, ctypes.byref(t),
            max_jobs, state_budget), "gpumas_engine_create")
        self._host = {}

    @staticmethod
    def _job(context, n, soa, first_event):
        return _Job(ctypes.cast(context._ptr, ctypes.c_void_p), n, _soa(soa),
                    first_event)

    def submit(self, context, n, soa, first_event=0):
        """Queue a job of n events in device memory; returns its ticket."""
        job = self._job(context, n, soa, first_event)
        t = ctypes.c_int()
        _check(self._lib.gpumas_engine_submit(self._ptr, ctypes.byref(job),
                                              ctypes.byref(t)),
               "gpumas_engine_submit")
        return t.value

    def submit_host(self, context, states, first_event=0):
        """Queue a job of pumas_state records from host memory (copied into
        the state budget). Returns its ticket, or None when the budget has
        no room now. The (states, results) arrays are filled when the
        ticket is reported done; get them with ``result(ticket)``."""
        s = np.array(states, dtype=STATE_DTYPE, copy=True, order="C")
        r = np.zeros(len(s), dtype=RESULT_DTYPE)
        t = ctypes.c_int()
        rc = self._lib.gpumas_engine_submit_host(
            self._ptr, context._ptr, len(s), s.ctypes.data, r.ctypes.data,
            first_event, ctypes.byref(t))
        if rc == RETURN_MEMORY_ERROR:
            return None
        _check(rc, "gpumas_engine_submit_host")
        self._host[t.value] = (s, r)
        return t.value

    def result(self, ticket):
        """(states, results) of a completed host job (once)."""
        return self._host.pop(ticket)

    def step(self, max_done=4096):
        """One graph batch; returns (completed tickets, pending jobs)."""
        done = (ctypes.c_int * max_done)()
        nd, pend = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.gpumas_engine_step(
            self._ptr, max_done, done, ctypes.byref(nd), ctypes.byref(pend)),
            "gpumas_engine_step")
        return list(done[:nd.value]), pend.value

    def run(self, jobs):
        """Run jobs [(context, n, soa, first_event), ...] to completion."""
        arr = (_Job * len(jobs))(*[self._job(*j) for j in jobs])
        _check(self._lib.gpumas_engine_run(self._ptr, len(jobs), arr),
               "gpumas_engine_run")

    def stats(self):
        st = _EngineStats()
        self._lib.gpumas_engine_stats(self._ptr, ctypes.byref(st))
        return {"launches": st.launches, "batches": st.batches,
                "kernel_ms": st.kernel_ms, "events": st.events,
                "budget_used": st.budget_used}

    def __del__(self):
        if getattr(self, "_ptr", None):
            self._lib.gpumas_engine_destroy(ctypes.byref(self._ptr))


def random_fill(seed, domain, event, first, n):
    """Draws first .. first + n - 1 of a Philox stream, computed on the GPU."""
    out = np.zeros(n, dtype=np.float64)
    _check(library().gpumas_random_fill(seed, domain, event, first, n,
                                        out.ctypes.data),
           "gpumas_random_fill")
    return out
