"""CPU oracles of the transport hot path -- test infrastructure only.

Two implementations sit behind the same batch interface (oracle.h):

* ``Reference``: the unmodified reference library (src/pumas.c compiled from
  its own source tree, see Makefile ``ref`` target), available where those
  sources are;
* ``Port``: the plain C restatement of port.c, which builds anywhere.

Both transport one event per ``pumas_context_transport`` call, with the
Philox stream of philox.h as random callback and the geometries of
include/gpumas_geometry.h as medium callback. Only tests, the smoke check and
the CPU baseline of the benchmark use this package; the GPU engine never
does.
"""
import ctypes
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libpumas_ref.so")
# The reference checkout: PUMAS_REFERENCE, else a directory named
# "reference" beside this repository.
REFERENCE_DIR = os.environ.get("PUMAS_REFERENCE", os.path.normpath(
    os.path.join(HERE, "..", "..", "reference")))

# pumas_state layout (pumas.h:289-309), padded to 8 bytes.
STATE_DTYPE = np.dtype([
    ("charge", "f8"), ("energy", "f8"), ("distance", "f8"),
    ("grammage", "f8"), ("time", "f8"), ("weight", "f8"),
    ("position", "f8", 3), ("direction", "f8", 3), ("decayed", "i4"),
    ("pad", "i4")])

RESULT_DTYPE = np.dtype([
    ("event", "i4"), ("medium_in", "i4"), ("medium_out", "i4"),
    ("status", "i4"), ("steps", "i4"), ("randn_done", "i4"),
    ("draws", "u8"), ("randn_next", "f8")])


# struct oracle_frame (oracle.h): a state, the medium index and the event.
FRAME_DTYPE = np.dtype([("state", STATE_DTYPE), ("medium", "i4"),
                        ("event", "i4")])


class Medium(ctypes.Structure):
    _fields_ = [("material", ctypes.c_int), ("density", ctypes.c_double)]


class Locals(ctypes.Structure):
    """struct gpumas_locals (include/gpumas_geometry.h)."""
    _fields_ = [("model", ctypes.c_int), ("rho0", ctypes.c_double),
                ("axis", ctypes.c_double * 3), ("h0", ctypes.c_double),
                ("lambda_", ctypes.c_double), ("eps", ctypes.c_double),
                ("magnet", ctypes.c_double * 3)]


class Geometry(ctypes.Structure):
    """struct gpumas_geometry (include/gpumas_geometry.h)."""
    _fields_ = [
        ("kind", ctypes.c_int), ("n_media", ctypes.c_int),
        ("media", ctypes.POINTER(Medium)),
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
        ("locals", ctypes.POINTER(Locals))]


class Config(ctypes.Structure):
    """struct oracle_config: the public settings of a pumas_context."""
    _fields_ = [
        ("energy_loss", ctypes.c_int), ("decay", ctypes.c_int),
        ("direction", ctypes.c_int), ("scattering", ctypes.c_int),
        ("event", ctypes.c_int),
        ("limit_energy", ctypes.c_double), ("limit_distance", ctypes.c_double),
        ("limit_grammage", ctypes.c_double), ("limit_time", ctypes.c_double),
        ("accuracy", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("carry", ctypes.c_int)]


def make_geometry(kind, media, **kw):
    """Build a Geometry whose arrays stay alive on the returned object."""
    g = Geometry()
    g.kind = kind
    keep = []
    m = (Medium * len(media))(*[Medium(int(a), float(b)) for a, b in media])
    keep.append(m)
    g.n_media = len(media)
    g.media = m
    g.uniform_medium = int(kw.get("uniform_medium", 0))
    if "slab_z" in kw:
        z = np.ascontiguousarray(kw["slab_z"], dtype=np.float64)
        sm = np.ascontiguousarray(
            kw.get("slab_medium", kw.get("slab_media")), dtype=np.int32)
        keep += [z, sm]
        g.n_slabs = len(sm)
        g.slab_z = z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        g.slab_medium = sm.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    if "hm_z" in kw:
        hz = np.ascontiguousarray(kw["hm_z"], dtype=np.float64)
        keep.append(hz)
        g.hm_ny, g.hm_nx = hz.shape
        g.hm_x0, g.hm_y0 = kw["hm_x0"], kw["hm_y0"]
        g.hm_dx, g.hm_dy = kw["hm_dx"], kw["hm_dy"]
        g.hm_z = hz.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        g.hm_below, g.hm_above = kw["hm_below"], kw["hm_above"]
        g.hm_ztop = kw["hm_ztop"]
    if kw.get("locals") is not None:
        arr = (Locals * len(media))()
        for a, d in zip(arr, kw["locals"]):
            a.model = int(d.get("model", 0))
            a.rho0 = float(d.get("rho0", 0.))
            a.axis[:] = [float(v) for v in d.get("axis", (0., 0., 1.))]
            a.h0 = float(d.get("h0", 0.))
            a.lambda_ = float(d.get("lambda_", 0.))
            a.eps = float(d.get("eps", 0.))
            a.magnet[:] = [float(v) for v in d.get("magnet", (0., 0., 0.))]
        keep.append(arr)
        g.locals = arr
    g._keep = keep
    return g


def build_port():
    """Compile the C restatement (quick, no reference needed)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def build_reference():
    """Compile the reference library from its own sources, if present."""
    src = os.path.join(REFERENCE_DIR, "src", "pumas.c")
    if not os.path.exists(src):
        return False
    subprocess.check_call(["make", "-s", "-C", HERE, "ref",
                           "REFERENCE=" + REFERENCE_DIR])
    return True


class _Oracle:
    prefix = None
    path = None

    def __init__(self, private=False):
        """Load the oracle library. Its physics is a global of the library:
        with `private`, a copy of the library is loaded instead, so that
        another physics (taus) can live beside the first one."""
        if not os.path.exists(self.path):
            raise FileNotFoundError(self.path)
        path = self.path
        if private:
            path = os.path.join(tempfile.mkdtemp(prefix="oracle"),
                                os.path.basename(self.path))
            shutil.copy(self.path, path)
        self.lib = ctypes.CDLL(path)
        p = self.prefix
        self._transport = getattr(self.lib, p + "_transport")
        self._transport.restype = ctypes.c_int
        self._transport.argtypes = [
            ctypes.POINTER(Config), ctypes.POINTER(Geometry), ctypes.c_int64,
            ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        self._mat = getattr(self.lib, p + "_material_index")
        self._mat.restype = ctypes.c_int
        self._mat.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        self._prop = getattr(self.lib, p + "_property")
        self._prop.restype = ctypes.c_int
        self._prop.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.c_double,
                               ctypes.POINTER(ctypes.c_double)]
        self._threads = getattr(self.lib, p + "_max_threads")
        self._threads.restype = ctypes.c_int

    def max_threads(self):
        return self._threads()

    def material_index(self, name):
        i = ctypes.c_int(-1)
        rc = self._mat(name.encode(), ctypes.byref(i))
        if rc != 0:
            raise KeyError(name)
        return i.value

    def property(self, which, scheme, material, kinetic):
        v = ctypes.c_double(0.)
        rc = self._prop(which, scheme, material, kinetic, ctypes.byref(v))
        if rc != 0:
            raise RuntimeError("property error %d" % rc)
        return v.value

    def transport(self, config, geometry, states, first_event=0,
                  n_threads=1, results=None):
        """Transport a copy of `states` (STATE_DTYPE); returns the final
        states and the per event results. With config.carry, each event
        continues the random state of `results` (a previous call's)."""
        s = np.array(states, dtype=STATE_DTYPE, copy=True, order="C")
        if results is None:
            r = np.zeros(len(s), dtype=RESULT_DTYPE)
        else:
            r = np.array(results, dtype=RESULT_DTYPE, copy=True, order="C")
        rc = self._transport(ctypes.byref(config), ctypes.byref(geometry),
                             len(s), first_event, s.ctypes.data,
                             r.ctypes.data, n_threads)
        if rc != 0:
            raise RuntimeError("oracle transport error %d" % rc)
        return s, r


class Port(_Oracle):
    """The C restatement of the reference transport (port.c)."""
    prefix = "oracle_port"
    path = PORT_LIB

    def __init__(self, dump_bytes, private=False):
        super().__init__(private)
        self.lib.oracle_port_load.restype = ctypes.c_int
        self.lib.oracle_port_load.argtypes = [ctypes.c_char_p,
                                              ctypes.c_int64]
        rc = self.lib.oracle_port_load(dump_bytes, len(dump_bytes))
        if rc != 0:
            raise RuntimeError("port load error %d" % rc)
        self.lib.oracle_port_uniform.restype = ctypes.c_double
        self.lib.oracle_port_uniform.argtypes = [
            ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
            ctypes.c_uint64]

    def uniform(self, seed, domain, event, n):
        return self.lib.oracle_port_uniform(seed, domain, event, n)


class PortDouble(Port):
    """The C restatement with its Coulomb functions in double instead of the
    reference's long double (port.c, ORACLE_COULOMB_DOUBLE): only for timing
    how much of the CPU baseline the long double arithmetic costs."""
    path = os.path.join(HERE, "_build", "liboracle_port_double.so")


class Reference(_Oracle):
    """The reference library driven as an oracle (ref_harness.c)."""
    prefix = "oracle_ref"
    path = REF_LIB

    def __init__(self, dump_path, private=False):
        super().__init__(private)
        self.lib.oracle_ref_load.restype = ctypes.c_int
        self.lib.oracle_ref_load.argtypes = [ctypes.c_char_p]
        rc = self.lib.oracle_ref_load(dump_path.encode())
        if rc != 0:
            raise RuntimeError("reference load error %d" % rc)


def _port_dcs_tables(self):
    """The per element DEL tables of the loaded dump: CSn and CSn_dK
    [4, n_elements, n_energies], DCS tables [3, n_elements, n_energies,
    n_table_dcs, 2], envelope exponents [3, n_elements, n_energies] and the
    DCS grid."""
    f = self.lib.oracle_port_dcs_tables
    f.restype = ctypes.c_int
    dims = (ctypes.c_int * 3)()
    f(dims, None, None, None, None, None)
    nel, ne, nx = dims
    csn = np.zeros((4, nel, ne))
    dk = np.zeros((4, nel, ne))
    dcs = np.zeros((3, nel, ne, nx, 2), dtype=np.float32)
    alpha = np.zeros((3, nel, ne), dtype=np.float32)
    x = np.zeros(nx, dtype=np.float32)
    rc = f(dims, csn.ctypes.data_as(ctypes.c_void_p),
           dk.ctypes.data_as(ctypes.c_void_p),
           dcs.ctypes.data_as(ctypes.c_void_p),
           alpha.ctypes.data_as(ctypes.c_void_p),
           x.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle tables error %d" % rc)
    return {"csn": csn, "csn_dk": dk, "dcs": dcs, "alpha": alpha, "x": x}


def _reference_dcs_tables(self, shape):
    """The same tables (but CSn_dK) computed by the reference's own
    functions on its loaded physics; `shape` = (n_elements, n_energies,
    n_table_dcs). Returns the tables and the wall times (s) of the cross
    sections and of the DCS rows."""
    nel, ne, nx = shape
    f = self.lib.oracle_ref_dcs_tables
    f.restype = ctypes.c_int
    csn = np.zeros((4, nel, ne))
    dcs = np.zeros((3, nel, ne, nx, 2), dtype=np.float32)
    alpha = np.zeros((3, nel, ne), dtype=np.float32)
    t = np.zeros(2)
    rc = f(csn.ctypes.data_as(ctypes.c_void_p),
           dcs.ctypes.data_as(ctypes.c_void_p),
           alpha.ctypes.data_as(ctypes.c_void_p),
           t.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("reference tables error %d" % rc)
    return {"csn": csn, "dcs": dcs, "alpha": alpha}, t


def _reference_record(self, config, geometry, states, first_event, period,
                      max_frames):
    """Transport with the reference's frame recorder; returns (states,
    results, frames [n, max_frames], frame counts)."""
    f = self.lib.oracle_ref_transport_record
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Geometry),
                  ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p]
    s = np.array(states, dtype=STATE_DTYPE, copy=True, order="C")
    r = np.zeros(len(s), dtype=RESULT_DTYPE)
    frames = np.zeros((len(s), max_frames), dtype=FRAME_DTYPE)
    length = np.zeros(len(s), dtype=np.int32)
    rc = f(ctypes.byref(config), ctypes.byref(geometry), len(s), first_event,
           s.ctypes.data, r.ctypes.data, period, max_frames,
           frames.ctypes.data, length.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle record error %d" % rc)
    return s, r, frames, length


Reference.transport_record = _reference_record
Reference.dcs_tables = _reference_dcs_tables


def _port_dcs_tabulate(self, n_threads=1):
    """The C restatement of the device table builder on the loaded
    physics: the tables of dcs_tables (without the DCS grid), computed."""
    t = self.dcs_tables()
    f = self.lib.oracle_port_dcs_tabulate
    f.restype = ctypes.c_int
    out = {k: np.zeros_like(t[k]) for k in ("csn", "csn_dk", "dcs",
                                            "alpha")}
    rc = f(*[out[k].ctypes.data_as(ctypes.c_void_p) for k in
             ("csn", "csn_dk", "dcs", "alpha")], ctypes.c_int(n_threads))
    if rc != 0:
        raise RuntimeError("oracle tabulation error %d" % rc)
    return out


Port.dcs_tabulate = _port_dcs_tabulate
Port.dcs_tables = _port_dcs_tables


def reference_available():
    return os.path.exists(REF_LIB)
