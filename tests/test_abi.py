"""The C ABI library: builds, loads and exports every declared symbol.

CPU only: no CUDA call is made (loading libgpumas.so needs libcudart only).
"""
import ctypes
import os
import re
import shutil

import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h)
           for h in ("gpumas.h", "gpumas_geometry.h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|double)\s+\**\s*(gpumas_\w+)\s*\(",
                             text, flags=re.M):
            names.append(m.group(1))
    return names


@pytest.mark.skipif(shutil.which("nvcc") is None and
                    not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="no nvcc")
def test_library_exports_declared_symbols():
    import pumas_gb300
    from pumas_gb300 import build
    lib = ctypes.CDLL(build.build())
    names = declared_functions()
    assert "gpumas_context_transport" in names
    assert "gpumas_physics_load" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # The geometry header's functions are inline host/device code, not
    # exported symbols.
    assert pumas_gb300.library() is not None


def test_no_product_import_of_oracle():
    """The product package never imports or links the oracle."""
    pkg = os.path.join(ROOT, "pumas_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath or "data" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text
                assert "oracle/" not in text
                assert "liboracle" not in text


def test_random_seed_set_get():
    """pumas_context_random_seed_set / _get semantics on the public context
    record (no device needed): a given key is kept, NULL draws one from the
    OS."""
    import ctypes
    import pumas_gb300 as pg
    lib = pg.library()
    ctx = pg._Context()
    u64 = ctypes.c_uint64
    lib.gpumas_context_random_seed_set.restype = ctypes.c_int
    lib.gpumas_context_random_seed_set.argtypes = [
        ctypes.POINTER(pg._Context), ctypes.POINTER(u64)]
    lib.gpumas_context_random_seed_get.restype = ctypes.c_int
    lib.gpumas_context_random_seed_get.argtypes = [
        ctypes.POINTER(pg._Context), ctypes.POINTER(u64)]
    assert lib.gpumas_context_random_seed_set(
        ctypes.byref(ctx), ctypes.byref(u64(0x0123456789ABCDEF))) == 0
    got = u64()
    assert lib.gpumas_context_random_seed_get(
        ctypes.byref(ctx), ctypes.byref(got)) == 0
    assert got.value == 0x0123456789ABCDEF == ctx.seed
    draws = set()
    for _ in range(3):
        assert lib.gpumas_context_random_seed_set(ctypes.byref(ctx),
                                                  None) == 0
        draws.add(ctx.seed)
    assert len(draws) == 3
    assert lib.gpumas_context_random_seed_get(None, ctypes.byref(got)) == \
        pg.RETURN_VALUE_ERROR
    lib.gpumas_physics_cutoff.restype = ctypes.c_double
    lib.gpumas_physics_cutoff.argtypes = [ctypes.c_void_p]
    assert lib.gpumas_physics_cutoff(None) == 0.


def test_loader_checks_dumps_before_the_device():
    """gpumas_physics_load checks a dump's format, DCS model names and
    particle before any device call: malformed dumps fail with the
    reference's codes, on a machine without a GPU too."""
    import ctypes
    import struct
    import pumas_gb300 as pg
    lib = pg.library()
    load = lib.gpumas_physics_load
    load.restype = ctypes.c_int
    load.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                     ctypes.c_size_t]
    ptr = ctypes.c_void_p()
    assert load(ctypes.byref(ptr), bytes(100), 100) == pg.RETURN_FORMAT_ERROR
    dump = pg.default_dump()
    assert load(ctypes.byref(ptr), dump, 7) == pg.RETURN_FORMAT_ERROR
    # The blob follows an 8 byte tag and size; its pointer table starts at
    # byte 80 and its data at byte 528 (pumas.c:2167-2196).
    ptrs = struct.unpack_from("53Q", dump, 8 + 80)
    pair = 8 + ptrs[51] - ptrs[0] + 528
    assert dump[pair:pair + 4] == b"SSR\0"
    bad = bytearray(dump)
    bad[pair:pair + 3] = b"XYZ"
    assert load(ctypes.byref(ptr), bytes(bad), len(bad)) == \
        pg.RETURN_MODEL_ERROR
    bad = bytearray(dump)
    struct.pack_into("i", bad, 8 + 40, 7)
    assert load(ctypes.byref(ptr), bytes(bad), len(bad)) == \
        pg.RETURN_UNKNOWN_PARTICLE
    assert not ptr.value


def test_loader_accepts_tau_and_model_dumps():
    """The shipped tau dump and the dumps with non-default DCS models pass
    the loader's checks: without a GPU the load stops at the first device
    call (GPUMAS_RETURN_DEVICE_ERROR); with one it succeeds."""
    import ctypes
    import pumas_gb300 as pg
    from cases import physics_dump
    lib = pg.library()
    load = lib.gpumas_physics_load
    load.restype = ctypes.c_int
    load.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                     ctypes.c_size_t]
    destroy = lib.gpumas_physics_destroy
    destroy.restype = None
    destroy.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    for name in ("muon", "tau", "muon_kkp", "muon_abb", "tau_bbks"):
        dump = physics_dump(name)
        ptr = ctypes.c_void_p()
        rc = load(ctypes.byref(ptr), dump, len(dump))
        assert rc in (pg.RETURN_SUCCESS, pg.RETURN_DEVICE_ERROR), (name, rc)
        if ptr.value:
            destroy(ctypes.byref(ptr))


def test_error_handler_catch_raise():
    """The error API of the reference (pumas_error_handler_set, _catch,
    _raise, _function; pumas.h:1110-1184) on errors that happen before any
    device call: the installed handler gets the code, the failing function
    and a message and the code is returned; caught errors are held until
    raised; the library never exits, with or without a handler."""
    import ctypes
    import pumas_gb300 as pg
    lib = pg.library()
    HANDLER = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_void_p,
                               ctypes.c_char_p)
    lib.gpumas_error_handler_set.argtypes = [HANDLER]
    lib.gpumas_error_handler_set.restype = None
    lib.gpumas_error_handler_get.restype = ctypes.c_void_p
    lib.gpumas_error_catch.argtypes = [ctypes.c_int]
    lib.gpumas_error_catch.restype = None
    lib.gpumas_error_raise.restype = ctypes.c_int
    lib.gpumas_error_function.argtypes = [ctypes.c_void_p]
    lib.gpumas_error_function.restype = ctypes.c_char_p
    load = lib.gpumas_physics_load
    load.restype = ctypes.c_int
    load.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                     ctypes.c_size_t]
    calls = []

    def on_error(rc, caller, message):
        calls.append((rc, lib.gpumas_error_function(caller), message))

    handler = HANDLER(on_error)
    ptr = ctypes.c_void_p()
    try:
        # No handler: the code only.
        assert lib.gpumas_error_handler_get() is None
        assert load(ctypes.byref(ptr), bytes(100), 100) == \
            pg.RETURN_FORMAT_ERROR
        lib.gpumas_error_handler_set(handler)
        assert lib.gpumas_error_handler_get() is not None
        assert load(ctypes.byref(ptr), bytes(100), 100) == \
            pg.RETURN_FORMAT_ERROR
        assert calls == [(pg.RETURN_FORMAT_ERROR, b"gpumas_physics_load",
                          b"gpumas_physics_load returned "
                          b"GPUMAS_RETURN_FORMAT_ERROR (11)")]
        # Caught errors: the first one is raised, the handler called once.
        calls.clear()
        lib.gpumas_error_catch(1)
        assert load(None, bytes(100), 100) == pg.RETURN_PHYSICS_ERROR
        assert load(ctypes.byref(ptr), bytes(100), 100) == \
            pg.RETURN_FORMAT_ERROR
        assert calls == []
        assert lib.gpumas_error_raise() == pg.RETURN_PHYSICS_ERROR
        assert [c[:2] for c in calls] == [
            (pg.RETURN_PHYSICS_ERROR, b"gpumas_physics_load")]
        # Raise without catch.
        calls.clear()
        assert lib.gpumas_error_raise() == pg.RETURN_RAISE_ERROR
        assert [c[:2] for c in calls] == [
            (pg.RETURN_RAISE_ERROR, b"gpumas_error_raise")]
        # A catch with no error raises success, without a call.
        calls.clear()
        lib.gpumas_error_catch(1)
        assert lib.gpumas_error_raise() == pg.RETURN_SUCCESS
        assert calls == []
    finally:
        lib.gpumas_error_catch(0)
        lib.gpumas_error_handler_set(HANDLER(0))
    assert lib.gpumas_error_handler_get() is None
