"""gpumas_physics_upload: the device physics from a live struct
pumas_physics, the path a C program that created or loaded its physics
with the reference takes (include/gpumas.h).

A live struct is the dump's blob whose pointers have been moved to the
addresses of this process (pumas_physics_load, pumas.c:2096-2122).
`live_struct` makes one from a dump in the same way. On the CPU, it is
checked against the reference's own live struct (pointer table relative to
the struct, header and data bytes). On the GPU, the physics uploaded from
it transports bit for bit as the one loaded from the dump.
"""
import ctypes

import numpy as np
import pytest

# Offsets in the struct (pumas.c:660-806): the header, the 53 data
# pointers, the three DCS function pointers, then the data.
POINTERS, N_POINTERS, DATA = 80, 53, 528


# Pointer table entries of the dE/dX file names and of the element,
# composition, composite and material name arrays (pumas.c:1557-1758), and
# the offset of an element's name pointer in struct atomic_element
# (pumas.c:510-523).
DEDX_FILENAME, ELEMENTS, COMPOSITIONS, COMPOSITES, NAMES = 2, 46, 47, 48, 49
ELEMENT_NAME = 32


def live_struct(dump, moved=None):
    """A writable copy of the dump's blob with its pointers moved to this
    buffer, as pumas_physics_load does (the data pointers, then the element,
    composition, composite and name arrays and the elements' names, and the
    dE/dX file names erased); keep the array alive while its address is
    used. The byte offsets of the moved pointers are appended to `moved`."""
    size = int(np.frombuffer(dump, dtype=np.int32, count=1, offset=4)[0])
    buf = np.frombuffer(bytearray(dump[8:8 + size]), dtype=np.uint8)
    hdr = buf[:44].view(np.int32)
    n_materials, n_composites, n_elements = int(hdr[2]), int(hdr[3]), \
        int(hdr[4])
    ptr = buf[POINTERS:POINTERS + 8 * N_POINTERS].view(np.uint64)
    base = buf.ctypes.data
    delta = base + DATA - int(ptr[0])

    def move(offset, n):
        """Shift n pointers at byte `offset`; returns their new values."""
        a = buf[offset:offset + 8 * n].view(np.uint64)
        a[:] = [(int(p) + delta) % (1 << 64) for p in a]
        if moved is not None:
            moved.extend(range(offset, offset + 8 * n, 8))
        return [int(p) for p in a]

    move(POINTERS, N_POINTERS)
    off = [int(p) - base for p in ptr]
    for e in move(off[ELEMENTS], n_elements):
        move(e - base + ELEMENT_NAME, 1)
    move(off[COMPOSITIONS], n_materials)
    move(off[COMPOSITES], n_composites)
    move(off[NAMES], n_materials)
    n_base = n_materials - n_composites
    buf[off[DEDX_FILENAME]:off[DEDX_FILENAME] + 8 * n_base] = 0
    return buf


def relative(buf, base, moved):
    """A copy of buf with the pointers at byte offsets `moved` made relative
    to base."""
    out = buf.copy()
    for o in moved:
        p = out[o:o + 8].view(np.uint64)
        p[0] = (int(p[0]) - base) % (1 << 64)
    return out


def test_live_struct_matches_reference(dump, tmp_path):
    """The emulated live struct is the reference's own, loaded from the same
    dump, byte for byte once every pointer is taken relative to its
    struct."""
    import oracle
    if not oracle.reference_available() and not oracle.build_reference():
        pytest.skip("reference sources not available")
    path = tmp_path / "muon.pumas"
    path.write_bytes(dump)
    ref = oracle.Reference(str(path), private=True)
    f = ref.lib.oracle_ref_physics
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.POINTER(ctypes.c_int)]
    size = ctypes.c_int()
    address = f(ctypes.byref(size))
    theirs = np.frombuffer((ctypes.c_char * size.value).from_address(
        address).raw, dtype=np.uint8)
    moved = []
    ours = live_struct(dump, moved)
    assert len(ours) == size.value
    assert len(moved) > N_POINTERS
    a = relative(ours, ours.ctypes.data, moved)
    b = relative(theirs, address, moved)
    # The three DCS function pointers after the data pointers
    # (pumas.c:796-801), which the loader sets (pumas.c:2124-2153), are
    # addresses in the reference's library and not part of the tables.
    a[DATA - 24:DATA] = b[DATA - 24:DATA] = 0
    assert np.array_equal(a, b)


@pytest.mark.gpu
def test_upload_transports_as_dump(gpu_physics, dump):
    import pumas_gb300 as pg
    from cases import CASES, make_states
    from conftest import gpu_context, gpu_geometry
    buf = live_struct(dump)
    uploaded = pg.Physics.upload(buf.ctypes.data)
    assert (uploaded.n_materials, uploaded.n_elements, uploaded.n_energies) \
        == (gpu_physics.n_materials, gpu_physics.n_elements,
            gpu_physics.n_energies)
    for name in ("rock_slab", "stack_backward_straggled"):
        case = CASES[name]
        s0 = make_states(name, n=2000, first_event=9)
        out = []
        for phys in (gpu_physics, uploaded):
            geo = gpu_geometry(phys, case["geometry"])
            ctx = gpu_context(phys, case["config"], case["seed"], geo)
            out.append(ctx.transport(s0, 9))
        (a, ra), (b, rb) = out
        assert a.tobytes() == b.tobytes()
        assert ra.tobytes() == rb.tobytes()
