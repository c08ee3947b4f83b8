"""Device table builder (gpumas_physics_tabulate) against the tables the
reference's pumas_physics_create wrote into the physics dumps (GPU).

The per element DEL tables -- restricted cross sections CSn and their PCHIP
slopes, DCS interpolation tables and envelope exponents -- are recomputed on
the GPU from each physics' own elements, energy grid, cutoff and DCS models,
and compared with the dump's (which tests/test_oracle.py shows to be the
output of the reference functions that the device code restates). The DCS
models run on the device with the device's logarithm, arc tangent and
power functions, so values agree to a few ulp: CSn within 1e-10 relative,
CSn_dK within 1e-9 of its column's scale, and at least 99.9 % of the single
precision table entries and envelope exponents bit for bit, the others
within 16 ulp.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHYSICS = ["muon", "tau", "muon_kkp", "muon_abb", "tau_bbks"]


def float_ulps(a, b):
    """Distance in units in the last place between float32 arrays."""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


@pytest.mark.parametrize("name", PHYSICS)
def test_device_tabulation_matches_dump(request, name):
    import oracle
    import pumas_gb300 as pg
    from cases import physics_dump
    from conftest import PARITY_REPORT
    dump = physics_dump(name)
    phys = pg.Physics(dump)
    got = phys.tabulate()
    port = oracle.Port(dump, private=True)
    want = port.dcs_tables()

    a, b = got["csn"], want["csn"]
    assert np.array_equal(a == 0., b == 0.)
    nz = b != 0.
    rel = np.abs(a[nz] - b[nz]) / np.abs(b[nz])
    # The ABB bremsstrahlung DCS (pumas.c:13824-13905) is a difference of
    # screening terms that cancel near the end point: a last bit difference
    # in one of their logarithms or arc tangents moves the DCS there, and the
    # integral, by up to about 1e-11.
    assert rel.max() <= 1E-10, rel.max()

    a, b = got["csn_dk"], want["csn_dk"]
    scale = np.maximum(np.abs(b).max(axis=2, keepdims=True), 1E-300)
    assert np.all(np.abs(a - b) <= 1E-09 * scale)

    n_same = n_all = 0
    worst = {}
    for key in ("dcs", "alpha"):
        a, b = got[key].ravel(), want[key].ravel()
        ulps = float_ulps(a, b)
        worst[key] = int(ulps.max())
        n_same += int(np.count_nonzero(ulps == 0))
        n_all += a.size
    PARITY_REPORT["tabulate " + name] = (n_same, n_all)
    print("%s: device tabulation %.1f ms, %d / %d single precision entries "
          "bit for bit, worst %s ulp" % (name, got["ms"], n_same, n_all,
                                         worst))
    assert n_same >= 0.999 * n_all
    # A slope is a difference quotient of double precision logarithms: a
    # last bit difference there can move its single precision value by a
    # few ulp.
    assert max(worst.values()) <= 16, worst
