"""Tau transport: physics made by the reference's pumas_physics_create for
PUMAS_PARTICLE_TAU (pumas_gb300/data/tau.pumas.gz), loaded like the muon
dump. Parity runs through the tau golden cases of tests/cases.py
(tau_stack_forward, tau_rock_csda_randomised, tau_rock_backward) in
test_gpu_parity.py and test_oracle.py; this file covers the particle
specific settings of pumas.c:1797-1804, 2592-2594 and 3157-3161.
"""
import gzip
import struct

import pytest

from cases import CASES


def test_shipped_tau_dump_header():
    """The dump's particle enum, c tau and mass (pumas.c:1797-1804)."""
    import pumas_gb300 as pg
    b = pg.default_dump("tau")
    hdr = struct.unpack("11i", b[8:52])
    ctau, mass = struct.unpack("2d", b[8 + 48:8 + 64])
    assert hdr[10] == pg.PARTICLE_TAU
    assert ctau == 87.03E-06 and mass == 1.77682
    with gzip.open(pg.DEFAULT_DUMP) as f:
        assert struct.unpack("11i", f.read(52)[8:52])[10] == pg.PARTICLE_MUON


@pytest.mark.gpu
def test_tau_physics_and_context_defaults(gpu_tau_physics):
    import pumas_gb300 as pg
    assert gpu_tau_physics.particle == pg.PARTICLE_TAU
    assert gpu_tau_physics.mass == 1.77682
    assert gpu_tau_physics.ctau == 87.03E-06
    ctx = pg.Context(gpu_tau_physics)
    # pumas_context_create: randomised decay for taus (pumas.c:2592-2594).
    assert ctx.mode.decay == pg.MODE_RANDOMISED


@pytest.mark.gpu
def test_forward_weighted_taus_are_refused(gpu_tau_physics):
    """pumas.c:3157-3161: weighted decay is invalid for forward taus."""
    import pumas_gb300 as pg
    from conftest import gpu_context, gpu_geometry
    case = CASES["tau_stack_forward"]
    cfg = dict(case["config"], decay=pg.MODE_WEIGHTED)
    geo = gpu_geometry(gpu_tau_physics, case["geometry"])
    ctx = gpu_context(gpu_tau_physics, cfg, 1, geo)
    with pytest.raises(pg.PumasError) as e:
        ctx.transport(pg.new_states(4))
    assert e.value.code == pg.RETURN_DECAY_ERROR
