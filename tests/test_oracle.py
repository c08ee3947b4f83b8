"""The CPU oracle, pinned against the reference (CPU only).

* known answers of the reference's own test suite for StandardRock tables
  (tests/test-pumas.c:892-986, 1141-1149);
* the Philox stream against the Random123 known answer vectors;
* the C restatement (oracle/port.c) against the golden fixtures made with
  the unmodified reference, bit for bit;
* the C restatement against a live run of the reference on fresh events,
  when the reference sources are available.
"""
import os

import numpy as np
import pytest

from cases import CASES, has_locals, make_states
from conftest import (GOLDEN, case_oracle, compare, oracle_config,
                      oracle_geometry)

RANGE, PROPER_TIME, KINETIC, STOPPING, STRAGGLING = 0, 1, 2, 3, 4
CSDA, MIXED = 0, 1


def test_table_known_answers(port):
    """Values of tests/test-pumas.c:909-936 for StandardRock (material 0)."""
    rock = port.material_index("StandardRock")
    assert rock == 0
    assert abs(port.property(STOPPING, CSDA, rock, 1.) - 1.823E-04) <= 1E-06
    assert abs(port.property(STOPPING, CSDA, rock, 1E+03) - 6.610E-04) <= 1E-07
    assert port.property(STOPPING, MIXED, rock, 1E+03) < 6.610E-04
    assert abs(port.property(STRAGGLING, 0, rock, 1E+03) - 3.743E-04) <= 1E-07
    assert abs(port.property(RANGE, CSDA, rock, 1.) - 5.518E+03) <= 1.
    assert abs(port.property(RANGE, CSDA, rock, 1E+03) - 2.449E+06) <= 1E+03
    assert port.property(RANGE, MIXED, rock, 1E+03) > 2.449E+06
    assert abs(port.property(KINETIC, CSDA, rock, 5.518E+03) - 1.) <= 1E-03
    assert abs(port.property(KINETIC, CSDA, rock, 2.449E+06) - 1E+03) <= 1.
    assert port.property(KINETIC, MIXED, rock, 2.449E+06) < 1E+03
    assert port.property(PROPER_TIME, CSDA, rock, 1.) < 5.475E+03
    assert port.property(PROPER_TIME, CSDA, rock, 1E-02) > 8.498


def test_table_values_match_reference(port, reference):
    rng = np.random.default_rng(3)
    for prop in (RANGE, PROPER_TIME, STOPPING, STRAGGLING):
        for material in range(4):
            for k in 10 ** rng.uniform(-3, 10, 200):
                a = port.property(prop, CSDA, material, k)
                b = reference.property(prop, CSDA, material, k)
                assert a == b


def test_philox_known_answers():
    from pumas_gb300 import workloads as W
    kat = [((0, 0, 0, 0), (0, 0),
            (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2,
            (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344),
            (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, out in kat:
        x = W.philox4x32_10(*[[c] for c in ctr], *key)
        assert tuple(int(v[0]) for v in x) == out


def test_philox_oracle_matches_numpy(port):
    from pumas_gb300 import workloads as W
    ev = np.arange(0, 300, dtype=np.uint64) * np.uint64(7919) + np.uint64(2**33)
    seed = 0x0123456789ABCDEF
    for n in (0, 1, 2, 5):
        for dom in (0, 1):
            a = W.uniform(seed, dom, ev, n)
            b = [port.uniform(seed, dom, int(e), n) for e in ev]
            assert np.array_equal(a, b)
            assert np.all((a > 0.) & (a < 1.))


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_golden(request, name):
    port = case_oracle(request, name, "port")
    data = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]
    s0 = data["initial"]
    assert np.array_equal(s0, make_states(name))
    geo = oracle_geometry(port, case["geometry"])
    cfg = oracle_config(case["config"], case["seed"])
    s1, r1 = port.transport(cfg, geo, s0, 0, 4)
    same, _ = compare(s1, r1, data["final"], data["results"])
    assert same.all(), "%d / %d events differ" % ((~same).sum(), len(same))
    assert np.array_equal(r1["draws"], data["results"]["draws"])
    assert np.array_equal(r1["steps"], data["results"]["steps"])


@pytest.mark.parametrize("name", sorted(n for n in CASES if has_locals(n)))
def test_reference_reproduces_locals_golden(reference, name):
    """The fixtures of media with local properties come from the reference
    alone: a rerun gives them back bit for bit, the stepping events do cross
    the non-uniform media and the fields do turn the tracks."""
    data = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]
    s0 = data["initial"]
    assert np.array_equal(s0, make_states(name))
    geo = oracle_geometry(reference, case["geometry"])
    cfg = oracle_config(case["config"], case["seed"])
    s1, r1 = reference.transport(cfg, geo, s0, 0, 4)
    same, _ = compare(s1, r1, data["final"], data["results"])
    assert same.all()
    assert np.all(r1["status"] == 0)
    if case["geometry"]["kind"] != 0:
        assert np.mean(r1["steps"]) > 10.
    # The field turns the tracks.
    turned = np.any(s1["direction"] != s0["direction"], axis=1)
    assert turned.mean() > 0.9


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_reference_fresh_events(request, reference, name):
    port = case_oracle(request, name, "port")
    reference = case_oracle(request, name, "reference")
    case = CASES[name]
    s0 = make_states(name, n=64, first_event=100000)
    geo_p = oracle_geometry(port, case["geometry"])
    geo_r = oracle_geometry(reference, case["geometry"])
    cfg = oracle_config(case["config"], case["seed"] + 1)
    a, ra = port.transport(cfg, geo_p, s0, 100000, 4)
    b, rb = reference.transport(cfg, geo_r, s0, 100000, 4)
    same, _ = compare(a, ra, b, rb)
    assert same.all()
    assert np.array_equal(ra["draws"], rb["draws"])


@pytest.mark.parametrize("name", ["rock_slab", "stack_backward_mixed",
                                  "water_time_limit"])
def test_coulomb_in_double_changes_no_event(name):
    """The reference evaluates the Coulomb functions of hard scatters in long
    double (pumas.c:7524-7683); the copy of the port built with double
    there (timed beside the CPU baseline) transports the same events to the
    same final states, bit for bit, on this host."""
    import oracle
    from cases import physics_dump
    oracle.build_port()
    dump = physics_dump("muon")
    case = CASES[name]
    s0 = make_states(name, n=600, first_event=4242)
    out = []
    for cls in (oracle.Port, oracle.PortDouble):
        o = cls(dump, private=True)
        geo = oracle_geometry(o, case["geometry"])
        cfg = oracle_config(case["config"], case["seed"])
        out.append(o.transport(cfg, geo, s0, 4242, 4))
    (a, ra), (b, rb) = out
    assert a.tobytes() == b.tobytes()
    assert ra.tobytes() == rb.tobytes()


def test_port_edge_cases(port):
    """Empty batches, bad directions, start outside the geometry and
    decayed states follow pumas.c:3135-3192."""
    import oracle
    rock = port.material_index("StandardRock")
    geo = oracle.make_geometry(1, [(rock, 0.)], slab_z=[0., 10.],
                               slab_medium=[0])
    cfg = oracle.Config(energy_loss=2, decay=0, direction=0, scattering=1,
                        event=1, limit_energy=1., accuracy=1E-02, seed=1)
    s, r = port.transport(cfg, geo, np.zeros(0, dtype=oracle.STATE_DTYPE))
    assert len(s) == 0
    s0 = np.zeros(4, dtype=oracle.STATE_DTYPE)
    s0["energy"] = 10.
    s0["weight"] = 1.
    s0["direction"][:, 2] = 1.
    s0["direction"][1] = (0., 0., 1.1)   # not normalised
    s0["position"][2, 2] = -1.           # outside of the slab
    s0["decayed"][3] = 1                 # already decayed
    s, r = port.transport(cfg, geo, s0)
    assert r["status"][0] == 0 and r["event"][0] == 16
    assert r["status"][1] == 5           # PUMAS_RETURN_DIRECTION_ERROR
    assert r["event"][2] == 16 and r["medium_in"][2] == -1
    assert r["event"][3] == 1024 and s["energy"][3] == 10.
    bad = oracle.Config(energy_loss=2, decay=0, direction=0, scattering=1,
                        event=1, limit_energy=1., accuracy=0., seed=1)
    s, r = port.transport(bad, geo, s0[:1])
    assert r["status"][0] == 1           # PUMAS_RETURN_ACCURACY_ERROR


@pytest.mark.parametrize("name", ["models_kkp_rock_slab",
                                  "models_abb_stack_forward"])
def test_dcs_model_changes_the_transport(port, request, name):
    """The same events with the default models end elsewhere: the model
    cases exercise their own DCS."""
    data = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]
    geo = oracle_geometry(port, case["geometry"])
    cfg = oracle_config(case["config"], case["seed"])
    s1, r1 = port.transport(cfg, geo, data["initial"], 0, 4)
    same, _ = compare(s1, r1, data["final"], data["results"])
    assert same.mean() < 0.5


def _chain(impl, seed, first, carry=1):
    from cases import CHAIN, run_chain, chain_states
    geo = oracle_geometry(impl, CHAIN["geometry"])

    def transport(cfg, states, results):
        c = oracle_config(cfg, seed)
        c.carry = carry
        return impl.transport(c, geo, states, first, 4, results)
    n = CHAIN["n"] if first == CHAIN["first_event"] else 64
    s0 = chain_states(n=n, seed=seed, first=first)
    return (s0,) + run_chain(transport, s0)


def test_port_chain_matches_golden(port):
    """Events transported over several calls (the loop of
    examples/pumas/geometry.c:269-312, each call continuing the random
    stream and Box-Muller cache of the event's previous call): the C
    restatement reproduces the reference's fixture bit for bit."""
    from cases import CHAIN
    data = np.load(os.path.join(GOLDEN, "chain_geometry_loop.npz"))
    s0, s1, r1, calls = _chain(port, CHAIN["seed"], CHAIN["first_event"])
    assert np.array_equal(s0, data["initial"])
    assert calls == int(data["calls"])
    same, _ = compare(s1, r1, data["final"], data["results"])
    assert same.all(), "%d / %d events differ" % ((~same).sum(), len(same))
    for f in ("draws", "randn_done", "randn_next"):
        assert np.array_equal(r1[f], data["results"][f]), f
    # The carry matters: the fast regime consumes draws, and restarting
    # the stream at each call replays those of the detailed regime.
    _, s2, r2, _ = _chain(port, CHAIN["seed"], CHAIN["first_event"], carry=0)
    both = s0["energy"] < 1E+02
    assert np.any(s2["energy"][both] != s1["energy"][both])
    assert np.array_equal(s2["energy"][~both], s1["energy"][~both])


def test_port_chain_matches_reference_fresh_events(port, reference):
    from cases import CHAIN
    a = _chain(port, CHAIN["seed"] + 1, 70000)
    b = _chain(reference, CHAIN["seed"] + 1, 70000)
    same, _ = compare(a[1], a[2], b[1], b[2])
    assert same.all()
    assert np.array_equal(a[2]["draws"], b[2]["draws"])


def test_reference_functions_reproduce_dump_dcs_tables(dump, port,
                                                       tmp_path):
    """The per element DEL tables of the shipped dump are those of the
    reference functions that the device table builder restates
    (compute_dcs_integral for CSn, dcs_tabulate_row and the low energy
    envelope exponents of compute_dcs_table): recomputed by the reference
    library on the loaded physics, they come out bit for bit. This pins
    which reference code the device tabulation must follow."""
    import oracle
    if not oracle.reference_available() and not oracle.build_reference():
        pytest.skip("reference sources not available")
    path = tmp_path / "muon.pumas"
    path.write_bytes(dump)
    ref = oracle.Reference(str(path), private=True)
    want = port.dcs_tables()
    shape = want["csn"].shape[1:] + (len(want["x"]),)
    got, seconds = ref.dcs_tables(shape)
    assert np.array_equal(got["csn"], want["csn"])
    assert np.array_equal(got["dcs"], want["dcs"])
    assert np.array_equal(got["alpha"], want["alpha"])
    assert np.all(seconds > 0.)


@pytest.mark.parametrize("name", ["muon", "tau", "muon_kkp", "muon_abb",
                                  "tau_bbks"])
def test_port_tabulation_matches_dump(name):
    """The C restatement of the device table builder (cross sections,
    their slopes, DCS tables and envelope exponents from the physics'
    elements, energy grid and DCS models) reproduces the tables that the
    reference's pumas_physics_create wrote into each physics dump, bit for
    bit."""
    import oracle
    from cases import physics_dump
    port = oracle.Port(physics_dump(name), private=True)
    want = port.dcs_tables()
    got = port.dcs_tabulate(4)
    for k in ("csn", "csn_dk", "dcs", "alpha"):
        assert np.array_equal(got[k], want[k]), k
