"""Generate the golden fixtures of the parity tests from the reference.

Runs every case of tests/cases.py through the unmodified reference library
(oracle/_ref, built from the reference sources by oracle/Makefile) and stores
the initial and final states and per event results as tests/golden/<case>.npz.
These fixtures let machines without the reference sources check the engine
against the reference's own outputs.

usage: python tests/golden/make_golden.py [case ...]   (default: all cases)
       python tests/golden/make_golden.py frames [case ...]   (recorder
       frames of the cases of RECORD_CASES)
       python tests/golden/make_golden.py physics   (the physics dumps with
       non-default DCS models of PHYSICS_MODELS, by the reference's
       pumas_physics_create)
       python tests/golden/make_golden.py chain   (events transported over
       several calls, the loop of examples/pumas/geometry.c:269-312, see
       tests/cases.py CHAIN)
"""
import gzip
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
import pumas_gb300  # noqa: E402
from cases import (CASES, CHAIN, chain_states, make_states,  # noqa: E402
                   physics_dump, run_chain)
from conftest import oracle_config, oracle_geometry  # noqa: E402


# Recorder cases: (case, recorder period, events, frames kept per event).
RECORD_CASES = [
    ("plain_csda", 1, 20, 4),
    ("rock_slab", 10, 24, 96),
    ("stack_forward_mixed", 5, 24, 96),
    ("stack_backward_straggled", 0, 24, 32),
    ("terrain_backward", 25, 16, 64),
]


# Physics dumps of the cases with non-default DCS models: name ->
# (particle, bremsstrahlung, pair production, photonuclear).
PHYSICS_MODELS = {
    "muon_kkp": ("muon", "KKP", "KKP", "BM"),
    "muon_abb": ("muon", "ABB", "SSR", "BBKS"),
    "tau_bbks": ("tau", "SSR", "SSR", "BBKS"),
}


def make_physics():
    """Build the dumps of PHYSICS_MODELS with the reference library."""
    ref = oracle.REFERENCE_DIR
    build = os.path.join(ROOT, "pumas_gb300", "data", "_build")
    exe = os.path.join(build, "make_physics")
    os.makedirs(build, exist_ok=True)
    subprocess.check_call([
        "cc", "-O3", "-std=c99", "-ffp-contract=off",
        "-I" + os.path.join(ref, "include"), "-o", exe,
        os.path.join(ROOT, "pumas_gb300", "data", "make_physics.c"),
        os.path.join(ref, "src", "pumas.c"), "-lm"])
    mdf = os.path.join(ROOT, "pumas_gb300", "data", "materials.xml")
    for name, models in PHYSICS_MODELS.items():
        dedx = os.path.join(build, "dedx-" + name)
        os.makedirs(dedx, exist_ok=True)
        raw = os.path.join(build, name + ".pumas")
        subprocess.check_call([exe, mdf, dedx, raw] + list(models))
        with open(raw, "rb") as f, gzip.GzipFile(
                physics_file(name), "wb", 9, mtime=0) as g:
            g.write(f.read())
        print("wrote", physics_file(name))


def physics_file(name):
    return os.path.join(HERE, "physics_%s.pumas.gz" % name)


def record_file(name, period):
    return os.path.join(HERE, "frames_%s_p%d.npz" % (name, period))


def make_frames(ref, names=None):
    """Frames of the reference's recorder for RECORD_CASES."""
    for name, period, n, max_frames in RECORD_CASES:
        if names and name not in names:
            continue
        case = CASES[name]
        s0 = make_states(name, n=n)
        geo = oracle_geometry(ref, case["geometry"])
        cfg = oracle_config(case["config"], case["seed"])
        s1, r1, frames, length = ref.transport_record(
            cfg, geo, s0, 0, period, max_frames)
        np.savez_compressed(record_file(name, period), initial=s0, final=s1,
                            results=r1, frames=frames, length=length,
                            period=period)
        print("%-28s period %d: %5.1f frames/event (max %d)" % (
            name, period, length.mean(), length.max()))


CHAIN_FILE = os.path.join(HERE, "chain_geometry_loop.npz")


def chain_transport(impl, seed, first_event):
    """The `transport` callable of cases.run_chain on a CPU oracle: every
    call carries each event's random state from its previous call."""
    geo = oracle_geometry(impl, CHAIN["geometry"])

    def transport(cfg, states, results):
        c = oracle_config(cfg, seed)
        c.carry = 1
        return impl.transport(c, geo, states, first_event, 8, results)
    return transport


def make_chain(ref):
    """The reference's final states after the loop of CHAIN."""
    s0 = chain_states()
    s1, r1, calls = run_chain(
        chain_transport(ref, CHAIN["seed"], CHAIN["first_event"]), s0)
    np.savez_compressed(CHAIN_FILE, initial=s0, final=s1, results=r1,
                        calls=calls)
    print("chain: %d events, %d calls, %.1f draws/event" % (
        len(s0), calls, r1["draws"].mean()))


def main():
    oracle.build_reference()
    dump = pumas_gb300.default_dump()
    path = os.path.join(ROOT, "pumas_gb300", "data", "_build", "golden.pumas")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "wb") as f:
        f.write(dump)
    ref = oracle.Reference(path)
    args = sys.argv[1:]
    if args and args[0] == "frames":
        make_frames(ref, args[1:])
        return
    if args and args[0] == "physics":
        make_physics()
        return
    if args and args[0] == "chain":
        make_chain(ref)
        return
    names = args or list(CASES)
    refs = {"muon": ref}
    for name in names:
        case = CASES[name]
        particle = case.get("physics", "muon")
        if particle not in refs:
            # Another physics in a private copy of the reference library.
            p = os.path.join(os.path.dirname(path), "golden_%s.pumas" %
                             particle)
            with open(p, "wb") as f:
                f.write(physics_dump(particle))
            refs[particle] = oracle.Reference(p, private=True)
        r = refs[particle]
        s0 = make_states(name)
        geo = oracle_geometry(r, case["geometry"])
        cfg = oracle_config(case["config"], case["seed"])
        s1, r1 = r.transport(cfg, geo, s0, 0, 8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), initial=s0,
                            final=s1, results=r1)
        print("%-28s %5d events, %7.1f steps/event, status %s" % (
            name, len(s0), r1["steps"].mean(), np.unique(r1["status"])))


if __name__ == "__main__":
    main()
