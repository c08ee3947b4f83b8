"""Generate the golden fixtures of the parity tests from the reference.

Runs every case of tests/cases.py through the unmodified reference library
(oracle/_ref, built from the reference sources by oracle/Makefile) and stores
the initial and final states and per event results as tests/golden/<case>.npz.
These fixtures let machines without the reference sources check the engine
against the reference's own outputs.

usage: python tests/golden/make_golden.py [case ...]   (default: all cases)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
import pumas_gb300  # noqa: E402
from cases import CASES, make_states  # noqa: E402
from conftest import oracle_config, oracle_geometry  # noqa: E402


def main():
    oracle.build_reference()
    dump = pumas_gb300.default_dump()
    path = os.path.join(ROOT, "pumas_gb300", "data", "_build", "golden.pumas")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "wb") as f:
        f.write(dump)
    ref = oracle.Reference(path)
    names = sys.argv[1:] or list(CASES)
    for name in names:
        case = CASES[name]
        s0 = make_states(name)
        geo = oracle_geometry(ref, case["geometry"])
        cfg = oracle_config(case["config"], case["seed"])
        s1, r1 = ref.transport(cfg, geo, s0, 0, 8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), initial=s0,
                            final=s1, results=r1)
        print("%-28s %5d events, %7.1f steps/event, status %s" % (
            name, len(s0), r1["steps"].mean(), np.unique(r1["status"])))


if __name__ == "__main__":
    main()
