"""Freeze the oracle's results on the cases of tests/oracle_cases.py.

    python tests/golden/make_oracle_goldens.py

writes tests/golden/oracle/<case>.npz (compressed): the state after the
case's steps, as tests/oracle_cases.state() defines it.  The cases are
deterministic (no random draws); the oracle is built with -ffp-contract=off,
so the files are the same on any host."""
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle_cases  # noqa: E402
from conftest import CONF, extract_case  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    oracle.build()
    d = tempfile.mkdtemp(prefix="rk_frozen_")
    extract_case("518_poly", os.path.join(d, "518_poly"))
    src = os.path.join(d, "518_poly", CONF["518_poly"])
    os.makedirs(oracle_cases.GOLDEN, exist_ok=True)
    for name in oracle_cases.CASES:
        conf = oracle_cases.make_conf(name, src, os.path.join(d, "518_poly", name + ".conf"))
        _, st = oracle_cases.run_oracle(oracle, conf, name)
        np.savez_compressed(os.path.join(oracle_cases.GOLDEN, name + ".npz"), **st)
        print(name, "entries", int(st["n_entries"][0]), "list updates", int(st["nl_updates"][0]),
              "interfaces left", int(st["n_interfaces"][0]))


if __name__ == "__main__":
    main()
