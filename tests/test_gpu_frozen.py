"""The FP64 GPU form against the oracle's frozen results (GPU): the state
after each case of tests/oracle_cases.py (Avalanche law, StickedLinks bonds
and rupture, the linkCells list, the dynamic guard) must equal the frozen
digests of tests/golden/oracle/ bit for bit.  The oracle only parses the
case's conf and hands the initial state over; the comparison is with the
committed files."""
import os

import numpy as np
import pytest

import oracle_cases
from conftest import CONF
from helpers import gpu_from_oracle, set_params_from_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(oracle_cases.CASES))
def test_gpu_reproduces_frozen_state(name, golden_dir, oracle_lib, gpu_lib):
    c = oracle_cases.CASES[name]
    conf = oracle_cases.make_conf(name, str(golden_dir / "518_poly" / CONF["518_poly"]),
                                  str(golden_dir / "518_poly" / ("gfrozen_" + name + ".conf")))
    o = oracle_lib.Oracle(conf)
    for p, v in c.get("after_load", []):
        o.set_param(p, 0, 0, v)
    g = gpu_from_oracle(o)
    set_params_from_oracle(g, o)
    n_if0 = len(o.interfaces())
    g.update_nl()
    n = 0
    for k in c["steps"]:
        n += g.step(k)["nl_updates"]
    _, _, broken = g.interfaces()
    st = oracle_cases.state(g.bodies(), g.entries(), n_if0 - int(broken.sum()), n)
    ref = dict(np.load(os.path.join(oracle_cases.GOLDEN, name + ".npz")))
    bad = oracle_cases.diff(ref, st)
    assert not bad, "%s: %s differ (max |dpos| %g)" % (name, bad, float(np.max(np.abs(ref["pos"] - st["pos"]))))
    g.close()
