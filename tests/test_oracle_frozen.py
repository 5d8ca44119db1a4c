"""The oracle against its frozen results (CPU): the Avalanche law,
StickedLinks bonds and rupture, the linkCells list and the dynamic guard --
the paths no reference golden pins -- must reproduce, bit for bit, the state
frozen in tests/golden/oracle/ (tests/oracle_cases.py, written by
tests/golden/make_oracle_goldens.py).  A change of the oracle's arithmetic
shows here before it can move the GPU checks with it."""
import os

import numpy as np
import pytest

import oracle_cases
from conftest import CONF


@pytest.mark.parametrize("name", sorted(oracle_cases.CASES))
def test_oracle_reproduces_frozen_state(name, golden_dir, oracle_lib, tmp_path):
    conf = oracle_cases.make_conf(name, str(golden_dir / "518_poly" / CONF["518_poly"]),
                                  str(golden_dir / "518_poly" / ("frozen_" + name + ".conf")))
    _, st = oracle_cases.run_oracle(oracle_lib, conf, name)
    ref = dict(np.load(os.path.join(oracle_cases.GOLDEN, name + ".npz")))
    bad = oracle_cases.diff(ref, st)
    assert not bad, "%s: %s differ (max |dpos| %g)" % (name, bad, float(np.max(np.abs(ref["pos"] - st["pos"]))))
