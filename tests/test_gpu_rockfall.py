"""Breakable bonded rockfall at size (GPU): 40 blocks of 500 hull grains with
vertex bonds made by the conf's own stickVerticesInClusters and Weibull
setVariableStickParams (the C++ host runs them at load), hitting a 30 degree
slope at 10 m/s.  The mixed form's set of broken interfaces equals the plain
FP64 form's after every one of the first 1000 steps, and bonds do break."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_rockfall_rupture_set_matches_plain_every_step(gpu_lib, tmp_path):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import HostScene, RK_FORM_MIXED
    sc = scenes.rockfall_bonded()
    conf = scenes.write_conf(sc, str(tmp_path))
    plain, mixed = HostScene(conf), HostScene(conf)
    mixed.gpu.set_form(RK_FORM_MIXED)
    for h in (plain, mixed):
        h.gpu.update_nl()
    _, _, b0 = plain.gpu.interfaces()
    nif = len(b0)
    assert nif > 20000 and np.sum(plain.gpu.entries()["bond"] >= 0) > 100000
    bad = []
    for step in range(1, 1001):
        plain.gpu.step(1)
        mixed.gpu.step(1)
        _, _, bp = plain.gpu.interfaces()
        _, _, bm = mixed.gpu.interfaces()
        if not np.array_equal(bp, bm):
            bad.append((step, int(np.sum(bp != bm))))
    broke = int(bp.sum() - b0.sum())
    print("interfaces %d, broken in 1000 steps %d, steps with different sets %s" % (nif, broke, bad[:10]))
    assert broke > 100
    assert not bad
    plain.close()
    mixed.close()
