"""BodyForce plugins on the GPU step (Rockable.cpp:2887-2901) against the
oracle (GPU): AttractingPoint and ViscousFluid bit for bit over 200 steps of
the 518-polyhedra scene (the fluid's density is small: its force, always
along +v^2, feeds back on the velocity); PreferredDirection, whose acos is
the device's and not the host C library's (both within 2 ulp of the exact
value), within 1e-13 of every field's range after one step and with the same
contact set after 200; the C++ host writes the plugin back like the
oracle."""
import ctypes
import os

import numpy as np
import pytest

from conftest import CONF, ROOT
from helpers import BODY_FIELDS, bitwise_equal, gpu_from_oracle, key_tuples
from test_oracle_bodyforce import CASE, LINES, with_line

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(LINES))
def test_body_force_steps_match_oracle(name, golden_dir, oracle_lib, gpu_lib, tmp_path):
    conf = with_line(golden_dir, tmp_path, LINES[name], name)
    o = oracle_lib.Oracle(conf)
    g = gpu_from_oracle(o)
    base = oracle_lib.Oracle(str(golden_dir / CASE / CONF[CASE]))
    for x in (o, g, base):
        x.update_nl()
    if name == "PreferredDirection":
        o.run(1)
        g.step(1)
        ob, gb = o.bodies(), g.bodies()
        for k in BODY_FIELDS:
            rng = max(float(np.abs(ob[k]).max()), 1e-300)
            assert float(np.abs(ob[k] - gb[k]).max()) <= 1e-13 * rng, k
        o.run(199)
        g.step(199)
    else:
        o.run(200)
        g.step(200)
    base.run(200)
    ob, gb, bb = o.bodies(), g.bodies(), base.bodies()
    # the plugin acts: the state differs from the run without it
    assert any(not np.array_equal(ob[k], bb[k]) for k in ["vel", "vrot"])
    assert key_tuples(o.entries()) == key_tuples(g.entries())
    if name != "PreferredDirection":
        bad = [k for k in BODY_FIELDS if not bitwise_equal(ob[k], gb[k])]
        assert not bad, bad
        oe, ge = o.entries(), g.entries()
        for k in ["dn", "fn", "ft"]:
            assert bitwise_equal(oe[k], ge[k]), k
    g.close()


def test_host_writes_body_force(golden_dir, oracle_lib, gpu_lib, tmp_path):
    conf = with_line(golden_dir, tmp_path, LINES["PreferredDirection"], "PreferredDirection")
    o = oracle_lib.Oracle(conf)
    o.save_conf(str(tmp_path / "oracle.conf"))
    lib = ctypes.CDLL(os.path.join(ROOT, "rockable_gb300", "_lib", "librk_host.so"))
    lib.rkh_open.restype = ctypes.c_void_p
    lib.rkh_error.restype = ctypes.c_char_p
    lib.rkh_save_conf.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.rkh_close.argtypes = [ctypes.c_void_p]
    h = lib.rkh_open(conf.encode())
    assert h, lib.rkh_error()
    assert lib.rkh_save_conf(h, str(tmp_path / "host.conf").encode()) == 0, lib.rkh_error()
    lib.rkh_close(h)
    pick = lambda p: [l for l in open(p).read().splitlines() if l.startswith("BodyForce")]
    assert pick(tmp_path / "host.conf") == pick(tmp_path / "oracle.conf") != []
