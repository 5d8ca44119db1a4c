"""The C++ host (conf in, conf out) driving the GPU engine reproduces the
reference's regression goldens text-identically (GPU), the way the
reference's own ctest compares them (src/Apps/run.cpp:38-92)."""
import os
import subprocess

import pytest

from conftest import CONF, ROOT

pytestmark = pytest.mark.gpu

CLI = os.path.join(ROOT, "rockable_gb300", "_lib", "rockable-gb300")


@pytest.mark.parametrize("case,out", [("512_particles", "conf101"), ("518_poly", "conf3001")])
def test_cli_reproduces_golden(case, out, golden_dir, gpu_lib, tmp_path):
    d = golden_dir / case
    r = subprocess.run([CLI, str(d / CONF[case]), "-o", str(tmp_path), "-n", str(tmp_path / out), "-r",
                        str(d / "golden.conf")], cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "regression: identical" in r.stdout


def _section(text, name):
    """The lines of a conf section: its header 'name N' and the N lines after."""
    lines = text.splitlines()
    for k, l in enumerate(lines):
        if l.startswith(name + " "):
            n = int(l.split()[1])
            return lines[k:k + 1 + n]
    return []


def test_host_bond_setup_matches_oracle(golden_dir, oracle_lib, gpu_lib, tmp_path):
    """The host's load-time bond setup -- stickVerticesInClusters
    (PreproCommand_stickVerticesInClusters.cpp:56-141) and a Weibull
    setVariableStickParams on the inner bonds (PreproCommand_setVariableStick
    Params.cpp:57-94) -- against the oracle's: the interfaces (pairs, bonds,
    per-interface parameters with their Weibull strengths) and the bonded
    vertex-vertex interactions written by each at load are text-identical."""
    import ctypes
    import re
    import oracle_cases
    case = "518_poly"
    src = str(golden_dir / case / CONF[case])
    conf = str(golden_dir / case / "v_bonds_host.conf")
    text = open(src).read()
    for a, b in oracle_cases.CASES["sticked_rupture_518"]["subs"]:
        text = re.sub(a, b, text, flags=re.M)
    k = text.index("Particles")
    text = text[:k] + oracle_cases.BOND_PARAMS + text[k:] + "stickVerticesInClusters 0.001\n" + \
        "setVariableStickParams fn0 inner 1000 5\n"
    open(conf, "w").write(text)
    o = oracle_lib.Oracle(conf)
    assert len(o.interfaces()) >= 5
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
    ot, ht = open(tmp_path / "oracle.conf").read(), open(tmp_path / "host.conf").read()
    for name in ["Interfaces", "Interactions"]:
        a, b = _section(ot, name), _section(ht, name)
        diff = [(k, x, y) for k, (x, y) in enumerate(zip(a, b)) if x != y]
        for k, x, y in diff[:3]:  # field by field
            print(name, k, [(f, u, v) for f, (u, v) in enumerate(zip(x.split(), y.split())) if u != v])
        assert len(a) > 1 and len(a) == len(b) and not diff, (name, len(a), len(b), len(diff))
