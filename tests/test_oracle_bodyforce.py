"""The oracle's BodyForce plugins (Rockable.cpp:1026-1040 parsing, 470-473
writing, 2887-2901 applying; src/BodyForces/BodyForce_*.cpp) against a
numpy statement of each plugin's formula on the loaded state (CPU)."""
import re

import numpy as np
import pytest

from conftest import CONF

CASE = "518_poly"
LINES = {
    "AttractingPoint": "BodyForce AttractingPoint 0.01 -0.02 0.03 1000",
    "ViscousFluid": "BodyForce ViscousFluid 0.001",
    "PreferredDirection": "BodyForce PreferredDirection 0 0 2 1 1 0 0.001",
}


def with_line(golden_dir, tmp_path, line, name):
    text = open(golden_dir / CASE / CONF[CASE]).read()
    k = text.index("Particles")
    dst = golden_dir / CASE / ("bf_%s.conf" % name)
    dst.write_text(text[:k] + line + "\n" + text[k:])
    return str(dst)


def qrot(q, u):
    s, v = q[:, :1], q[:, 1:]
    t = 2.0 * np.cross(v, u)
    return u + s * t + np.cross(v, t)


def unit(a):
    n = np.linalg.norm(a, axis=1, keepdims=True)
    return np.where(n > 0, a / np.where(n > 0, n, 1.0), a)


@pytest.mark.parametrize("name", sorted(LINES))
def test_body_force_formula(name, golden_dir, oracle_lib, tmp_path):
    """At load the oracle's accelerations pass adds the plugin's force and
    moment to every free body: the difference to the same scene without it
    is the formula evaluated on the loaded state."""
    base = oracle_lib.Oracle(str(golden_dir / CASE / CONF[CASE]))
    o = oracle_lib.Oracle(with_line(golden_dir, tmp_path, LINES[name], name))
    kind, prm, vol = o.body_force()
    assert kind == {"AttractingPoint": 1, "PreferredDirection": 2, "ViscousFluid": 3}[name]
    assert np.array_equal(prm, [float(x) for x in LINES[name].split()[2:]])
    b, b0, st = o.bodies(), base.bodies(), o.body_static()
    nd = o.n_driven
    F = np.zeros_like(b["force"])
    M = np.zeros_like(b["moment"])
    if name == "AttractingPoint":
        d = unit(prm[:3] - b["pos"])
        F = (st["mass"] * prm[3])[:, None] * d
    elif name == "ViscousFluid":
        F = (0.5 * 0.47 * prm[0] * vol ** (2.0 / 3.0))[:, None] * b["vel"] ** 2
    else:
        axb = unit(qrot(b["Q"], np.broadcast_to(prm[:3] / np.linalg.norm(prm[:3]), b["pos"].shape)))
        axis = prm[3:6] / np.linalg.norm(prm[3:6])
        u = unit(np.cross(axis, axb))
        cosa = axb @ axis
        ang = np.arccos(np.clip(cosa, -1, 1))
        sgn = np.where(cosa < 0, 1.0, -1.0)
        ang = np.where(cosa < 0, np.pi - ang, ang)
        M = (2.0 * prm[6] / np.pi * sgn * ang)[:, None] * u
    F[:nd] = 0.0
    M[:nd] = 0.0
    scale = max(np.abs(F).max(), np.abs(M).max())
    assert scale > 0
    tol = 1e-9 * (scale + np.abs(b0["force"]).max() + np.abs(b0["moment"]).max())
    assert np.abs((b["force"] - b0["force"]) - F).max() <= tol
    assert np.abs((b["moment"] - b0["moment"]) - M).max() <= tol


@pytest.mark.parametrize("name", sorted(LINES))
def test_body_force_written_back(name, golden_dir, oracle_lib, tmp_path):
    """save_conf writes the plugin after gravity, as read (the preferred
    direction's axes normalised), at the header's default stream precision
    (6 significant digits, like the gravity line)."""
    o = oracle_lib.Oracle(with_line(golden_dir, tmp_path, LINES[name], name))
    out = tmp_path / "o.conf"
    o.save_conf(str(out))
    lines = out.read_text().splitlines()
    k = [i for i, l in enumerate(lines) if l.startswith("gravity ")][0]
    got = lines[k + 1].split()
    assert got[:2] == LINES[name].split()[:2]
    want = [float(x) for x in LINES[name].split()[2:]]
    if name == "PreferredDirection":
        want[0:3] = list(np.array(want[0:3]) / np.linalg.norm(want[0:3]))
        want[3:6] = list(np.array(want[3:6]) / np.linalg.norm(want[3:6]))
    assert np.allclose([float(x) for x in got[2:]], want, rtol=1e-5, atol=0)
