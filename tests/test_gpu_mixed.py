"""Mixed-precision form against the FP64 form (GPU).

From the same state, one step in each form: the set of active contacts is the
same and the contact forces and the body resultants agree within 1e-4 of the
force scale (the largest contact normal force of the step).  The FP64 form is
itself bit-identical to the oracle (test_gpu_parity.py), so this bounds the
mixed form's error against the reference arithmetic."""
import numpy as np
import pytest

from conftest import CONF
from helpers import gpu_from_oracle
from test_gpu_parity import variant_conf

pytestmark = pytest.mark.gpu
TOL = 1e-4


def clone(g_src, scene, form):
    """A new engine holding the state (bodies + neighbour list) of g_src."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene
    g = GpuScene(form=form)
    g.upload_shapes(scene["shape_tables"])
    st = g_src.bodies()
    b = dict(scene["bodies"])
    for k in ["pos", "vel", "acc", "Q", "vrot", "arot"]:
        b[k] = st[k]
    g.upload_bodies(b, scene["n_driven"])
    scenes.set_scene_params(g, scene)
    g.upload_entries(g_src.entries())
    return g


def force_errors(g64, gm):
    e64, em = g64.entries(), gm.entries()
    assert len(e64["i"]) == len(em["i"])
    act = e64["active"]
    flips = int(np.sum(act != em["active"]))
    both = act & em["active"]
    fmax = float(np.max(np.abs(e64["fn"][act]))) if act.any() else 1.0
    err_fn = float(np.max(np.abs(e64["fn"][both] - em["fn"][both]))) / fmax if both.any() else 0.0
    err_ft = float(np.max(np.abs(e64["ft"][both] - em["ft"][both]))) / fmax if both.any() else 0.0
    b64, bm = g64.bodies(), gm.bodies()
    err_F = float(np.max(np.abs(b64["force"] - bm["force"]))) / fmax
    return {"flips": flips, "active": int(act.sum()), "fn": err_fn, "ft": err_ft, "F": err_F, "fmax": fmax}


def test_mixed_one_step_518_friction(golden_dir, oracle_lib, gpu_lib):
    from rockable_gb300.abi import RK_FORM_MIXED
    case = "518_poly"
    conf = variant_conf(str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_mixed.conf"),
                        subs=[(r"^muContact 0 0 0$", "muContact 0 0 0.4"), (r"^muContact 0 1 0$", "muContact 0 1 0.4"),
                              (r"^gravity 0 0 0$", "gravity 0 0 -9.81")])
    o = oracle_lib.Oracle(conf)
    g64 = gpu_from_oracle(o)
    gm = gpu_from_oracle(o)
    gm.set_form(RK_FORM_MIXED)
    g64.update_nl()
    gm.update_nl()
    g64.step(1)
    gm.step(1)
    r = force_errors(g64, gm)
    print("518 one step:", r)
    assert r["flips"] == 0
    assert r["fn"] <= TOL and r["ft"] <= TOL and r["F"] <= TOL, r


def test_mixed_one_step_settled_column(gpu_lib):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.column_collapse(n=3000, nshapes=128)
    gs = scenes.settle(scene, steps=2000)
    gs.step(50)
    g64 = clone(gs, scene, RK_FORM_FP64)
    gm = clone(gs, scene, RK_FORM_MIXED)
    g64.update_nl()
    gm.update_nl()
    g64.step(1)
    gm.step(1)
    r = force_errors(g64, gm)
    print("column one step:", r)
    assert r["active"] > 1000
    assert r["flips"] <= max(1, r["active"] // 10000)
    assert r["fn"] <= TOL and r["F"] <= TOL, r
    # a short horizon: the contact population and energy stay together
    g64.step(200)
    gm.step(200)
    s64, sm = g64.stats(), gm.stats()
    print("after 200 steps:", s64, sm)
    assert abs(s64["n_active"] - sm["n_active"]) <= 0.01 * s64["n_active"] + 5
    assert abs(s64["e_trans"] - sm["e_trans"]) <= 0.05 * s64["e_trans"] + 1e-12
