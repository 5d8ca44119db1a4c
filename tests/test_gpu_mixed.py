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


def force_errors(g64, gm, n_driven=0):
    """Largest errors of the step's contact forces and of the free bodies'
    resultants, over the step's largest contact normal force (the driven
    bodies' resultants, sums of thousands of FP32-rounded terms that feed no
    state, are reported apart)."""
    e64, em = g64.entries(), gm.entries()
    assert len(e64["i"]) == len(em["i"])
    act = e64["active"]
    flips = int(np.sum(act != em["active"]))
    both = act & em["active"]
    fmax = float(np.max(np.abs(e64["fn"][act]))) if act.any() else 1.0
    err_fn = float(np.max(np.abs(e64["fn"][both] - em["fn"][both]))) / fmax if both.any() else 0.0
    err_ft = float(np.max(np.abs(e64["ft"][both] - em["ft"][both]))) / fmax if both.any() else 0.0
    b64, bm = g64.bodies(), gm.bodies()
    dF = np.abs(b64["force"] - bm["force"]).max(axis=1)
    err_F = float(dF[n_driven:].max()) / fmax
    err_Fd = float(dF[:n_driven].max()) / fmax if n_driven else 0.0
    return {"flips": flips, "active": int(act.sum()), "fn": err_fn, "ft": err_ft, "F": err_F, "F_driven": err_Fd,
            "fmax": fmax}


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
    scene = scenes.column_collapse(n=3000, nshapes=128, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=2000)
    gs.step(50)
    g64 = clone(gs, scene, RK_FORM_FP64)
    gm = clone(gs, scene, RK_FORM_MIXED)
    g64.update_nl()
    gm.update_nl()
    g64.step(1)
    gm.step(1)
    r = force_errors(g64, gm, scene["n_driven"])
    print("column one step:", r)
    assert r["active"] > 1000
    assert r["flips"] <= max(1, r["active"] // 10000)
    # a resultant adds up to a few dozen contact terms, each within TOL of
    # the largest force (per-body relative errors: the per-result test)
    assert r["fn"] <= TOL and r["F"] <= 3 * TOL, r
    # a short horizon: the contact population and energy stay together
    g64.step(200)
    gm.step(200)
    s64, sm = g64.stats(), gm.stats()
    print("after 200 steps:", s64, sm)
    assert abs(s64["n_active"] - sm["n_active"]) <= 0.01 * s64["n_active"] + 5
    assert abs(s64["e_trans"] - sm["e_trans"]) <= 0.05 * s64["e_trans"] + 1e-12


def _sticked_variant(golden_dir):
    case = "518_poly"
    conf = variant_conf(
        str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_stick_mixed.conf"),
        subs=[(r"^forceLaw Default", "forceLaw StickedLinks"), (r"^muContact 0 0 0$", "muContact 0 0 0.3"),
              (r"^gravity 0 0 0$", "gravity 0 0 -500"), (r"^dt .*$", "dt 2e-07")],
        append="knInnerBond 0 0 100\nktInnerBond 0 0 80\nkrInnerBond 0 0 1e-4\nen2InnerBond 0 0 0.1\n"
               "fn0InnerBond 0 0 0.05\nft0InnerBond 0 0 0.05\nmom0InnerBond 0 0 1.0\npowInnerBond 0 0 2\n")
    open(conf, "a").write("stickVerticesInClusters 0.001\n")
    return conf


def test_mixed_rupture_set_matches_plain(golden_dir, oracle_lib, gpu_lib):
    """Bonded scene (stickVerticesInClusters, StickedLinks law, strengths
    lowered so that bonds break): the set of broken interfaces of the mixed
    form equals the FP64 form's after every 50 steps."""
    from helpers import set_params_from_oracle
    from rockable_gb300.abi import RK_FORM_FP64, RK_FORM_MIXED
    o = oracle_lib.Oracle(_sticked_variant(golden_dir))
    for name, v in [("fn0InnerBond", 2e-5), ("ft0InnerBond", 1e-6)]:
        o.set_param(name, 0, 0, v)
    g64 = gpu_from_oracle(o, form=RK_FORM_FP64)
    gm = gpu_from_oracle(o, form=RK_FORM_MIXED)
    for g in (g64, gm):
        set_params_from_oracle(g, o)
        g.update_nl()
    seen = 0
    for k in range(6):
        g64.step(50)
        gm.step(50)
        _, _, b64 = g64.interfaces()
        _, _, bm = gm.interfaces()
        assert np.array_equal(b64, bm), (k, np.flatnonzero(b64 != bm)[:10])
        seen = int(b64.sum())
    assert seen > 0


def test_long_run_statistics_match_plain(gpu_lib):
    """A 3000-step column collapse in the mixed form and with the learned
    skin: the time averages of the kinetic energy and of the coordination
    number stay within 5 % of the FP64 form's (the trajectories themselves
    diverge, as in any granular flow)."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.column_collapse(n=3000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=1200)
    src = scenes.scene_from_gpu(scene, gs)
    gs.close()
    series = {}
    for name in ["plain", "mixed", "skin"]:
        g = GpuScene(form=RK_FORM_FP64 if name == "plain" else RK_FORM_MIXED)
        g.upload_shapes(src["shape_tables"])
        g.upload_bodies(src["bodies"], src["n_driven"])
        scenes.set_scene_params(g, src)
        g.upload_entries(src["entries"])
        if name == "skin":
            g.set_skin(use_mlp=True, skin_min=0.05 * scene["dVerlet"], skin_max=4.0 * scene["dVerlet"],
                       interval_min=2, interval_max=1000, seed=5)
        ke, z = [], []
        for _ in range(12):
            g.step(250)
            st = g.stats()
            ke.append(st["e_trans"] + st["e_rot"])
            z.append(st["coordination"])
        series[name] = (np.mean(ke), np.mean(z))
        g.close()
    print("long-run means (kinetic energy, coordination):", series)
    for name in ["mixed", "skin"]:
        for q in range(2):
            ref = series["plain"][q]
            assert abs(series[name][q] - ref) <= 0.05 * abs(ref), (name, q, series)


def test_mixed_free_flight_tracks_fp64():
    """No contacts: 200 grains far apart, spinning fast about random axes
    (torque-free precession through Euler's equations) and falling under
    gravity for 5000 steps.  The mixed form advances the FP64 state by FP32
    increments whose relative error is at most 2^-24; a constant increment
    (free fall) repeats its rounding every step, so the state deviates from
    the FP64 form's by up to ~1e-7 of its accumulated change, and no more.
    The quaternions stay unit to FP64 precision."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.drop_bodies(scenes.column_collapse(n=200, nshapes=16, semi=(0.0025, 0.0075)), [0])
    b = dict(scene["bodies"])
    rng = np.random.default_rng(21)
    n = len(b["mass"])
    b["pos"] = np.asarray(b["pos"]) * 20.0
    b["vel"] = rng.normal(size=(n, 3))
    b["vrot"] = rng.normal(size=(n, 3)) * 40.0
    scene = dict(scene, bodies=b, entries=None)
    out = {}
    for form in (RK_FORM_FP64, RK_FORM_MIXED):
        g = GpuScene(form=form)
        g.upload_shapes(scene["shape_tables"])
        g.upload_bodies(b, scene["n_driven"])
        scenes.set_scene_params(g, scene)
        g.update_nl()
        g.step(5000)
        out[form] = g.bodies()
        g.close()
    a, m = out[RK_FORM_FP64], out[RK_FORM_MIXED]
    assert len(a["pos"]) == n
    rel = 4 * 2.0 ** -24
    t = 5000 * scene["dt"]
    g = np.linalg.norm(scene["gravity"])
    # per body: the length of the path (|v0| t + g t^2 / 2) and of the velocity change (g t)
    moved = np.linalg.norm(b["vel"], axis=1) * t + 0.5 * g * t * t
    dv_acc = g * t
    dpos = np.linalg.norm(a["pos"] - m["pos"], axis=1)
    dv = np.linalg.norm(a["vel"] - m["vel"], axis=1)
    dq = np.abs(a["Q"] - m["Q"]).max()
    dw = (np.linalg.norm(a["vrot"] - m["vrot"], axis=1) / np.linalg.norm(a["vrot"], axis=1)).max()
    unit = np.abs(np.linalg.norm(m["Q"], axis=1) - 1.0).max()
    print("free flight: |dQ| %.3g |dpos| %.3g m (moved %.3g) |dw|/|w| %.3g |dv| %.3g m/s (change %.3g), ||Q|-1| %.3g"
          % (dq, dpos.max(), moved.max(), dw, dv.max(), dv_acc, unit))
    assert np.abs(a["vrot"]).max() > 20.0  # spinning throughout
    assert np.all(dpos <= rel * moved + 1e-12), float(np.max(dpos - rel * moved))
    assert np.all(dv <= rel * dv_acc + 1e-12), float(np.max(dv - rel * dv_acc))
    # rotations of at most ~0.6 rad: the same relative bound on the quaternions
    assert dq <= 1e-7 and dw <= 1e-5, (dq, dw)
    assert unit <= 1e-14


def per_result_errors(g0, g64, gm, n_driven, bound):
    """Per-result relative errors of the mixed form against the FP64 form
    after one step from the same state (g0: the bodies before it):
      fn, ft   per active entry, |mixed - fp64| / max(|fp64|, 1e-6 x the
               step's median |fn|) (the floor keeps a contact that has just
               touched, with a force near zero, from dominating);
      Mi, Mj   per active entry, the moment terms on i and on j over the
               contact's largest possible moment |f| x (the body's bounding
               radius) (a contact whose force passes near the centre has a
               small moment that FP32 lever arms resolve only to that scale);
      force,   per free body, |mixed - fp64| / the sum of the magnitudes of
      moment   the body's active contact forces (its own force scale: a body
               near equilibrium has a small net force);
      pos, Q   per free body, |mixed - fp64| / the step's change |fp64 - before|
               (floors 1e-15 for pos, 1e-10 for Q: the unit quaternion is
               renormalised every step, exactly only to FP64 rounding, 1e-16,
               of |Q| = 1, so smaller rotations are compared at that floor).
    Returns, per quantity, the largest error, the 99.9th percentile and the
    fraction within 1e-4."""
    e64, em = g64.entries(), gm.entries()
    both = e64["active"] & em["active"]
    med = float(np.median(np.abs(e64["fn"][both]))) if both.any() else 1.0
    floor = 1e-6 * med
    fn_err = np.abs(em["fn"][both] - e64["fn"][both]) / np.maximum(np.abs(e64["fn"][both]), floor)
    ftm = np.linalg.norm(e64["ft"][both], axis=1)
    ft_err = np.linalg.norm(em["ft"][both] - e64["ft"][both], axis=1) / np.maximum(ftm, floor)
    b64, bm = g64.bodies(), gm.bodies()
    nb = len(b64["pos"])
    scale = np.zeros(nb)
    mag = np.abs(e64["fn"][both]) + ftm
    np.add.at(scale, e64["i"][both], mag)
    np.add.at(scale, e64["j"][both], mag)
    out = {}
    free = slice(n_driven, nb)
    have = scale[free] > 0
    for k in ["force", "moment"]:
        out[k] = np.linalg.norm(bm[k][free] - b64[k][free], axis=1)[have] / scale[free][have]
    for k, floor_k in [("pos", 1e-15), ("Q", 1e-10)]:
        step = np.linalg.norm(b64[k][free] - g0[k][free], axis=1)
        out[k] = np.linalg.norm(bm[k][free] - b64[k][free], axis=1) / np.maximum(step, floor_k)
    out["fn"], out["ft"] = fn_err, ft_err
    (f64, mi64, mj64), (_, mim, mjm) = g64.contributions(), gm.contributions()
    fmag = np.linalg.norm(f64[both], axis=1)
    for k, a64, am, owner in [("Mi", mi64, mim, e64["i"]), ("Mj", mj64, mjm, e64["j"])]:
        scale = np.maximum(fmag * bound[owner[both]], 1e-300)
        out[k] = np.linalg.norm(am[both] - a64[both], axis=1) / scale
    return {k: {"max": float(v.max()) if len(v) else 0.0, "p999": float(np.percentile(v, 99.9)) if len(v) else 0.0,
                "within_1e-4": float(np.mean(v <= 1e-4)) if len(v) else 1.0, "n": int(len(v))}
            for k, v in out.items()}


def test_mixed_per_result_relative_errors_settled_column(gpu_lib):
    """One step from a settled, contact-rich column in both forms (the dense
    pile settled by gravity between walls for 20000 steps, scenes.loaded, and
    released): per-result relative errors (per_result_errors).  The normal
    and tangential forces and the moment terms of 99.9 % of the active
    contacts, the body resultants (relative to the body's own contact
    forces) and the step's motion agree within 1e-4."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.column_collapse(n=3000, nshapes=128, semi=(0.0025, 0.0075), column=(0.2, 0.2, 1.5), walls=True)
    src = scenes.loaded(scene, 20000)
    gs = GpuScene(form=RK_FORM_FP64)
    gs.upload_shapes(src["shape_tables"])
    gs.upload_bodies(src["bodies"], src["n_driven"])
    scenes.set_scene_params(gs, src)
    gs.upload_entries(src["entries"])
    scene = src
    g64 = clone(gs, scene, RK_FORM_FP64)
    gm = clone(gs, scene, RK_FORM_MIXED)
    g64.update_nl()
    gm.update_nl()
    before = g64.bodies()
    g64.step(1)
    gm.step(1)
    bound = np.array([scene["shapes"][k]["bound"] for k in scene["bodies"]["shape"]]) * scene["bodies"]["homothety"]
    r = per_result_errors(before, g64, gm, scene["n_driven"], bound)
    print("per-result relative errors:", r)
    assert r["fn"]["n"] > 1000
    for k in ["fn", "ft", "Mi", "Mj", "force", "moment", "pos", "Q"]:
        assert r[k]["p999"] <= 1e-4, (k, r[k])


def test_headline_contact_set_equals_fp64_rebuild_every_step(gpu_lib):
    """The headline form (mixed precision, learned skin with exact contact
    detection) on a contact-rich column for 1000 steps: the dense pile,
    settled by gravity between walls for 20000 steps and released, collapses;
    at every 10th step the headline form's active sub-contact set equals the
    one the FP64 form finds at the same positions from a neighbour list
    rebuilt from scratch (a fresh context: rk_update_nl, then the load-time
    force evaluation)."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.column_collapse(n=2000, nshapes=64, semi=(0.0025, 0.0075), column=(0.15, 0.15, 1.5), walls=True)
    src = scenes.loaded(scene, 20000)
    h = GpuScene(form=RK_FORM_MIXED)
    h.upload_shapes(src["shape_tables"])
    h.upload_bodies(src["bodies"], src["n_driven"])
    scenes.set_scene_params(h, src)
    h.upload_entries(src["entries"])
    d = src["dVerlet"]
    h.set_skin(use_mlp=True, skin_min=0.1 * d, skin_max=4.0 * d, interval_min=2, interval_max=300, seed=7,
               exact_contacts=True)

    def active_keys(e):
        a = e["active"]
        return set(zip(e["i"][a].tolist(), e["j"][a].tolist(), e["type"][a].tolist(), e["isub"][a].tolist(),
                       e["jsub"][a].tolist()))

    checked, mismatched, active = 0, [], []
    for step in range(1, 1001):
        h.step(1)
        if step % 10:
            continue
        st = h.bodies()
        ha = active_keys(h.entries())
        f = GpuScene(form=RK_FORM_FP64)
        f.upload_shapes(src["shape_tables"])
        b = dict(src["bodies"])
        for k in ["pos", "vel", "acc", "Q", "vrot", "arot"]:
            b[k] = st[k]
        f.upload_bodies(b, src["n_driven"])
        scenes.set_scene_params(f, src)
        f.update_nl()
        f.accelerations()
        fa = active_keys(f.entries())
        f.close()
        checked += 1
        active.append(len(fa))
        if ha != fa:
            mismatched.append((step, len(ha - fa), len(fa - ha)))
    print("checked %d steps, load %s, active contacts %d..%d, mismatches %s, skin %s" % (
        checked, src["load"], min(active), max(active), mismatched[:10], h.skin_stats()))
    assert checked == 100 and np.mean(active) >= 2000  # at least one active sub-contact per grain
    assert not mismatched
