"""Learned Verlet skin (GPU): the FP16 network's gradients against the CPU
FP64 model, and the skin policy on a settled pile -- the exact guard keeps the
contacts of a run that rebuilds every step, and the network's proposals are
compared with the method without it."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _engine(scene):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene
    g = GpuScene()
    g.upload_shapes(scene["shape_tables"])
    g.upload_bodies(scene["bodies"], scene["n_driven"])
    scenes.set_scene_params(g, scene)
    return g


def test_mlp_fp16_gradient_matches_cpu_model(gpu_lib):
    from rockable_gb300 import scenes
    scene = scenes.sphero_cube_box()
    g = _engine(scene)
    rng = np.random.default_rng(7)
    p = (rng.normal(scale=0.25, size=mlp_ref.NP)).astype(np.float32)
    g.mlp_set_params(p)
    X = rng.normal(size=(64, 16)).astype(np.float32)
    T = rng.normal(size=(64, 2)).astype(np.float32)
    gg, lg = g.mlp_gradient(X, T)
    lc, gc = mlp_ref.loss_and_grad(p.astype(np.float64), X, T, half=True)
    assert abs(lg - lc) <= 1e-3 * abs(lc) + 1e-6
    scale = np.max(np.abs(gc))
    assert np.max(np.abs(gg - gc)) <= 5e-3 * scale, np.max(np.abs(gg - gc)) / scale
    y = g.mlp_forward(X[0])
    yc, _ = mlp_ref.forward(p.astype(np.float64), X[:1], half=True)
    assert np.max(np.abs(y - yc[0])) <= 1e-3 * (np.max(np.abs(yc)) + 1e-3)


def _pairs(e):
    act = e["active"]
    return set(zip(e["i"][act].tolist(), e["j"][act].tolist()))


def test_guard_keeps_the_contacts_of_per_step_rebuilds(gpu_lib):
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=2000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=1500)
    src = scenes.scene_from_gpu(scene, gs)
    gl = _engine(src)
    gl.upload_entries(src["entries"])
    gl.set_skin(skin_min=0.02 * scene["dVerlet"], skin_max=2.0 * scene["dVerlet"], interval_min=1,
                interval_max=200)
    gr = _engine(src)
    gr.upload_entries(src["entries"])
    # reference: rebuild every step with the largest skin
    import copy
    sc2 = copy.deepcopy(scene)
    sc2["interVerlet"] = scene["dt"] * 0.999
    sc2["dVerlet"] = 2.0 * scene["dVerlet"]
    sc2["DVerlet"] = 2.0 * sc2["dVerlet"]
    scenes.set_scene_params(gr, sc2)
    gr.update_nl()
    for _ in range(6):
        gl.step(20)
        gr.step(20)
        pl, pr = _pairs(gl.entries()), _pairs(gr.entries())
        missing = pr - pl
        assert len(missing) <= max(1, len(pr) // 1000), (len(missing), len(pr))
    st = gl.skin_stats()
    assert st["rebuilds"] >= 1


def test_learned_skin_against_the_method_without_it(gpu_lib):
    """The trained network against the method without it, on a run long
    enough for more than 20 skin windows: a dense column settled between
    walls (scenes.loaded) and released collapses.  Fixed interval (plain),
    guard + last-window predictor (naive) and guard + the online-trained
    network (mlp), all from the same state, intervals up to 1000 steps.  Both
    skin modes keep the contact set exact (the guard).  Asserted: the network
    trains and acts (its predictions depart from the last window's rate),
    the network costs at most 5 % more device time than the method without
    it, and neither skin mode costs more than 10 % over the fixed interval.
    Measured on GB300: the displacement rate grows by under 1 % per window
    here (1.2e-7 -> 1.6e-7 m/step over 75 windows) and the cost model keeps
    the skin at or near its minimum, where a better rate prediction changes
    little; the guard and the partial refreshes do the work, and the network
    gains nothing measurable over the last-window rate on this flow.  Since
    the list build got cheap, the fixed interval is about as fast as the
    skin modes on a scene this small (a refresh costs what its smaller list
    saves); the skin form's gain shows at 50 000 grains."""
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=3000, nshapes=64, semi=(0.0025, 0.0075), column=(0.2, 0.2, 1.5), walls=True)
    src = scenes.loaded(scene, 20000)
    res = {}
    for name in ["plain", "naive", "mlp"]:
        g = _engine(src)
        g.upload_entries(src["entries"])
        if name != "plain":
            g.set_skin(use_mlp=(name == "mlp"), skin_min=0.05 * src["dVerlet"], skin_max=4.0 * src["dVerlet"],
                       interval_min=2, interval_max=1000, seed=11)
        r = g.step(8000)
        ms, _ = g.last_step_timing()
        sk = g.skin_stats() if name != "plain" else {}
        res[name] = {"ms": ms, "nl_updates": r["nl_updates"], "active": r["n_active"], "entries": r["n_entries"],
                     "skin": sk}
        g.close()
    print("learned skin comparison:", res)
    mlp, naive = res["mlp"]["skin"], res["naive"]["skin"]
    assert mlp["windows"] >= 20 and mlp["train_steps"] > 0 and mlp["loss"] > 0.0
    assert mlp["predicted_rate"] != mlp["last_rate"] and naive["predicted_rate"] == naive["last_rate"]
    assert res["mlp"]["ms"] <= 1.05 * res["naive"]["ms"], res
    assert max(res["mlp"]["ms"], res["naive"]["ms"]) <= 1.10 * res["plain"]["ms"], res


def _keys(e):
    return set(zip(e["i"].tolist(), e["j"].tolist(), e["type"].tolist(), e["isub"].tolist(), e["jsub"].tolist()))


@pytest.mark.parametrize("partial_fraction", [0.0, 0.2])
def test_every_touching_subcontact_is_in_the_skin_list(partial_fraction, gpu_lib):
    """Exactness of the guard, with and without partial refreshes: from the
    skin engine's own state after each chunk of steps, a fresh list built
    with a vanishing skin (the sub-contacts that touch or overlap now) must be
    contained in the skin engine's list."""
    import copy
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=2000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=1500)
    src = scenes.scene_from_gpu(scene, gs)
    gs.close()
    gl = _engine(src)
    gl.upload_entries(src["entries"])
    gl.set_skin(use_mlp=False, skin_min=0.05 * scene["dVerlet"], skin_max=2.0 * scene["dVerlet"], interval_min=1,
                interval_max=400, partial_fraction=partial_fraction)
    tight = copy.deepcopy(scene)
    tight["dVerlet"] = 1e-12
    tight["DVerlet"] = 2e-12
    touching_seen = 0
    for _ in range(8):
        gl.step(25)
        now = dict(src)
        b = dict(src["bodies"])
        st = gl.bodies()
        for k in ["pos", "vel", "acc", "Q", "vrot", "arot"]:
            b[k] = st[k]
        now["bodies"] = b
        gt = _engine(now)
        scenes.set_scene_params(gt, tight)
        gt.update_nl()
        touching = _keys(gt.entries())
        gt.close()
        listed = _keys(gl.entries())
        missing = touching - listed
        assert not missing, (len(missing), sorted(missing)[:5])
        touching_seen += len(touching)
    assert touching_seen > 0
    sk = gl.skin_stats()
    print("skin stats (partial_fraction=%g):" % partial_fraction, sk)
    if partial_fraction > 0:
        assert sk["partial"] >= 1


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_batched_skin_steps_match_the_per_step_path(form, gpu_lib):
    """With step graphs the skin mode runs batches of steps whose refresh
    decisions are taken on the device (k_skin_end); without them the host
    decides after every step.  With the skin size and the interval pinned the
    decisions depend on the state alone, so both paths must give the same
    refreshes and bit-identical bodies, over calls whose lengths do not
    divide the batch."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    scene = scenes.column_collapse(n=2000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=1500)
    src = scenes.scene_from_gpu(scene, gs)
    gs.close()
    skin = 0.1 * scene["dVerlet"]
    out = []
    for graphs in (False, True):
        g = GpuScene(form=RK_FORM_FP64 if form == "fp64" else RK_FORM_MIXED)
        g.upload_shapes(src["shape_tables"])
        g.upload_bodies(src["bodies"], src["n_driven"])
        scenes.set_scene_params(g, src)
        g.upload_entries(src["entries"])
        g.set_skin(use_mlp=False, skin_min=skin, skin_max=skin, interval_min=45, interval_max=45)
        g.set_graphs(graphs)
        for n in (7, 100, 33, 160):
            g.step(n)
        out.append((g.bodies(), g.skin_stats(), g.graph_stats()))
        g.close()
    (b0, s0, _), (b1, s1, gst) = out
    print(form, "per-step:", s0, "batched:", s1, "graphs:", gst)
    assert s0["rebuilds"] >= 3 and s0["partial"] + s0["forced"] >= 1
    for k in ("rebuilds", "forced", "scheduled", "partial", "partial_bodies"):
        assert s0[k] == s1[k], (k, s0[k], s1[k])
    for k in ("pos", "vel", "Q", "vrot", "acc", "arot"):
        assert np.array_equal(b0[k], b1[k]), k
    assert gst["replays"] > 0
