"""Step graphs and batched scenes (GPU): replaying a step as one CUDA graph,
and running several independent scenes in one context, give bit-identical
results to the launch-by-launch path and to each scene run alone."""
import numpy as np
import pytest

from helpers import bitwise_equal

pytestmark = pytest.mark.gpu


def _engine(scene, form=0, entries=None, graphs=False):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene
    g = GpuScene(form=form)
    g.upload_shapes(scene["shape_tables"])
    g.upload_bodies(scene["bodies"], scene["n_driven"])
    if scene.get("scene_of") is not None:
        g.set_scenes(scene["scene_of"])
    scenes.set_scene_params(g, scene)
    if entries is not None:
        g.upload_entries(entries)
    else:
        g.update_nl()
    g.set_graphs(graphs)
    return g


@pytest.mark.parametrize("form", [0, 1])
def test_graph_replay_is_bitwise_identical(form, gpu_lib):
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=3000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=800)
    src = scenes.scene_from_gpu(scene, gs)
    gs.close()
    a = _engine(src, form, src["entries"], graphs=False)
    b = _engine(src, form, src["entries"], graphs=True)
    a.step(250)
    b.step(250)
    st = b.graph_stats()
    assert st["replays"] == 250
    assert st["captures"] >= 3  # re-captured after each of the rebuilds
    ba, bb = a.bodies(), b.bodies()
    for k in ["pos", "vel", "acc", "Q", "vrot", "arot", "force", "moment"]:
        assert bitwise_equal(ba[k], bb[k]), k
    ea, eb = a.entries(), b.entries()
    for k in ["i", "j", "fn", "ft", "dn"]:
        assert bitwise_equal(ea[k], eb[k]), k


def test_batched_scenes_match_each_scene_alone(gpu_lib):
    from rockable_gb300 import scenes
    bt = scenes.slope_batch(nscenes=4, nmin=300, nmax=1500, nshapes=32)
    gs = scenes.settle(bt, steps=2000, relax_steps=600)
    bt = scenes.scene_from_gpu(bt, gs)
    gs.close()
    whole = _engine(bt, graphs=True)
    whole.step(260)
    wb = whole.bodies()
    st = whole.stats()
    assert st["n_active"] > 0
    total_entries = 0
    for k in range(4):
        part = scenes.part_of(bt, k)
        g = _engine(part)
        g.step(260)
        pb = g.bodies()
        idx = bt["index_of"][k]
        for key in ["pos", "vel", "Q", "vrot", "force", "moment"]:
            assert bitwise_equal(wb[key][idx], pb[key]), (k, key)
        total_entries += g.stats()["n_entries"]
        g.close()
    assert total_entries == st["n_entries"]


def test_batched_headline_form_matches_each_scene_alone(gpu_lib):
    """The headline form (mixed precision, learned skin with exact contact
    detection) over four batched slope scenes: every scene's bodies after
    100 steps agree with the same scene run alone in that form within 1e-5
    of each field's range.  The skin of the batch decides its rebuilds for
    all scenes at once, so a scene's list may be refreshed at other steps
    than alone: the contacts found are the same, but the mixed form sums a
    body's contact terms in FP32 in lanes set by the terms' positions in the
    list, so the two runs differ at FP32 rounding and drift apart slowly."""
    from rockable_gb300 import scenes
    bt = scenes.slope_batch(nscenes=4, nmin=300, nmax=1500, nshapes=32)
    gs = scenes.settle(bt, steps=2000, relax_steps=600)
    bt = scenes.scene_from_gpu(bt, gs)
    gs.close()

    def headline(sc):
        g = _engine(sc, 1, None, graphs=True)
        d = sc["dVerlet"]
        g.set_skin(use_mlp=True, skin_min=0.1 * d, skin_max=4.0 * d, interval_min=2, interval_max=300, seed=3,
                   exact_contacts=True)
        return g

    whole = headline(bt)
    whole.step(100)
    wb = whole.bodies()
    assert whole.stats()["n_active"] > 0
    for k in range(4):
        part = scenes.part_of(bt, k)
        g = headline(part)
        g.step(100)
        pb = g.bodies()
        idx = bt["index_of"][k]
        for key in ["pos", "vel", "Q", "vrot"]:
            rng = max(float(np.abs(pb[key]).max()), 1e-30)
            assert float(np.abs(wb[key][idx] - pb[key]).max()) <= 1e-5 * rng, (k, key)
        g.close()
    whole.close()


def test_autotuned_block_sizes_change_no_result(gpu_lib):
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=3000, nshapes=64, semi=(0.0025, 0.0075))
    gs = scenes.settle(scene, steps=800)
    src = scenes.scene_from_gpu(scene, gs)
    gs.close()
    for form in [0, 1]:
        a = _engine(src, form, src["entries"])
        b = _engine(src, form, src["entries"], graphs=True)
        b.autotune(2)
        a.step(230)
        b.step(230)
        tpb = b.block_sizes()
        assert all(v in (32, 64, 128, 256, 512) for v in tpb.values()), tpb
        ba, bb = a.bodies(), b.bodies()
        for k in ["pos", "vel", "Q", "vrot", "force", "moment"]:
            assert bitwise_equal(ba[k], bb[k]), (form, k)
        a.close()
        b.close()


def test_packed_kinematics_round_trip(gpu_lib):
    """rk_download/upload_kinematics_packed move exactly the six kinematic
    arrays, in the documented order."""
    from rockable_gb300 import scenes
    scene = scenes.column_collapse(n=700, nshapes=16, semi=(0.0025, 0.0075))
    g = _engine(scene)
    g.step(20)
    n = g.n
    buf = np.zeros(19 * n)
    g.download_kinematics_packed(buf)
    b = g.bodies()
    parts = np.split(buf, np.cumsum([3 * n, 3 * n, 3 * n, 4 * n, 3 * n]))
    for k, part in zip(["pos", "vel", "acc", "Q", "vrot", "arot"], parts):
        assert bitwise_equal(part, b[k].ravel()), k
    rng = np.random.default_rng(3)
    new = rng.normal(size=19 * n)
    g.upload_kinematics_packed(new)
    g.synchronize()
    b2 = g.bodies()
    parts = np.split(new, np.cumsum([3 * n, 3 * n, 3 * n, 4 * n, 3 * n]))
    for k, part in zip(["pos", "vel", "acc", "Q", "vrot", "arot"], parts):
        assert bitwise_equal(part, b2[k].ravel()), k
    g.close()
