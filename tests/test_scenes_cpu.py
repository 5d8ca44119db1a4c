"""Scene generators (CPU): the column with removable walls and body removal
keep the seeded grains and remap the neighbour-list entries in key order."""
import numpy as np


def test_walls_do_not_change_the_grains():
    from rockable_gb300 import scenes
    a = scenes.column_collapse(n=500, nshapes=16)
    b = scenes.column_collapse(n=500, nshapes=16, walls=True)
    assert b["n_driven"] == 5 and b["walls"] == [1, 2, 3, 4]
    for k in ["pos", "Q", "shape", "mass"]:
        assert np.array_equal(a["bodies"][k][1:], b["bodies"][k][5:]), k
    # walls flush with the column: every grain (rotated vertices plus the
    # rounding radius) inside it
    lo, hi = _extents(b)
    assert np.all(lo[5:, :2] >= -0.25 - 1e-12) and np.all(hi[5:, :2] <= 0.25 + 1e-12)
    assert np.all(lo[5:, 2] >= 0.005 - 1e-12)  # on or above the floor plate's top face


def _extents(sc):
    """World-frame bounds (vertices plus rounding radius) of every body."""
    b = sc["bodies"]
    lo = np.zeros((len(b["mass"]), 3))
    hi = np.zeros_like(lo)
    for k, (s, q, x, h) in enumerate(zip(b["shape"], b["Q"], b["pos"], b["homothety"])):
        w, a, c, d = q
        R = np.array([[1 - 2 * (c * c + d * d), 2 * (a * c - w * d), 2 * (a * d + w * c)],
                      [2 * (a * c + w * d), 1 - 2 * (a * a + d * d), 2 * (c * d - w * a)],
                      [2 * (a * d - w * c), 2 * (c * d + w * a), 1 - 2 * (a * a + c * c)]])
        v = h * np.asarray(sc["shapes"][s]["vertices"]) @ R.T + x
        r = h * sc["shapes"][s]["radius"]
        lo[k], hi[k] = v.min(0) - r, v.max(0) + r
    return lo, hi


def test_packing_is_dense_at_rest_without_overlap_and_seeded():
    """The column's loose random packing (host/rk_pack.cpp): every grain at
    rest, several touching neighbours per grain, no overlap anywhere -- checked
    independently by the oracle's neighbour list after one step (every
    sub-contact's dn at or above minus the packer's tolerance) -- and the same
    positions from a second, uncached run."""
    import tempfile
    from oracle import oracle
    from rockable_gb300 import scenes
    sc = scenes.column_collapse(n=1500, nshapes=64, column=(0.2, 0.2, 1.5))
    st = sc["pack"]
    assert st["at_rest"] == 1500 and st["max_overlap"] <= 0.0
    # lowest of 16 drop sites per grain: a dense pile where grains touch
    assert st["coordination"] >= 4.5 and st["coordination"] == 2 * st["touching_pairs"] / 1500
    assert st["solid_fraction_bulk"] >= 0.48
    oracle.build()
    o = oracle.Oracle(scenes.write_conf(sc, tempfile.mkdtemp(prefix="rk_pack_")))
    o.update_nl()
    o.run(1)
    e = o.entries()
    assert len(e["dn"]) > 10 * 1500 and e["dn"].min() >= -2e-9
    b = sc["bodies"]
    pos, st2 = scenes.pack(sc["shapes"], b["shape"][1:], b["Q"][1:], b["mass"][1:] / 2700.0, (-0.1, -0.1, 0.005),
                           (0.1, 0.1, 1.5), tries=16, cache=False)
    assert np.array_equal(pos, b["pos"][1:])
    assert all(st2[k] == st[k] for k in ["touching_pairs", "on_floor", "moves", "at_rest"])


def test_drop_bodies_remaps_entries_in_key_order():
    from rockable_gb300 import scenes
    sc = scenes.column_collapse(n=50, nshapes=4, walls=True)
    # entries between every body pair (i < j) in key order, a few touching the walls
    i, j = np.triu_indices(len(sc["bodies"]["mass"]), 1)
    e = {"i": i.astype(np.int32), "j": j.astype(np.int32), "type": np.zeros(len(i), np.int32),
         "isub": np.zeros(len(i), np.int32), "jsub": np.zeros(len(i), np.int32), "fn": np.arange(len(i), dtype=float),
         "ft": np.zeros((len(i), 3))}
    sc["entries"] = e
    d = scenes.drop_bodies(sc, sc["walls"])
    assert d["n_driven"] == 1 and len(d["bodies"]["mass"]) == 51
    de = d["entries"]
    keep = ~np.isin(e["i"], [1, 2, 3, 4]) & ~np.isin(e["j"], [1, 2, 3, 4])
    assert len(de["i"]) == keep.sum()
    assert np.array_equal(de["fn"], e["fn"][keep])
    key = de["i"].astype(np.int64) * 1000 + de["j"]
    assert np.all(np.diff(key) > 0)
    old = {0: 0, **{k: k - 4 for k in range(5, 55)}}
    assert np.array_equal(de["i"], [old[x] for x in e["i"][keep]])
    assert np.array_equal(d["bodies"]["pos"][1:], sc["bodies"]["pos"][5:])


def test_sphero_cube_box_runs_on_the_oracle():
    """Workload config 0 (512 sphero-cubes on a lattice in a box of 6 plates,
    Default law, brute-force neighbour list, 20k steps of 1e-6 s) written as
    a Rockable conf and run by the oracle: the top layer falls freely by
    g t^2 / 2, nothing leaves the box or sinks through the floor by more than
    a contact overlap, and contacts form."""
    import tempfile
    from oracle import oracle
    from rockable_gb300 import scenes
    oracle.build()
    sc = scenes.sphero_cube_box()
    o = oracle.Oracle(scenes.write_conf(sc, tempfile.mkdtemp(prefix="rk_cubes_")))
    assert o.n == 518 and o.n_driven == 6 and o.law == 0
    o.update_nl()
    p0 = o.bodies()["pos"][6:].copy()
    steps = 20000
    o.run(steps)
    p = o.bodies()["pos"][6:]
    assert np.all(np.isfinite(p))
    t = steps * sc["dt"]
    fall = 0.5 * 9.81 * t * t
    top = np.argmax(p0[:, 2])
    assert abs((p0[top, 2] - p[top, 2]) - fall) <= 0.05 * fall
    L = float(np.max(sc["bodies"]["pos"][:6, 0]))  # the box's side (wall plates at 0 and L)
    assert np.all(p[:, :2] > 0.0) and np.all(p[:, :2] < L)
    # a cube resting on a face has its centre half a side plus the rounding (0.5 mm) above the
    # floor; the contact overlap under its weight is far below a micrometre
    assert p[:, 2].min() >= 0.5e-3 - 1e-6
    assert o.stats()["n_active"] > 0
