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
    # walls flush with the column, outside every grain's bounding sphere
    bound = np.array([s["bound"] for s in b["shapes"]])
    g = b["bodies"]["pos"][5:]
    r = bound[b["bodies"]["shape"][5:]]
    assert np.all(np.abs(g[:, 0]) + r <= 0.25 + 1e-12) and np.all(np.abs(g[:, 1]) + r <= 0.25 + 1e-12)


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
