"""Scenes whose oracle results are frozen in tests/golden/oracle/: the paths
that no reference golden pins (Avalanche law, StickedLinks bonds and their
rupture, the linkCells neighbour list, the dynamic NL guard).  Each is a
variant of the reference's 518-polyhedra test input (the substitutions below
applied to its conf), advanced by a fixed number of steps.

tests/golden/make_oracle_goldens.py runs the oracle on them and writes the
exact state (bodies, neighbour-list keys and history, bonds left, list
updates) as .npz files; test_oracle_frozen.py checks that the oracle still
reproduces them and test_gpu_frozen.py that the FP64 GPU form does, bit for
bit."""
import os
import re

import numpy as np

BODY_FIELDS = ["pos", "vel", "acc", "Q", "vrot", "arot", "force", "moment"]
ENTRY_FIELDS = ["dn", "fn", "ft", "mom", "damp"]
BOND_PARAMS = ("knInnerBond 0 0 100\nktInnerBond 0 0 80\nkrInnerBond 0 0 1e-4\nen2InnerBond 0 0 0.1\n"
               "fn0InnerBond 0 0 0.05\nft0InnerBond 0 0 0.05\nmom0InnerBond 0 0 1.0\npowInnerBond 0 0 2\n")

CASES = {
    "avalanche_518": {
        "subs": [(r"^forceLaw Default", "forceLaw Avalanche"), (r"^muContact 0 0 0$", "muContact 0 0 0.3"),
                 (r"^krContact 0 0 0$", "krContact 0 0 1e-3"), (r"^murContact 0 0 0$", "murContact 0 0 0.1"),
                 (r"^dt .*$", "dt 1e-07")],
        "steps": [150]},
    "sticked_rupture_518": {
        "subs": [(r"^forceLaw Default", "forceLaw StickedLinks"), (r"^muContact 0 0 0$", "muContact 0 0 0.3"),
                 (r"^gravity 0 0 0$", "gravity 0 0 -500"), (r"^dt .*$", "dt 2e-07")],
        "append": BOND_PARAMS, "tail": "stickVerticesInClusters 0.001\n",
        # bond strengths lowered after the load, so that bonds break
        "after_load": [("fn0InnerBond", 2e-5), ("ft0InnerBond", 1e-6)],
        "steps": [50, 50, 50, 50]},
    "linkcells_518": {
        "subs": [(r"^UpdateNL bruteForce$", "UpdateNL linkCells"), (r"^dt .*$", "dt 2e-07"),
                 (r"^gravity 0 0 0$", "gravity 0 0 -9.81"), (r"^muContact 0 0 0$", "muContact 0 0 0.4")],
        "steps": [100, 100, 100]},
    "dynamic_guard_518": {
        "subs": [(r"^dynamicUpdateNL 0$", "dynamicUpdateNL 1\ndispUpdateNL 3e-6\nangleUpdateNL 0.5"),
                 (r"^interVerlet .*$", "interVerlet 1"), (r"^dt .*$", "dt 2e-07"),
                 (r"^gravity 0 0 0$", "gravity 0 0 -9.81")],
        "steps": [200]},
}
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle")


def make_conf(name, src_conf, dst):
    """The case's conf, from the extracted 518_poly input conf."""
    c = CASES[name]
    text = open(src_conf).read()
    for a, b in c["subs"]:
        text, n = re.subn(a, b, text, flags=re.M)
        assert n > 0, a
    if c.get("append"):
        k = text.index("Particles")
        text = text[:k] + c["append"] + text[k:]
    text += c.get("tail", "")
    with open(dst, "w") as f:
        f.write(text)
    return dst


def _digest(a):
    import hashlib
    a = np.ascontiguousarray(a)
    return np.frombuffer(hashlib.sha256(a.tobytes() + str(a.dtype).encode() + str(a.shape).encode()).digest(), np.uint8)


def state(bodies, entries, n_interfaces, nl_updates):
    """The frozen quantities of a run, as SHA-256 digests of the bit
    patterns (any difference shows): every body field, the entry keys, every
    entry field over all entries; in full: the positions (to locate a
    difference), the number of entries, the bonds left (unbroken interfaces)
    and the list updates."""
    out = {"pos": np.asarray(bodies["pos"], np.float64)}
    for k in BODY_FIELDS:
        out["digest_" + k] = _digest(np.asarray(bodies[k], np.float64))
    keys = np.stack([np.asarray(entries[k], np.int64) for k in ["i", "j", "type", "isub", "jsub"]], 1)
    out["digest_keys"] = _digest(keys)
    out["digest_bond"] = _digest(np.asarray(entries["bond"], np.int64))
    for k in ENTRY_FIELDS:
        out["digest_e_" + k] = _digest(np.asarray(entries[k], np.float64))
    out["n_entries"] = np.array([len(keys)], np.int64)
    out["n_interfaces"] = np.array([n_interfaces], np.int64)
    out["nl_updates"] = np.array([nl_updates], np.int64)
    return out


def run_oracle(oracle_mod, conf, name):
    """The case on the oracle: load, initial list update, the steps; returns
    the oracle and its frozen state."""
    c = CASES[name]
    o = oracle_mod.Oracle(conf)
    for p, v in c.get("after_load", []):
        o.set_param(p, 0, 0, v)
    o.update_nl()
    n = 0
    for k in c["steps"]:
        n += o.run(k)
    return o, state(o.bodies(), o.entries(), len(o.interfaces()), n)


def diff(a, b):
    """Names of the frozen quantities that differ (bit patterns for floats)."""
    bad = []
    for k in a:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        if x.shape != y.shape:
            bad.append(k + " (shape)")
        elif x.dtype.kind == "f":
            if not np.array_equal(x.view(np.uint64), y.astype(np.float64).view(np.uint64)):
                bad.append(k)
        elif not np.array_equal(x, y):
            bad.append(k)
    return bad
