"""FP64 GPU step against the oracle, bit for bit (GPU).

Every test loads a scene with the oracle, hands the same state to the CUDA
engine through the C ABI, advances both and requires identical IEEE bit
patterns for every body field and every neighbour-list entry."""
import os
import re

import numpy as np
import pytest

from conftest import CONF
from helpers import BODY_FIELDS, bitwise_equal, gpu_from_oracle, key_tuples

pytestmark = pytest.mark.gpu


def assert_bodies_equal(o, g, where=""):
    ob, gb = o.bodies(), g.bodies()
    bad = {k: float(np.max(np.abs(ob[k] - gb[k]))) for k in BODY_FIELDS if not bitwise_equal(ob[k], gb[k])}
    assert not bad, "%s body fields differ (max abs diff): %s" % (where, bad)


def assert_entries_equal(o, g, where=""):
    oe, ge = o.entries(), g.entries()
    ko, kg = key_tuples(oe), key_tuples(ge)
    if ko != kg:
        so, sg = set(ko), set(kg)
        raise AssertionError("%s entry keys differ: %d oracle, %d gpu, only-oracle %s, only-gpu %s" % (
            where, len(ko), len(kg), sorted(so - sg)[:5], sorted(sg - so)[:5]))
    for k in ["dn", "fn", "ft", "mom", "damp"]:
        assert bitwise_equal(oe[k], ge[k]), "%s entry field %s differs (max %g)" % (
            where, k, float(np.max(np.abs(oe[k] - ge[k]))))
    assert np.array_equal(oe["bond"], ge["bond"]), where + " bond indices differ"


def variant_conf(src, dst, subs=(), append=""):
    text = open(src).read()
    for a, b in subs:
        text, n = re.subn(a, b, text, flags=re.M)
        assert n > 0, a
    k = text.index("Particles")
    text = text[:k] + append + text[k:] if append else text
    open(dst, "w").write(text)
    return dst


@pytest.mark.parametrize("case", ["512_particles", "518_poly"])
def test_load_nl_and_10_steps_bitwise(case, golden_dir, oracle_lib, gpu_lib):
    o = oracle_lib.Oracle(str(golden_dir / case / CONF[case]))
    g = gpu_from_oracle(o)
    assert_entries_equal(o, g, "upload")
    o.update_nl()
    g.update_nl()
    assert_entries_equal(o, g, "initial NL update")
    o.run(10)
    g.step(10)
    assert_bodies_equal(o, g, "after 10 steps")
    assert_entries_equal(o, g, "after 10 steps")


def _fmt(v, prec):
    return "%.*e" % (prec, v)


@pytest.mark.parametrize("case,prec", [("512_particles", 16), ("518_poly", 13)])
def test_gpu_state_matches_reference_golden_text(case, prec, golden_dir, oracle_lib, gpu_lib):
    """The GPU state after 10 steps, printed like Rockable::saveConf, equals
    the reference's regression golden (Particles and Interactions)."""
    o = oracle_lib.Oracle(str(golden_dir / case / CONF[case]))
    g = gpu_from_oracle(o)
    g.update_nl()
    g.set_record_geometry(True)
    g.step(10)
    gold = open(str(golden_dir / case / "golden.conf")).read().split("\n")
    k = [i for i, l in enumerate(gold) if l.startswith("Particles")][0]
    n = int(gold[k].split()[1])
    b = g.bodies()
    for i in range(n):
        toks = gold[k + 2 + i].split()
        vals = np.concatenate([b["pos"][i], b["vel"][i], b["acc"][i], b["Q"][i], b["vrot"][i], b["arot"][i]])
        mine = [_fmt(v, prec) for v in vals]
        assert mine == toks[4:], "body %d differs from the golden" % i
    ki = k + 2 + n
    ni = int(gold[ki].split()[1])
    e = g.entries(geometry=True)
    act = np.nonzero(e["active"])[0]
    assert len(act) == ni
    import decimal
    for r, idx in enumerate(act):
        toks = gold[ki + 1 + r].split()
        key = [e["i"][idx], e["j"][idx], e["type"][idx], e["isub"][idx], e["jsub"][idx]]
        assert [int(t) for t in toks[:5]] == [int(x) for x in key]
        # the normal is printed rounded toward zero; compare it through decimal truncation
        for d in range(3):
            exact = decimal.Decimal(float(e["n"][idx][d]))
            g_val = decimal.Decimal(toks[5 + d])
            assert abs(exact - g_val) <= abs(exact) * decimal.Decimal("1e-%d" % prec) + decimal.Decimal("1e-300")
        rest = [e["dn"][idx], *e["pos"][idx], *e["vel"][idx], e["fn"][idx], *e["ft"][idx], *e["mom"][idx],
                e["damp"][idx]]
        assert [_fmt(v, prec) for v in rest] == toks[8:], "interaction %d differs from the golden" % r


def test_nl_rebuilds_over_300_steps_bitwise(golden_dir, oracle_lib, gpu_lib, tmp_path):
    """Three periodic NL rebuilds (interVerlet = 100 steps) with contacts
    appearing and disappearing: keys and carried history stay identical."""
    case = "518_poly"
    conf = variant_conf(str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_nl.conf"),
                        subs=[(r"^dt .*$", "dt 2e-07"), (r"^gravity 0 0 0$", "gravity 0 0 -9.81")])
    o = oracle_lib.Oracle(conf)
    g = gpu_from_oracle(o)
    o.update_nl()
    g.update_nl()
    for _ in range(3):
        n_o = o.run(100)
        r = g.step(100)
        assert r["nl_updates"] == n_o == 2
        assert_entries_equal(o, g, "rebuild")
    assert_bodies_equal(o, g, "after 300 steps")


def test_avalanche_law_bitwise(golden_dir, oracle_lib, gpu_lib):
    case = "518_poly"
    conf = variant_conf(str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_av.conf"),
                        subs=[(r"^forceLaw Default", "forceLaw Avalanche"), (r"^muContact 0 0 0$", "muContact 0 0 0.3"),
                              (r"^krContact 0 0 0$", "krContact 0 0 1e-3"), (r"^murContact 0 0 0$", "murContact 0 0 0.1"),
                              (r"^dt .*$", "dt 1e-07")])
    o = oracle_lib.Oracle(conf)
    assert o.law == 1
    g = gpu_from_oracle(o)
    o.update_nl()
    g.update_nl()
    o.run(150)
    g.step(150)
    assert_bodies_equal(o, g, "avalanche")
    assert_entries_equal(o, g, "avalanche")


def test_default_law_friction_rolling_damping_bitwise(golden_dir, oracle_lib, gpu_lib):
    case = "518_poly"
    conf = variant_conf(str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_def.conf"),
                        subs=[(r"^muContact 0 0 0$", "muContact 0 0 0.4"), (r"^muContact 0 1 0$", "muContact 0 1 0.2"),
                              (r"^krContact 0 0 0$", "krContact 0 0 1e-3"), (r"^murContact 0 0 0$", "murContact 0 0 0.05"),
                              (r"^numericalDampingCoeff 0$", "numericalDampingCoeff 0.2"),
                              (r"^gravity 0 0 0$", "gravity 0 0 -9.81"), (r"^dt .*$", "dt 2e-07")])
    o = oracle_lib.Oracle(conf)
    g = gpu_from_oracle(o)
    o.update_nl()
    g.update_nl()
    o.run(150)
    g.step(150)
    assert_bodies_equal(o, g, "default+friction")
    assert_entries_equal(o, g, "default+friction")


def test_servo_tritri_isostatic_bitwise(golden_dir, oracle_lib, gpu_lib):
    """512 spheres in the box with the tritriIsostaticCompression servo of the
    test's drivingSystem.txt acting on the walls."""
    case = "512_particles"
    d = golden_dir / case
    o = oracle_lib.Oracle(str(d / CONF[case]), driving=str(d / "drivingSystem.txt"))
    assert o.controls()["servo"][0] == 1
    g = gpu_from_oracle(o)
    o.update_nl()
    g.update_nl()
    o.run(50)
    g.step(50)
    assert_bodies_equal(o, g, "servo")
    assert_entries_equal(o, g, "servo")


def test_dynamic_guard_rebuilds_bitwise(golden_dir, oracle_lib, gpu_lib):
    case = "518_poly"
    conf = variant_conf(str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_dyn.conf"),
                        subs=[(r"^dynamicUpdateNL 0$", "dynamicUpdateNL 1\ndispUpdateNL 3e-6\nangleUpdateNL 0.5"),
                              (r"^interVerlet .*$", "interVerlet 1"), (r"^dt .*$", "dt 2e-07"),
                              (r"^gravity 0 0 0$", "gravity 0 0 -9.81")])
    o = oracle_lib.Oracle(conf)
    assert o.flow()["dynamicUpdateNL"] == 1
    g = gpu_from_oracle(o)
    o.update_nl()
    g.update_nl()
    n_o = o.run(200)
    r = g.step(200)
    assert n_o > 0
    assert r["nl_updates"] == n_o
    assert_bodies_equal(o, g, "guard")
    assert_entries_equal(o, g, "guard")


def test_sticked_links_bonds_and_rupture_bitwise(golden_dir, oracle_lib, gpu_lib):
    """Bonds created by stickVerticesInClusters, StickedLinks law; after the
    load the bond strengths are lowered in both engines so that bonds break
    during the GPU steps: rupture set, carried history and bodies identical."""
    from helpers import set_params_from_oracle
    case = "518_poly"
    conf = variant_conf(
        str(golden_dir / case / CONF[case]), str(golden_dir / case / "v_stick.conf"),
        subs=[(r"^forceLaw Default", "forceLaw StickedLinks"), (r"^muContact 0 0 0$", "muContact 0 0 0.3"),
              (r"^gravity 0 0 0$", "gravity 0 0 -500"), (r"^dt .*$", "dt 2e-07")],
        append="knInnerBond 0 0 100\nktInnerBond 0 0 80\nkrInnerBond 0 0 1e-4\nen2InnerBond 0 0 0.1\n"
               "fn0InnerBond 0 0 0.05\nft0InnerBond 0 0 0.05\nmom0InnerBond 0 0 1.0\npowInnerBond 0 0 2\n")
    open(conf, "a").write("stickVerticesInClusters 0.001\n")
    o = oracle_lib.Oracle(conf)
    assert o.law == 2
    n0 = len(o.interfaces())
    assert n0 >= 5
    g = gpu_from_oracle(o)
    assert_entries_equal(o, g, "bonds upload")
    o.update_nl()
    g.update_nl()
    assert_entries_equal(o, g, "bonds NL")
    for name, v in [("fn0InnerBond", 2e-5), ("ft0InnerBond", 1e-6)]:
        o.set_param(name, 0, 0, v)
    set_params_from_oracle(g, o)
    for _ in range(4):
        o.run(50)
        g.step(50)
        assert_entries_equal(o, g, "bonds run")
    _, _, broken = g.interfaces()
    assert int(broken.sum()) == len(broken) - len(o.interfaces())
    assert int(broken.sum()) > 0
    assert_bodies_equal(o, g, "bonds")


def test_stats_match_oracle(golden_dir, oracle_lib, gpu_lib):
    """rk_get_stats (Rockable::getKineticEnergy, Rockable.cpp:3958-3970; the
    coordination 2 A / N_free and the broken-bond count) against the oracle's
    after a bonded run with ruptures: the counts exactly (the context counts
    the interfaces broken since its creation, the oracle since its load,
    whose force evaluation already broke some), the kinetic energies to
    1e-12 (the device reduction adds in another order)."""
    import oracle_cases
    from helpers import set_params_from_oracle
    name = "sticked_rupture_518"
    conf = oracle_cases.make_conf(name, str(golden_dir / "518_poly" / CONF["518_poly"]),
                                  str(golden_dir / "518_poly" / "v_stats.conf"))
    o = oracle_lib.Oracle(conf)
    for p, v in oracle_cases.CASES[name]["after_load"]:
        o.set_param(p, 0, 0, v)
    g = gpu_from_oracle(o)
    set_params_from_oracle(g, o)
    broken_at_upload = int(o.stats()["n_broken"])
    o.update_nl()
    g.update_nl()
    o.run(200)
    g.step(200)
    so, sg = o.stats(), g.stats()
    assert int(so["n_active"]) == sg["n_active"]
    assert int(so["n_broken"]) - broken_at_upload == sg["n_broken"] and sg["n_broken"] > 0
    _, _, broken = g.interfaces()
    assert int(broken.sum()) == sg["n_broken"]
    assert so["coordination"] == pytest.approx(sg["coordination"], rel=1e-15)
    for k in ["e_trans", "e_rot"]:
        assert sg[k] == pytest.approx(so[k], rel=1e-12), k
