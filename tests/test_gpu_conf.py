"""Device-formatted conf sections (rk_format_conf, the role of
Rockable::saveConf's Particles and Interactions, Rockable.cpp:547-580)
against the same text made on the host from the downloaded state (GPU).
The reference's own goldens pass through it too: the C++ host writes its
conf files with it (test_gpu_host.py)."""
import numpy as np
import pytest

from test_fmt_cpu import toward_zero

pytestmark = pytest.mark.gpu


def printf_e(x, prec, tz=False):
    """printf("%.*e"): Python's correctly rounded formatting (ties to even),
    or the exact value truncated for the normals (test_fmt_cpu.py checks
    both against the formatter)."""
    return toward_zero(x, prec) if tz else "%.*e" % (prec, x)


@pytest.mark.parametrize("prec", [16, 13])
def test_device_conf_text_equals_printf(prec, gpu_lib):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene
    scene = scenes.column_collapse(n=1500, nshapes=64, semi=(0.0025, 0.0075), column=(0.15, 0.15, 1.5))
    g = GpuScene()
    g.upload_shapes(scene["shape_tables"])
    g.upload_bodies(scene["bodies"], scene["n_driven"])
    scenes.set_scene_params(g, scene)
    g.set_shape_names([s["name"] for s in scene["shapes"]])
    g.update_nl()
    g.step(300)
    g.set_record_geometry(True)
    g.step(1)
    part, inter, na = g.format_conf(prec)
    b = g.bodies()
    st = scene["bodies"]
    want = []
    for k in range(len(b["pos"])):
        vals = [b["pos"][k], b["vel"][k], b["acc"][k], b["Q"][k], b["vrot"][k], b["arot"][k]]
        nums = [printf_e(st["homothety"][k], prec)] + [printf_e(v, prec) for a in vals for v in a]
        want.append(" ".join([scene["shapes"][st["shape"][k]]["name"], str(st["group"][k]), str(st["cluster"][k])] +
                             nums))
    assert part == "\n".join(want) + "\n"
    e = g.entries(geometry=True)
    act = np.nonzero((e["dn"] < 0.0) | (e["bond"] >= 0))[0]
    assert na == len(act) > 100
    lines = []
    for k in act:
        f = [printf_e(v, prec, True) for v in e["n"][k]] + [printf_e(e["dn"][k], prec)]
        f += [printf_e(v, prec) for v in list(e["pos"][k]) + list(e["vel"][k])] + [printf_e(e["fn"][k], prec)]
        f += [printf_e(v, prec) for v in list(e["ft"][k]) + list(e["mom"][k])] + [printf_e(e["damp"][k], prec)]
        lines.append(" ".join([str(e["i"][k]), str(e["j"][k]), str(e["type"][k]), str(e["isub"][k]),
                               str(e["jsub"][k])] + f))
    assert inter == "\n".join(lines) + "\n"
    g.close()
