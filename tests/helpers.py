"""Test helpers: hand the oracle's state to the GPU engine through the C ABI."""
import numpy as np

from rockable_gb300.abi import GpuScene, RK_FORM_FP64


def gpu_from_oracle(o, device=0, form=RK_FORM_FP64):
    g = GpuScene(device=device, form=form)
    g.upload_shapes(o.shapes())
    st = o.body_static()
    b = o.bodies()
    g.upload_bodies({"pos": b["pos"], "vel": b["vel"], "acc": b["acc"], "Q": b["Q"], "vrot": b["vrot"],
                     "arot": b["arot"], "homothety": st["homothety"], "mass": st["mass"],
                     "inertia": st["inertia"], "shape": st["shape"], "group": st["group"],
                     "cluster": st["cluster"]}, o.n_driven)
    set_params_from_oracle(g, o)
    f = o.interfaces()
    if len(f):
        params = np.concatenate([f[:, 4:11], np.zeros((len(f), 1))], axis=1)
        g.upload_interfaces(f[:, 0], f[:, 1], f[:, 3], params, f[:, 11])
    e = o.entries()
    g.upload_entries(e)
    c = o.controls()
    if c["n"] or c["servo"][0]:
        servo = {"kind": c["servo"][0], "icontr": c["servo"][1], "walls": c["servo"][2:8],
                 "pressure": c["pressure"]}
        g.set_controls(c["type"], c["body"], c["value"], c["vec"], servo)
    kind, prm, vol = o.body_force()
    if kind:
        g.set_body_force(kind, prm, vol)
    return g


def set_params_from_oracle(g, o):
    """Law table, time step and flow scalars of the oracle's scene."""
    sc = o.scalars()
    fl = o.flow()
    G, tab = o.table()
    g.set_params(t=sc["t"], dt=sc["dt"], gravity=(sc["gx"], sc["gy"], sc["gz"]), DVerlet=sc["DVerlet"],
                 dVerlet=sc["dVerlet"], interVerlet=sc["interVerlet"], interVerletC=fl["interVerletC"],
                 law=o.law, ngroup=G, table=tab, numerical_damping=sc["numDamp"],
                 params_in_interfaces=int(fl["paramsInInterfaces"]), dynamic_update_nl=int(fl["dynamicUpdateNL"]),
                 disp_update_nl=fl["dispUpdateNL"], angle_update_nl=fl["angleUpdateNL"])


BODY_FIELDS = ["pos", "vel", "acc", "Q", "vrot", "arot", "force", "moment"]


def compare_bodies(ob, gb, fields=BODY_FIELDS):
    """Max |difference| per field (0.0 means bit-identical values)."""
    return {k: float(np.max(np.abs(ob[k] - gb[k]))) if len(ob[k]) else 0.0 for k in fields}


def bitwise_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def key_tuples(e):
    return list(zip(e["i"].tolist(), e["j"].tolist(), e["type"].tolist(), e["isub"].tolist(), e["jsub"].tolist()))
