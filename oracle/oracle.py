"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, the smoke check and the CPU-baseline leg of bench.py import
this module: it is the checker of the CUDA path, never the thing measured.
`build()` compiles oracle/_build/librk_oracle.so with the Makefile next to it.
"""
import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.environ.get("RK_ORACLE_LIB", os.path.join(HERE, "_build", platform.machine(), "librk_oracle.so"))
_lib = None

RK_NPARAM = 22


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, I, D, L64 = C.c_void_p, C.c_int, C.c_double, C.c_long
        sig = {
            "orc_load": (P, [C.c_char_p]), "orc_last_error": (C.c_char_p, []), "orc_free": (None, [P]),
            "orc_read_driving": (I, [P, C.c_char_p]), "orc_update_nl": (None, [P]), "orc_run": (I, [P, I]),
            "orc_integrate": (L64, [P, C.c_char_p, L64]), "orc_save_conf": (I, [P, C.c_char_p]),
            "orc_nbodies": (I, [P]), "orc_ndriven": (I, [P]), "orc_get_bodies": (None, [P, P]),
            "orc_set_bodies": (None, [P, P]), "orc_nentries": (L64, [P]), "orc_get_entries": (None, [P, P, P]),
            "orc_nactive": (L64, [P]), "orc_ninterfaces": (L64, [P]), "orc_get_interfaces": (None, [P, P]),
            "orc_get_scalars": (None, [P, P]), "orc_get_stats": (None, [P, P]), "orc_law_id": (I, [P]),
            "orc_option": (C.c_char_p, [P, C.c_char_p]), "orc_nshapes": (I, [P]),
            "orc_get_shape_sizes": (None, [P, P]), "orc_get_shapes": (None, [P] + [P] * 9),
            "orc_get_body_static": (None, [P] * 7), "orc_ngroup": (I, [P]), "orc_get_table": (None, [P, P]),
            "orc_ncontrols": (I, [P]), "orc_get_controls": (None, [P] * 7), "orc_get_flow": (None, [P, P]),
            "orc_set_variant": (None, [P]), "orc_set_param": (I, [P, C.c_char_p, I, I, D]),
            "orc_get_body_force": (I, [P, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One scene simulated by the CPU restatement."""

    def __init__(self, conf_path, driving=None):
        self.h = lib().orc_load(conf_path.encode())
        if not self.h:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        if driving:
            if lib().orc_read_driving(self.h, driving.encode()) != 0:
                raise RuntimeError("oracle: " + lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    # -- running
    def update_nl(self):
        lib().orc_update_nl(self.h)

    def run(self, n):
        return lib().orc_run(self.h, int(n))

    def integrate(self, outdir, max_steps=0):
        return lib().orc_integrate(self.h, outdir.encode(), int(max_steps))

    def save_conf(self, path):
        return lib().orc_save_conf(self.h, path.encode())

    def set_param(self, name, g1, g2, value):
        if lib().orc_set_param(self.h, name.encode(), g1, g2, float(value)) != 0:
            raise KeyError(name)

    # -- state
    @property
    def n(self):
        return lib().orc_nbodies(self.h)

    @property
    def n_driven(self):
        return lib().orc_ndriven(self.h)

    def bodies(self):
        a = np.zeros((self.n, 29))
        lib().orc_get_bodies(self.h, _p(a))
        return {"pos": a[:, 0:3], "vel": a[:, 3:6], "acc": a[:, 6:9], "Q": a[:, 9:13], "vrot": a[:, 13:16],
                "arot": a[:, 16:19], "force": a[:, 19:22], "moment": a[:, 22:25], "homothety": a[:, 25],
                "mass": a[:, 26]}

    def entries(self):
        n = lib().orc_nentries(self.h)
        k = np.zeros((n, 5), dtype=np.int64)
        s = np.zeros((n, 21))
        if n:
            lib().orc_get_entries(self.h, _p(k), _p(s))
        return {"i": k[:, 0], "j": k[:, 1], "type": k[:, 2], "isub": k[:, 3], "jsub": k[:, 4],
                "n": s[:, 0:3], "dn": s[:, 3], "prev_dn": s[:, 4], "pos": s[:, 5:8], "vel": s[:, 8:11],
                "fn": s[:, 11], "ft": s[:, 12:15], "mom": s[:, 15:18], "damp": s[:, 18],
                "bond": s[:, 19].astype(np.int64), "active": s[:, 20].astype(bool)}

    def interfaces(self):
        n = lib().orc_ninterfaces(self.h)
        a = np.zeros((n, 12))
        if n:
            lib().orc_get_interfaces(self.h, _p(a))
        return a

    def scalars(self):
        a = np.zeros(15)
        lib().orc_get_scalars(self.h, _p(a))
        keys = ["t", "dt", "tmax", "interVerlet", "interConf", "DVerlet", "dVerlet", "iconf", "nDriven",
                "numDamp", "totalBrokenArea", "nbroken", "gx", "gy", "gz"]
        return dict(zip(keys, a))

    def flow(self):
        a = np.zeros(6)
        lib().orc_get_flow(self.h, _p(a))
        return dict(zip(["interVerletC", "dynamicUpdateNL", "dispUpdateNL", "angleUpdateNL",
                         "paramsInInterfaces", "needUpdate"], a))

    def stats(self):
        a = np.zeros(5)
        lib().orc_get_stats(self.h, _p(a))
        return dict(zip(["e_trans", "e_rot", "n_active", "coordination", "n_broken"], a))

    def body_force(self):
        """(kind, conf parameters, V h^3 per body) of the BodyForce plugin."""
        p = np.zeros(8)
        v = np.zeros(self.n)
        k = lib().orc_get_body_force(self.h, _p(p), _p(v))
        return k, p[:[0, 4, 7, 1][k]], v

    @property
    def law(self):
        return lib().orc_law_id(self.h)

    def shapes(self):
        z = np.zeros(5, dtype=np.int64)
        lib().orc_get_shape_sizes(self.h, _p(z))
        ns, nv, ne, nf, nfv = [int(x) for x in z]
        out = {"vert_ofs": np.zeros(ns + 1, np.int32), "vertices": np.zeros(3 * nv),
               "edge_ofs": np.zeros(ns + 1, np.int32), "edges": np.zeros(2 * max(ne, 1), np.int32),
               "face_ofs": np.zeros(ns + 1, np.int32), "face_vofs": np.zeros(nf + 1, np.int32),
               "face_verts": np.zeros(max(nfv, 1), np.int32), "radius": np.zeros(ns), "obb": np.zeros(15 * ns)}
        lib().orc_get_shapes(self.h, *[_p(out[k]) for k in ["vert_ofs", "vertices", "edge_ofs", "edges", "face_ofs",
                                                            "face_vofs", "face_verts", "radius", "obb"]])
        return out

    def body_static(self):
        n = self.n
        out = {"shape": np.zeros(n, np.int32), "group": np.zeros(n, np.int32), "cluster": np.zeros(n, np.int32),
               "homothety": np.zeros(n), "mass": np.zeros(n), "inertia": np.zeros((n, 3))}
        lib().orc_get_body_static(self.h, *[_p(out[k]) for k in ["shape", "group", "cluster", "homothety", "mass",
                                                                 "inertia"]])
        return out

    def table(self):
        g = lib().orc_ngroup(self.h)
        t = np.zeros(RK_NPARAM * g * g)
        lib().orc_get_table(self.h, _p(t))
        return g, t

    def controls(self):
        n = lib().orc_ncontrols(self.h)
        t = np.zeros(max(n, 1), np.int32)
        b = np.zeros(max(n, 1), np.int32)
        v = np.zeros(max(n, 1))
        vec = np.zeros(3 * max(n, 1))
        servo = np.zeros(8, np.int32)
        pr = np.zeros(1)
        lib().orc_get_controls(self.h, _p(t), _p(b), _p(v), _p(vec), _p(servo), _p(pr))
        return {"n": n, "type": t[:n], "body": b[:n], "value": v[:n], "vec": vec[:3 * n].reshape(-1, 3),
                "servo": servo, "pressure": float(pr[0])}
