"""ctypes binding of the C ABI declared in include/rk_gpu.h (librk_gpu.so).

`GpuScene` owns one rk_ctx (one scene on one GPU) and converts numpy arrays to
the ABI's structs.  The library is the in-tree build under rockable_gb300/_lib;
there is no CPU fallback: if the library or a CUDA device is missing, the
calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_lib", "librk_gpu.so")

RK_OK = 0
RK_LAW = {"Default": 0, "Avalanche": 1, "StickedLinks": 2}
RK_FORM_FP64, RK_FORM_MIXED = 0, 1
RK_BF = {"none": 0, "AttractingPoint": 1, "PreferredDirection": 2, "ViscousFluid": 3}
RK_NPARAM = 22
ERRORS = {-1: "RK_ERR_ARG", -2: "RK_ERR_CUDA", -3: "RK_ERR_CAPACITY", -4: "RK_ERR_UNSUPPORTED",
          -5: "RK_ERR_TIMEOUT", -6: "RK_ERR_STATE", -7: "RK_ERR_NUMERIC"}

P = C.c_void_p
I32P = C.POINTER(C.c_int32)
DP = C.POINTER(C.c_double)
I64 = C.c_int64


class RkConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("form", C.c_int), ("entry_capacity", I64)]


class RkShapes(C.Structure):
    _fields_ = [("nshapes", C.c_int32), ("vert_ofs", P), ("vertices", P), ("edge_ofs", P), ("edges", P),
                ("face_ofs", P), ("face_vofs", P), ("face_verts", P), ("radius", P), ("obb", P)]


class RkBodies(C.Structure):
    _fields_ = [("n", I64), ("n_driven", I64), ("pos", P), ("vel", P), ("acc", P), ("Q", P), ("vrot", P),
                ("arot", P), ("homothety", P), ("mass", P), ("inertia", P), ("shape", P), ("group", P),
                ("cluster", P)]


class RkParams(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("gravity", C.c_double * 3), ("DVerlet", C.c_double),
                ("dVerlet", C.c_double), ("interVerlet", C.c_double), ("interVerletC", C.c_double),
                ("numerical_damping", C.c_double), ("law", C.c_int32), ("params_in_interfaces", C.c_int32),
                ("dynamic_update_nl", C.c_int32), ("disp_update_nl", C.c_double),
                ("angle_update_nl", C.c_double), ("ngroup", C.c_int32), ("table", P)]


class RkEntries(C.Structure):
    _fields_ = [("n", I64), ("i", P), ("j", P), ("type", P), ("isub", P), ("jsub", P), ("dn", P), ("fn", P),
                ("ft", P), ("mom", P), ("damp", P), ("bond", P)]


class RkInterfaces(C.Structure):
    _fields_ = [("n", I64), ("i", P), ("j", P), ("dn0", P), ("params", P), ("is_inner", P)]


class RkControl(C.Structure):
    _fields_ = [("type", C.c_int32), ("body", C.c_int32), ("value", C.c_double), ("vec", C.c_double * 3)]


class RkServo(C.Structure):
    _fields_ = [("kind", C.c_int32), ("icontr", C.c_int32), ("walls", C.c_int32 * 6), ("pressure", C.c_double)]


class RkSkinConfig(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("use_mlp", C.c_int32), ("skin_min", C.c_double), ("skin_max", C.c_double),
                ("dverlet_ratio", C.c_double), ("interval_min", C.c_int32), ("interval_max", C.c_int32),
                ("learning_rate", C.c_double), ("train_steps", C.c_int32), ("seed", C.c_uint64),
                ("partial_fraction", C.c_double), ("exact_contacts", C.c_int32)]


class RkSkinStats(C.Structure):
    _fields_ = [("rebuilds", I64), ("forced", I64), ("scheduled", I64), ("skin", C.c_double), ("interval", I64),
                ("last_rate", C.c_double), ("predicted_rate", C.c_double), ("loss", C.c_double),
                ("partial", I64), ("partial_bodies", I64), ("train_steps", I64), ("windows", I64),
                ("rebuild_ms", C.c_double), ("partial_ms", C.c_double)]


class RkStepReport(C.Structure):
    _fields_ = [("steps_done", I64), ("nl_updates", I64), ("n_entries", I64), ("n_active", I64),
                ("n_broken", I64), ("t", C.c_double)]


class RkStats(C.Structure):
    _fields_ = [("e_trans", C.c_double), ("e_rot", C.c_double), ("n_entries", I64), ("n_active", I64),
                ("n_broken", I64), ("nl_updates", I64), ("coordination", C.c_double)]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "rk_abi_version": (C.c_int, []),
    "rk_create": (C.c_int, [C.POINTER(P), C.POINTER(RkConfig)]),
    "rk_destroy": (None, [P]),
    "rk_last_error": (C.c_char_p, [P]),
    "rk_upload_shapes": (C.c_int, [P, C.POINTER(RkShapes)]),
    "rk_upload_bodies": (C.c_int, [P, C.POINTER(RkBodies)]),
    "rk_set_params": (C.c_int, [P, C.POINTER(RkParams)]),
    "rk_upload_entries": (C.c_int, [P, C.POINTER(RkEntries)]),
    "rk_upload_interfaces": (C.c_int, [P, C.POINTER(RkInterfaces)]),
    "rk_set_controls": (C.c_int, [P, C.POINTER(RkControl), C.c_int32, C.POINTER(RkServo)]),
    "rk_set_body_force": (C.c_int, [P, C.c_int, P, C.c_int32, P]),
    "rk_download_contributions": (C.c_int, [P, P, P, P]),
    "rk_extract_mean_velocity": (C.c_int, [P, P]),
    "rk_extract_dn_stat": (C.c_int, [P, P]),
    "rk_extract_cluster_aabb": (C.c_int, [P, C.c_int32, P]),
    "rk_extract_duo_balance": (C.c_int, [P, C.c_int32, C.c_int32, P]),
    "rk_download_body": (C.c_int, [P, I64, P]),
    "rk_set_shape_names": (C.c_int, [P, C.POINTER(C.c_char_p), C.c_int32]),
    "rk_format_conf": (C.c_int, [P, C.c_int32, C.c_char_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64)]),
    "rk_set_record_geometry": (C.c_int, [P, C.c_int]),
    "rk_set_form": (C.c_int, [P, C.c_int]),
    "rk_set_broadphase": (C.c_int, [P, C.c_int]),
    "rk_set_scenes": (C.c_int, [P, P]),
    "rk_set_graphs": (C.c_int, [P, C.c_int]),
    "rk_set_autotune": (C.c_int, [P, C.c_int]),
    "rk_get_block_sizes": (C.c_int, [P, P]),
    "rk_get_graph_stats": (C.c_int, [P, P, P]),
    "rk_accelerations": (C.c_int, [P]),
    "rk_update_nl": (C.c_int, [P]),
    "rk_step": (C.c_int, [P, I64, C.POINTER(RkStepReport)]),
    "rk_synchronize": (C.c_int, [P]),
    "rk_num_bodies": (I64, [P]),
    "rk_num_entries": (I64, [P]),
    "rk_num_interfaces": (I64, [P]),
    "rk_download_bodies": (C.c_int, [P] * 9),
    "rk_download_entries": (C.c_int, [P] * 16),
    "rk_download_interfaces": (C.c_int, [P] * 4),
    "rk_get_stats": (C.c_int, [P, C.POINTER(RkStats)]),
    "rk_last_step_timing": (C.c_int, [P, DP, C.POINTER(I64)]),
    "rk_upload_kinematics": (C.c_int, [P] * 7),
    "rk_set_profiling": (C.c_int, [P, C.c_int]),
    "rk_get_profile": (C.c_int, [P, P, P]),
    "rk_sort_keys": (C.c_int, [P, I64, C.c_int, C.c_int, P]),
    "rk_upload_kinematics_packed": (C.c_int, [P, P]),
    "rk_download_kinematics_packed": (C.c_int, [P, P]),
    "rk_sort_keys_noalloc": (C.c_int, [P, I64, C.c_int, C.c_int, P]),
    "rk_set_skin": (C.c_int, [P, C.POINTER(RkSkinConfig)]),
    "rk_get_skin_stats": (C.c_int, [P, C.POINTER(RkSkinStats)]),
    "rk_mlp_num_params": (C.c_int, []),
    "rk_mlp_set_params": (C.c_int, [P, P]),
    "rk_mlp_get_params": (C.c_int, [P, P]),
    "rk_mlp_forward": (C.c_int, [P, P, P]),
    "rk_mlp_gradient": (C.c_int, [P, P, P, C.c_int32, P, P]),
}

_lib = None


def load(path=LIBPATH):
    """Load librk_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("librk_gpu.so is not built (run __graft_entry__.build()): " + path)
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class RkError(RuntimeError):
    pass


class GpuScene:
    """One rk_ctx; arrays passed in are numpy, outputs are numpy."""

    def __init__(self, device=0, form=RK_FORM_FP64, entry_capacity=0):
        self.L = load()
        self.h = P()
        self._owned = True
        cfg = RkConfig(device, form, entry_capacity)
        rc = self.L.rk_create(C.byref(self.h), C.byref(cfg))
        if rc != RK_OK:
            raise RkError("rk_create failed: %s" % ERRORS.get(rc, rc))
        self._keep = []

    @classmethod
    def attach(cls, handle, owner):
        """A view of a context created elsewhere (the C++ host's), kept alive
        by `owner`; close() leaves the context to its owner."""
        g = cls.__new__(cls)
        g.L = load()
        g.h = P(handle)
        g._owned = False
        g._keep = [owner]
        return g

    def close(self):
        if self.h:
            if self._owned:
                self.L.rk_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != RK_OK:
            raise RkError("%s: %s: %s" % (what, ERRORS.get(rc, rc), self.L.rk_last_error(self.h).decode()))

    # ---- uploads
    def upload_shapes(self, sh):
        a = {k: _c(sh[k], np.int32) for k in ["vert_ofs", "edge_ofs", "edges", "face_ofs", "face_vofs", "face_verts"]}
        a.update({k: _c(sh[k], np.float64) for k in ["vertices", "radius", "obb"]})
        s = RkShapes(len(a["radius"]), *[_p(a[k]) for k in ["vert_ofs", "vertices", "edge_ofs", "edges", "face_ofs",
                                                            "face_vofs", "face_verts", "radius", "obb"]])
        self._chk(self.L.rk_upload_shapes(self.h, C.byref(s)), "rk_upload_shapes")

    def upload_bodies(self, b, n_driven):
        f = {k: _c(b[k], np.float64) for k in ["pos", "vel", "acc", "Q", "vrot", "arot", "homothety", "mass",
                                                "inertia"]}
        i = {k: _c(b[k], np.int32) for k in ["shape", "group", "cluster"]}
        n = len(f["mass"])
        s = RkBodies(n, n_driven, *[_p(f[k]) for k in ["pos", "vel", "acc", "Q", "vrot", "arot", "homothety",
                                                       "mass", "inertia"]], *[_p(i[k]) for k in ["shape", "group",
                                                                                                  "cluster"]])
        self._chk(self.L.rk_upload_bodies(self.h, C.byref(s)), "rk_upload_bodies")

    def set_params(self, t, dt, gravity, DVerlet, dVerlet, interVerlet, interVerletC, law, ngroup, table,
                   numerical_damping=0.0, params_in_interfaces=0, dynamic_update_nl=0, disp_update_nl=1.0,
                   angle_update_nl=1.0):
        tab = _c(table, np.float64)
        self._keep = [tab]
        p = RkParams(t, dt, (C.c_double * 3)(*gravity), DVerlet, dVerlet, interVerlet, interVerletC,
                     numerical_damping, law, params_in_interfaces, dynamic_update_nl, disp_update_nl,
                     angle_update_nl, ngroup, _p(tab))
        self._chk(self.L.rk_set_params(self.h, C.byref(p)), "rk_set_params")

    def upload_entries(self, e):
        ii = {k: _c(e[k], np.int32) for k in ["i", "j", "type", "isub", "jsub", "bond"]}
        ff = {k: _c(e[k], np.float64) for k in ["dn", "fn", "ft", "mom", "damp"]}
        s = RkEntries(len(ii["i"]), *[_p(ii[k]) for k in ["i", "j", "type", "isub", "jsub"]],
                      *[_p(ff[k]) for k in ["dn", "fn", "ft", "mom", "damp"]], _p(ii["bond"]))
        self._chk(self.L.rk_upload_entries(self.h, C.byref(s)), "rk_upload_entries")

    def upload_interfaces(self, i, j, dn0, params, is_inner):
        a = [_c(i, np.int32), _c(j, np.int32), _c(dn0, np.float64), _c(params, np.float64), _c(is_inner, np.int32)]
        s = RkInterfaces(len(a[0]), *[_p(x) for x in a])
        self._chk(self.L.rk_upload_interfaces(self.h, C.byref(s)), "rk_upload_interfaces")

    def set_controls(self, types, bodies, values, vecs, servo=None):
        n = len(types)
        arr = (RkControl * max(n, 1))()
        for k in range(n):
            arr[k].type = int(types[k])
            arr[k].body = int(bodies[k])
            arr[k].value = float(values[k])
            for d in range(3):
                arr[k].vec[d] = float(vecs[k][d])
        sv = RkServo()
        if servo is not None:
            sv.kind = int(servo["kind"])
            sv.icontr = int(servo["icontr"])
            for d in range(6):
                sv.walls[d] = int(servo["walls"][d])
            sv.pressure = float(servo["pressure"])
        self._chk(self.L.rk_set_controls(self.h, arr, n, C.byref(sv)), "rk_set_controls")

    def set_body_force(self, kind, params=(), body_volume=None):
        """The BodyForce plugin `kind` (a name of RK_BF or its number) with
        its conf parameters; body_volume (V h^3 per body) for ViscousFluid."""
        k = RK_BF[kind] if isinstance(kind, str) else int(kind)
        p = np.ascontiguousarray(params, np.float64)
        v = None if body_volume is None else np.ascontiguousarray(body_volume, np.float64)
        self._chk(self.L.rk_set_body_force(self.h, k, _p(p) if len(p) else None, len(p),
                                           _p(v) if v is not None else None), "rk_set_body_force")

    def set_broadphase(self, mode):
        self._chk(self.L.rk_set_broadphase(self.h, int(mode)), "rk_set_broadphase")

    def set_graphs(self, on=True):
        self._chk(self.L.rk_set_graphs(self.h, int(bool(on))), "rk_set_graphs")

    def graph_stats(self):
        a, b = C.c_int64(0), C.c_int64(0)
        self._chk(self.L.rk_get_graph_stats(self.h, C.byref(a), C.byref(b)), "rk_get_graph_stats")
        return {"captures": a.value, "replays": b.value}

    def autotune(self, rounds=2):
        self._chk(self.L.rk_set_autotune(self.h, int(rounds)), "rk_set_autotune")

    def block_sizes(self):
        a = (C.c_int32 * 4)()
        self._chk(self.L.rk_get_block_sizes(self.h, a), "rk_get_block_sizes")
        return {"narrow": a[0], "resultants": a[1], "global_vertices": a[2], "drift": a[3]}

    def set_scenes(self, scene_of):
        a = None if scene_of is None else _c(scene_of, np.int32)
        self._keep.append(a)
        self._chk(self.L.rk_set_scenes(self.h, _p(a)), "rk_set_scenes")

    def set_form(self, form):
        self._chk(self.L.rk_set_form(self.h, int(form)), "rk_set_form")

    def set_record_geometry(self, on=True):
        self._chk(self.L.rk_set_record_geometry(self.h, 1 if on else 0), "rk_set_record_geometry")

    # ---- running
    def accelerations(self):
        self._chk(self.L.rk_accelerations(self.h), "rk_accelerations")

    def update_nl(self):
        self._chk(self.L.rk_update_nl(self.h), "rk_update_nl")

    def step(self, n=1):
        r = RkStepReport()
        self._chk(self.L.rk_step(self.h, int(n), C.byref(r)), "rk_step")
        return {k: getattr(r, k) for k, _ in RkStepReport._fields_}

    def synchronize(self):
        self._chk(self.L.rk_synchronize(self.h), "rk_synchronize")

    def last_step_timing(self):
        ms = C.c_double()
        k = I64()
        self._chk(self.L.rk_last_step_timing(self.h, C.byref(ms), C.byref(k)), "rk_last_step_timing")
        return ms.value, k.value

    def upload_kinematics(self, pos=None, vel=None, acc=None, Q=None, vrot=None, arot=None):
        """Host arrays must stay alive until the next synchronising call."""
        self._chk(self.L.rk_upload_kinematics(self.h, _p(pos), _p(vel), _p(acc), _p(Q), _p(vrot), _p(arot)),
                  "rk_upload_kinematics")

    def upload_kinematics_packed(self, buf):
        """buf: C-contiguous float64 array of 19 n values (pos, vel, acc, Q,
        vrot, arot); must stay alive until the next synchronising call."""
        if buf.dtype != np.float64 or not buf.flags["C_CONTIGUOUS"] or buf.size != 19 * self.n:
            raise ValueError("packed kinematics: a C-contiguous float64 array of 19 x %d values" % self.n)
        self._chk(self.L.rk_upload_kinematics_packed(self.h, _p(buf)), "rk_upload_kinematics_packed")

    def download_kinematics_packed(self, buf):
        if buf.dtype != np.float64 or not buf.flags["C_CONTIGUOUS"] or buf.size != 19 * self.n:
            raise ValueError("packed kinematics: a C-contiguous float64 array of 19 x %d values" % self.n)
        self._chk(self.L.rk_download_kinematics_packed(self.h, _p(buf)), "rk_download_kinematics_packed")
        return buf

    def set_profiling(self, on=True):
        self._chk(self.L.rk_set_profiling(self.h, 1 if on else 0), "rk_set_profiling")

    def set_skin(self, enabled=True, use_mlp=True, skin_min=1e-5, skin_max=1e-3, dverlet_ratio=2.0,
                 interval_min=5, interval_max=1000, learning_rate=3e-3, train_steps=2, seed=1, partial_fraction=0.2,
                 exact_contacts=True):
        cfg = RkSkinConfig(1 if enabled else 0, 1 if use_mlp else 0, skin_min, skin_max, dverlet_ratio, interval_min,
                           interval_max, learning_rate, train_steps, seed, partial_fraction, 1 if exact_contacts else 0)
        self._chk(self.L.rk_set_skin(self.h, C.byref(cfg)), "rk_set_skin")

    def skin_stats(self):
        st = RkSkinStats()
        self._chk(self.L.rk_get_skin_stats(self.h, C.byref(st)), "rk_get_skin_stats")
        return {k: getattr(st, k) for k, _ in RkSkinStats._fields_}

    def mlp_num_params(self):
        return self.L.rk_mlp_num_params()

    def mlp_set_params(self, p):
        p = _c(p, np.float32)
        self._chk(self.L.rk_mlp_set_params(self.h, _p(p)), "rk_mlp_set_params")

    def mlp_get_params(self):
        p = np.zeros(self.mlp_num_params(), np.float32)
        self._chk(self.L.rk_mlp_get_params(self.h, _p(p)), "rk_mlp_get_params")
        return p

    def mlp_forward(self, x):
        x = _c(x, np.float32)
        y = np.zeros(2, np.float32)
        self._chk(self.L.rk_mlp_forward(self.h, _p(x), _p(y)), "rk_mlp_forward")
        return y

    def mlp_gradient(self, X, T):
        X = _c(X, np.float32)
        T = _c(T, np.float32)
        g = np.zeros(self.mlp_num_params(), np.float32)
        loss = np.zeros(1, np.float32)
        self._chk(self.L.rk_mlp_gradient(self.h, _p(X), _p(T), len(X), _p(g), _p(loss)), "rk_mlp_gradient")
        return g, float(loss[0])

    PHASES = ["controls", "drift", "glob_vertices", "narrow_force", "gather_accel", "breakage", "nl_rebuild", "guard"]

    def profile(self):
        ms = np.zeros(8)
        n = np.zeros(8, np.int64)
        self._chk(self.L.rk_get_profile(self.h, _p(ms), _p(n)), "rk_get_profile")
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.PHASES)}

    # ---- downloads
    @property
    def n(self):
        return self.L.rk_num_bodies(self.h)

    @property
    def n_entries(self):
        return self.L.rk_num_entries(self.h)

    def bodies(self, out=None):
        """Body state as float64 arrays; with `out` (a dict of C-contiguous
        float64 arrays, e.g. pinned buffers), only the fields it holds are
        downloaded, into those arrays."""
        n = self.n
        names = ["pos", "vel", "acc", "Q", "vrot", "arot", "force", "moment"]
        if out is None:
            out = {k: np.zeros((n, 4 if k == "Q" else 3)) for k in names}
        for k, v in out.items():
            if k not in names or v.dtype != np.float64 or not v.flags["C_CONTIGUOUS"] or v.size != n * (
                    4 if k == "Q" else 3):
                raise ValueError("bodies(out=...): %s must be a C-contiguous float64 array of %d x %d" % (
                    k, n, 4 if k == "Q" else 3))
        self._chk(self.L.rk_download_bodies(self.h, *[_p(out.get(k)) for k in names]), "rk_download_bodies")
        return out

    def entries(self, geometry=False):
        n = self.n_entries
        o = {k: np.zeros(n, np.int32) for k in ["i", "j", "type", "isub", "jsub", "bond"]}
        o.update({"dn": np.zeros(n), "fn": np.zeros(n), "damp": np.zeros(n), "ft": np.zeros((n, 3)),
                  "mom": np.zeros((n, 3)), "active": np.zeros(n, np.uint8)})
        g = {k: (np.zeros((n, 3)) if geometry else None) for k in ["n", "pos", "vel"]}
        if n:
            self._chk(self.L.rk_download_entries(
                self.h, _p(o["i"]), _p(o["j"]), _p(o["type"]), _p(o["isub"]), _p(o["jsub"]), _p(o["dn"]),
                _p(o["fn"]), _p(o["ft"]), _p(o["mom"]), _p(o["damp"]), _p(o["bond"]), _p(o["active"]),
                _p(g["n"]), _p(g["pos"]), _p(g["vel"])), "rk_download_entries")
        if geometry:
            o.update(g)
        o["active"] = o["active"].astype(bool)
        return o

    def set_shape_names(self, names):
        arr = (C.c_char_p * max(len(names), 1))(*[n.encode() for n in names])
        self._chk(self.L.rk_set_shape_names(self.h, arr, len(names)), "rk_set_shape_names")

    def format_conf(self, precision=16):
        """(Particles lines, Interactions lines, number of the latter) of a
        conf file, formatted on the device (rk_format_conf)."""
        lp, li, na = C.c_int64(), C.c_int64(), C.c_int64()
        self._chk(self.L.rk_format_conf(self.h, precision, None, 0, C.byref(lp), C.byref(li), C.byref(na)),
                  "rk_format_conf")
        buf = C.create_string_buffer(lp.value + li.value + 1)
        self._chk(self.L.rk_format_conf(self.h, precision, buf, lp.value + li.value, C.byref(lp), C.byref(li),
                                        C.byref(na)), "rk_format_conf")
        raw = buf.raw[:lp.value + li.value].decode()
        return raw[:lp.value], raw[lp.value:], na.value

    def contributions(self):
        """Per-entry force on i and moments on i and j of the last force
        evaluation (key order; meaningful for the active entries)."""
        ne = self.n_entries
        f, mi, mj = np.zeros((ne, 3)), np.zeros((ne, 3)), np.zeros((ne, 3))
        if ne:
            self._chk(self.L.rk_download_contributions(self.h, _p(f), _p(mi), _p(mj)), "rk_download_contributions")
        return f, mi, mj

    # ---- data extractors on the device (src/DataExtractors/*.cpp)
    def mean_velocity(self):
        """MeanVelocity: mean |v| over all bodies."""
        m = np.zeros(1)
        self._chk(self.L.rk_extract_mean_velocity(self.h, _p(m)), "rk_extract_mean_velocity")
        return float(m[0])

    def dn_stat(self):
        """dnStat over the active entries: dict of dnMin, dnMax, dnMean,
        dnMeanNeg, dnMeanPos, nbNeg, nbPos and pos (contact point of dnMin)."""
        o = np.zeros(10)
        self._chk(self.L.rk_extract_dn_stat(self.h, _p(o)), "rk_extract_dn_stat")
        return {"dnMin": o[0], "dnMax": o[1], "dnMean": o[2], "dnMeanNeg": o[3], "dnMeanPos": o[4],
                "nbNeg": int(o[5]), "nbPos": int(o[6]), "pos": o[7:10].copy()}

    def cluster_aabb(self, cluster):
        """ClusterAABB: (min[3], max[3]) of the cluster's bodies' vertices
        enlarged by their radii (zeros for an empty cluster)."""
        o = np.zeros(7)
        self._chk(self.L.rk_extract_cluster_aabb(self.h, int(cluster), _p(o)), "rk_extract_cluster_aabb")
        return o[1:4].copy(), o[4:7].copy()

    def duo_balance(self, i, j):
        """DuoBalance: sub-contacts of the pair (i, j) with dn < 0, by type."""
        o = np.zeros(4, dtype=np.int64)
        self._chk(self.L.rk_extract_duo_balance(self.h, int(i), int(j), _p(o)), "rk_extract_duo_balance")
        return o

    def body(self, b):
        """TrackBody's fields of body b: dict of pos, vel, acc, Q, vrot, arot,
        force, moment."""
        o = np.zeros(25)
        self._chk(self.L.rk_download_body(self.h, int(b), _p(o)), "rk_download_body")
        return {"pos": o[0:3], "vel": o[3:6], "acc": o[6:9], "Q": o[9:13], "vrot": o[13:16], "arot": o[16:19],
                "force": o[19:22], "moment": o[22:25]}

    def interfaces(self):
        n = self.L.rk_num_interfaces(self.h)
        i = np.zeros(n, np.int32)
        j = np.zeros(n, np.int32)
        b = np.zeros(n, np.uint8)
        if n:
            self._chk(self.L.rk_download_interfaces(self.h, _p(i), _p(j), _p(b)), "rk_download_interfaces")
        return i, j, b.astype(bool)

    def stats(self):
        s = RkStats()
        self._chk(self.L.rk_get_stats(self.h, C.byref(s)), "rk_get_stats")
        return {k: getattr(s, k) for k, _ in RkStats._fields_}


# ------------------------------------------------------------ C++ host --
HOSTPATH = os.path.join(os.path.dirname(LIBPATH), "librk_host.so")
_host = None


def load_host(path=HOSTPATH):
    """Load librk_host.so, the C++ host (conf in, conf out) over librk_gpu."""
    global _host
    if _host is None:
        if not os.path.exists(path):
            raise RuntimeError("librk_host.so is not built (run __graft_entry__.build()): " + path)
        load()
        L = C.CDLL(path)
        sig = {"rkh_open": (P, [C.c_char_p]), "rkh_error": (C.c_char_p, []), "rkh_close": (None, [P]),
               "rkh_read_driving": (C.c_int, [P, C.c_char_p]), "rkh_run": (C.c_int, [P, C.c_long]),
               "rkh_save_conf": (C.c_int, [P, C.c_char_p]), "rkh_context": (P, [P])}
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _host = L
    return _host


class HostScene:
    """A conf file loaded by the C++ host (conf and shape parsing, the
    preprocessing commands such as stickVerticesInClusters, the plugins),
    which uploads it to an engine context; `gpu` is a GpuScene view of that
    context for direct rk_* calls (rk_step, rk_set_form, downloads)."""

    def __init__(self, conf, driving=None):
        self.H = load_host()
        self.h = self.H.rkh_open(conf.encode())
        if not self.h:
            raise RkError("rkh_open: " + self.H.rkh_error().decode())
        if driving and self.H.rkh_read_driving(self.h, driving.encode()) != 0:
            raise RkError("rkh_read_driving: " + self.H.rkh_error().decode())
        self.gpu = GpuScene.attach(self.H.rkh_context(self.h), self)

    def save_conf(self, path):
        if self.H.rkh_save_conf(self.h, path.encode()) != 0:
            raise RkError("rkh_save_conf: " + self.H.rkh_error().decode())

    def close(self):
        if self.h:
            self.gpu.close()
            self.H.rkh_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
