"""Seeded synthetic scenes of the benchmark workloads.

Rockable ships no benchmark inputs; these generators build scenes with the
shapes, sizes and value distributions of the workloads the engine is measured
on, as numpy arrays ready for the C ABI, and can write them as Rockable
`.conf` / `.shp` files (Rockable.cpp:440-610, Shape.cpp:130-170 formats) so
that the reference CPU path reads exactly the same scene.

Grains are convex sphero-polyhedra: the convex hull of k ~ U{8..20} points on
an ellipsoid, Minkowski-summed with a sphere of radius 5% of the smallest
semi-axis.  Vertices are expressed in the principal frame of inertia, like
Rockable's shape library requires (Shape.hpp:60-62).
"""
import math
import os

import numpy as np

SEED = 20261203


# ------------------------------------------------------------------ shapes --
def _hull(points):
    from scipy.spatial import ConvexHull
    h = ConvexHull(points)
    used = np.unique(h.simplices)
    remap = -np.ones(len(points), dtype=np.int64)
    remap[used] = np.arange(len(used))
    verts = points[used]
    tris = remap[h.simplices]
    # outward orientation
    c = verts.mean(axis=0)
    for t in tris:
        a, b, d = verts[t[0]], verts[t[1]], verts[t[2]]
        if np.dot(np.cross(b - a, d - a), a - c) < 0:
            t[1], t[2] = t[2], t[1]
    return verts, tris


def _mass_properties(verts, tris):
    """Volume, centroid and inertia tensor (unit density) of a closed
    triangulated polyhedron, by signed tetrahedra from the origin."""
    V = 0.0
    C = np.zeros(3)
    J = np.zeros((3, 3))  # second moments  int x_i x_j dV
    for t in tris:
        a, b, c = verts[t[0]], verts[t[1]], verts[t[2]]
        v = np.dot(a, np.cross(b, c)) / 6.0
        V += v
        C += v * (a + b + c) / 4.0
        s = a + b + c
        J += v / 20.0 * (np.outer(a, a) + np.outer(b, b) + np.outer(c, c) + np.outer(s, s))
    C /= V
    J -= V * np.outer(C, C)
    inertia = np.trace(J) * np.eye(3) - J
    return V, C, inertia


def hull_shape(rng, name, kmin=8, kmax=20, semi_lo=0.0025, semi_hi=0.0075, rfrac=0.05):
    """One convex sphero-polyhedron (dict of the Shape fields)."""
    while True:
        k = int(rng.integers(kmin, kmax + 1))
        ax = rng.uniform(semi_lo, semi_hi, 3)
        d = rng.normal(size=(k, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        p = d * ax
        try:
            verts, tris = _hull(p)
        except Exception:
            continue
        if len(verts) >= 4:
            break
    V, C, I = _mass_properties(verts, tris)
    verts = verts - C
    w, R = np.linalg.eigh(I)
    if np.linalg.det(R) < 0:
        R[:, 0] = -R[:, 0]
    verts = verts @ R  # coordinates in the principal frame
    r = rfrac * float(ax.min())
    # faces: triangles; edges: unique vertex pairs of the triangles
    edges = set()
    for t in tris:
        for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            edges.add((min(a, b), max(a, b)))
    edges = sorted(edges)
    area = sum(0.5 * np.linalg.norm(np.cross(verts[t[1]] - verts[t[0]], verts[t[2]] - verts[t[0]])) for t in tris)
    vol = V + area * r + 4.0 / 3.0 * math.pi * r ** 3  # rounding shell to first order plus the corner sphere
    i_over_m = w / V
    lo = verts.min(axis=0) - r
    hi = verts.max(axis=0) + r
    return {"name": name, "radius": r, "volume": vol, "I/m": i_over_m, "vertices": verts, "edges": np.array(edges),
            "faces": [list(map(int, t)) for t in tris], "obb_center": 0.5 * (lo + hi), "obb_extent": 0.5 * (hi - lo),
            "bound": float(np.max(np.linalg.norm(verts, axis=1)) + r)}


def plate_shape(name, half, r):
    """A square plate (4 vertices, 1 face) in the z = 0 plane, like the wall
    shapes of Rockable's test inputs."""
    v = np.array([[half, half, 0.0], [half, -half, 0.0], [-half, -half, 0.0], [-half, half, 0.0]])
    return {"name": name, "radius": r, "volume": (2 * half) ** 2 * 2 * r,
            "I/m": np.array([(2 * half) ** 2 / 12.0, (2 * half) ** 2 / 12.0, (2 * half) ** 2 / 6.0]),
            "vertices": v, "edges": np.array([[0, 1], [0, 3], [1, 2], [2, 3]]), "faces": [[0, 1, 2, 3]],
            "obb_center": np.zeros(3), "obb_extent": np.array([half + r, half + r, r]), "bound": half * 1.5 + r}


def flatten_shapes(shapes):
    vo, eo, fo, fvo = [0], [0], [0], [0]
    verts, edges, fverts, rad, obb = [], [], [], [], []
    for s in shapes:
        verts.append(np.asarray(s["vertices"], dtype=np.float64))
        edges.append(np.asarray(s["edges"], dtype=np.int32).reshape(-1, 2))
        for f in s["faces"]:
            fverts.extend(f)
            fvo.append(len(fverts))
        vo.append(vo[-1] + len(s["vertices"]))
        eo.append(eo[-1] + len(s["edges"]))
        fo.append(fo[-1] + len(s["faces"]))
        rad.append(s["radius"])
        obb.extend(list(s["obb_center"]) + [1, 0, 0, 0, 1, 0, 0, 0, 1] + list(s["obb_extent"]))
    return {"vert_ofs": np.array(vo, np.int32), "vertices": np.concatenate(verts).ravel(),
            "edge_ofs": np.array(eo, np.int32), "edges": np.concatenate(edges).ravel().astype(np.int32),
            "face_ofs": np.array(fo, np.int32), "face_vofs": np.array(fvo, np.int32),
            "face_verts": np.array(fverts, np.int32), "radius": np.array(rad), "obb": np.array(obb, np.float64)}


def random_quaternions(rng, n):
    """Uniform rotations (Shoemake)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(u1) * np.cos(2 * np.pi * u3), np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
                  np.sqrt(1 - u1) * np.cos(2 * np.pi * u2), np.sqrt(u1) * np.sin(2 * np.pi * u3)], axis=1)
    return q / np.linalg.norm(q, axis=1)[:, None]


def resting_quaternions(rng, n, tilt_deg=25.0):
    """Orientations of grains lying flat, as in a settled pile: the shape's
    third principal axis (largest moment of inertia: the grain's shortest
    dimension) near the vertical, tilted by a uniform angle up to tilt_deg
    about a random horizontal axis, turned by a uniform angle about the
    vertical and flipped upside down half of the time."""
    turn = rng.uniform(0.0, 2.0 * np.pi, n)
    flip = rng.random(n) < 0.5
    tilt = np.radians(tilt_deg) * rng.random(n)
    az = rng.uniform(0.0, 2.0 * np.pi, n)
    qz = np.stack([np.cos(0.5 * turn), np.zeros(n), np.zeros(n), np.sin(0.5 * turn)], 1)
    qf = np.where(flip[:, None], np.array([0.0, 1.0, 0.0, 0.0]), np.array([1.0, 0.0, 0.0, 0.0]))
    qt = np.stack([np.cos(0.5 * tilt), np.sin(0.5 * tilt) * np.cos(az), np.sin(0.5 * tilt) * np.sin(az),
                   np.zeros(n)], 1)
    q = _qmul(qt, _qmul(qz, qf))
    return q / np.linalg.norm(q, axis=1)[:, None]


def _quat_from_to(a, b):
    """Unit quaternion (w, x, y, z) of the shortest rotation taking unit
    vector a to unit vector b."""
    c = float(np.dot(a, b))
    if c < -1.0 + 1e-12:  # opposite: half turn about any axis normal to a
        ax = np.cross(a, [1.0, 0.0, 0.0])
        if np.linalg.norm(ax) < 1e-6:
            ax = np.cross(a, [0.0, 1.0, 0.0])
        ax /= np.linalg.norm(ax)
        return np.array([0.0, ax[0], ax[1], ax[2]])
    v = np.cross(a, b)
    q = np.array([1.0 + c, v[0], v[1], v[2]])
    return q / np.linalg.norm(q)


def stable_face_quaternions(rng, shapes, shape_of):
    """Orientations of grains resting on a face: for each grain, the hull
    facet nearest its centre of mass along its outward normal (for a convex
    body that facet always holds it in equilibrium on a flat support: the
    centre of mass projects inside it) is turned face down, then the grain is
    turned by a uniform angle about the vertical."""
    down = np.array([0.0, 0.0, -1.0])
    face_q = {}
    for s in np.unique(shape_of):
        v = np.asarray(shapes[s]["vertices"])
        best, qb = None, None
        for f in shapes[s]["faces"]:
            a, b, c = v[f[0]], v[f[1]], v[f[-1]]
            nrm = np.cross(b - a, c - a)
            ln = np.linalg.norm(nrm)
            if ln == 0.0:
                continue
            nrm /= ln
            h = float(np.dot(a, nrm))  # distance of the facet plane from the centre of mass
            if h > 0.0 and (best is None or h < best):
                best, qb = h, _quat_from_to(nrm, down)
        face_q[int(s)] = qb if qb is not None else np.array([1.0, 0.0, 0.0, 0.0])
    n = len(shape_of)
    turn = rng.uniform(0.0, 2.0 * np.pi, n)
    qz = np.stack([np.cos(0.5 * turn), np.zeros(n), np.zeros(n), np.sin(0.5 * turn)], 1)
    qf = np.array([face_q[int(s)] for s in shape_of])
    q = _qmul(qz, qf)
    return q / np.linalg.norm(q, axis=1)[:, None]


# ------------------------------------------------------------------ scenes --
def deposit(rng, radii, half_x, half_y, z0, gap=1e-5):
    """Loose random packing by ballistic deposition: each grain, in the given
    order, drops vertically at a random (x, y) in the column and stops on the
    floor or on the first bounding sphere it meets (no rolling)."""
    rmax = float(np.max(radii))
    cs = 2.0 * rmax
    nx = max(1, int(2 * half_x / cs))
    ny = max(1, int(2 * half_y / cs))
    cap = 64
    cells = np.zeros((nx, ny, cap, 4))  # x y z r of the grains of each column cell
    count = np.zeros((nx, ny), dtype=np.int64)
    top = np.zeros((nx, ny))
    pos = np.zeros((len(radii), 3))
    for k, r in enumerate(radii):
        x = rng.uniform(-half_x + r, half_x - r)
        y = rng.uniform(-half_y + r, half_y - r)
        cx = min(nx - 1, int((x + half_x) / cs))
        cy = min(ny - 1, int((y + half_y) / cs))
        z = z0 + r
        x0, x1, y0, y1 = max(cx - 1, 0), min(cx + 2, nx), max(cy - 1, 0), min(cy + 2, ny)
        blk = cells[x0:x1, y0:y1]
        cnt = count[x0:x1, y0:y1]
        mask = np.arange(cap)[None, None, :] < cnt[:, :, None]
        c = blk[mask]
        if len(c):
            d2 = (c[:, 0] - x) ** 2 + (c[:, 1] - y) ** 2
            rr = (c[:, 3] + r + gap) ** 2
            hit = d2 < rr
            if hit.any():
                z = max(z, float(np.max(c[hit, 2] + np.sqrt(rr[hit] - d2[hit]))))
        pos[k] = (x, y, z)
        if count[cx, cy] == cap:  # keep the highest grains of a cell only
            lo = int(np.argmin(cells[cx, cy, :, 2]))
            cells[cx, cy, lo] = (x, y, z, r)
        else:
            cells[cx, cy, count[cx, cy]] = (x, y, z, r)
            count[cx, cy] += 1
    return pos


PACK_MAGIC = 0x524b5041434b3033  # "RKPACK03"


def _cache_dir():
    import tempfile
    d = os.environ.get("RK_SCENE_CACHE", os.path.join(tempfile.gettempdir(), "rockable_gb300_scenes"))
    os.makedirs(d, exist_ok=True)
    return d


def pack(shapes, shape_of, Q, volume, lo, hi, scale=None, tol=1e-9, seed=SEED, max_iters=200, tries=1, cache=True):
    """Loose random packing by sequential ballistic deposition with the exact
    grain geometry (the CPU packer host/rk_pack.cpp): the grains, with the
    given shapes (indices into `shapes`), uniform scale factors and
    orientations, one at a time from a seeded random point of the footprint
    [lo, hi] (x, y, side walls there), fall onto the floor lo z or the grains
    already there and slide without friction (translating only) until three
    supports hold them, within `tol`; they never overlap.  With tries > 1,
    each grain is dropped from that many random points and kept where it
    comes to rest lowest (denser packings).  Returns
    (positions (n, 3), stats).  The result is cached by the hash of its input
    (RK_SCENE_CACHE or the temp directory), so that the processes of one
    benchmark run pack once."""
    import hashlib
    import subprocess
    import tempfile
    n = len(shape_of)
    nv = np.array([len(s["vertices"]) for s in shapes], np.int32)
    rad = np.array([s["radius"] for s in shapes], np.float64)
    verts = np.concatenate([np.asarray(s["vertices"], np.float64).ravel() for s in shapes])
    scale = np.ones(n) if scale is None else np.asarray(scale, np.float64)
    prm = np.array(list(lo) + list(hi) + [tol, float(seed)], np.float64)
    parts = [np.array([PACK_MAGIC, len(shapes)], np.int64).tobytes(), nv.tobytes(), rad.tobytes(), verts.tobytes(),
             np.array([n], np.int64).tobytes(), np.asarray(shape_of, np.int32).tobytes(), scale.tobytes(),
             np.ascontiguousarray(Q, np.float64).tobytes(), np.asarray(volume, np.float64).tobytes(), prm.tobytes(),
             np.array([max_iters, tries], np.int64).tobytes()]
    blob = b"".join(parts)
    from . import build_ext
    exe = build_ext.build_packer()
    key = hashlib.sha1(blob + open(os.path.join(build_ext.HERE, "host", "rk_pack.cpp"), "rb").read()).hexdigest()
    out_path = os.path.join(_cache_dir(), "pack_%s.bin" % key)
    if cache and os.path.exists(out_path) and os.path.getsize(out_path) == 8 * (3 * n + 8):
        raw = np.fromfile(out_path, np.float64)
    else:
        with tempfile.TemporaryDirectory(prefix="rk_pack_") as d:
            inp = os.path.join(d, "in.bin")
            tmp = os.path.join(d, "out.bin")
            with open(inp, "wb") as f:
                f.write(blob)
            r = subprocess.run([exe, inp, tmp], capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("rk_pack failed (%d): %s" % (r.returncode, r.stderr))
            raw = np.fromfile(tmp, np.float64)
            if cache:
                os.replace(tmp, out_path)
    s = raw[3 * n:]
    return raw[:3 * n].reshape(n, 3), {"touching_pairs": int(s[0]), "on_floor": int(s[1]), "top": float(s[2]),
                                       "solid_fraction": float(s[3]), "moves": int(s[4]), "at_rest": int(s[5]),
                                       "max_overlap": float(s[6])}


def rockfall_bonded(nclusters=40, per=500, seed=SEED, nshapes=1024, semi=(0.005, 0.01), slope_deg=30.0,
                    v0=10.0, density=2700.0, kn=1e7, kt=1e7, en2=0.25, mu=0.4, dt=1e-6, bond_kn=1e5,
                    bond_kt=1e5, fn0_scale=1e3, fn0_m=5.0, ft0=1e3, eps=None, target_bonds=120000):
    """Breakable bonded rockfall: `nclusters` blocks of `per` hull grains
    (semi-axes U[0.5, 1.0] cm: 1-2 cm grains), each block packed on its own
    (pack(), about a 10 cm cube) and given its own cluster id, in a grid
    just above a rigid plate inclined at `slope_deg`, all moving at `v0`
    straight down.  StickedLinks law: contacts at kn, and inner bonds made
    at load by the conf's own preprocessing commands --
    stickVerticesInClusters eps (PreproCommand_stickVerticesInClusters.cpp:
    56-141: vertex-vertex bonds between grains of one cluster whose vertex
    spheres come within eps) and setVariableStickParams fn0 inner
    <fn0_scale> <fn0_m> 0 (PreproCommand_setVariableStickParams.cpp:57-94:
    Weibull tensile strengths).  eps defaults to the distance that gives
    about `target_bonds` vertex pairs.  The bonds' rest distance is zero
    (the interface's dn0, never set by that command), so a bond made across
    a gap starts in tension: at bond_kn = 1e5 N/m a gap of a few mm pulls
    with a few hundred N, below the strengths, and the blocks hold together
    until they hit the slope.  Returns a scene (for write_conf) with
    "conf_extra" (bond parameters) and "conf_tail" (the two commands)."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    th = math.radians(slope_deg)
    shapes = [plate_shape("SLOPE", 1.0, 0.01)]
    shapes += [hull_shape(rng, "R%04d" % k, semi_lo=semi[0], semi_hi=semi[1]) for k in range(nshapes)]
    bmax = max(float(sh["bound"]) for sh in shapes[1:])
    side = 0.1
    blocks = []
    for c in range(nclusters):
        so = rng.integers(1, nshapes + 1, per)
        Qc = stable_face_quaternions(rng, shapes, so)
        vol = np.array([shapes[k]["volume"] for k in so])
        pos, st = pack(shapes, so, Qc, vol, (-0.5 * side, -0.5 * side, 0.0), (0.5 * side, 0.5 * side, 1.0),
                       seed=seed + 1 + c, tries=16)
        blocks.append((so, Qc, pos, st))
    # the slope: plate through the origin, normal n, downhill direction u
    n = np.array([math.sin(th), 0.0, math.cos(th)])
    u = np.array([math.cos(th), 0.0, -math.sin(th)])
    qs = np.array([math.cos(0.5 * th), 0.0, math.sin(0.5 * th), 0.0])
    ncol = int(math.ceil(math.sqrt(nclusters * 1.6)))
    nrow = int(math.ceil(nclusters / ncol))
    pitch = 1.3 * side
    P, Q, S, K = [], [], [], []
    for c, (so, Qc, pos, st) in enumerate(blocks):
        a, b = c % ncol, c // ncol
        centre = (a - 0.5 * (ncol - 1)) * pitch * u + np.array([0.0, (b - 0.5 * (nrow - 1)) * pitch, 0.0])
        p = pos + centre
        # lift the block along the vertical until its lowest grain is 2 mm
        # (plus the rounding) above the plate (grain extents from their
        # bounding spheres)
        r = np.array([shapes[k]["bound"] for k in so])
        gap = (p @ n - r).min()
        p = p + ((0.002 - gap) / n[2]) * np.array([0.0, 0.0, 1.0])
        P.append(p)
        Q.append(Qc)
        S.append(so)
        K.append(np.full(per, c + 1, np.int32))
    pos = np.concatenate(P)
    Qa = np.concatenate(Q)
    so = np.concatenate(S)
    cl = np.concatenate(K)
    out = _assemble(shapes, [-0.01 * n], [qs], pos, Qa, so, density, "StickedLinks", kn, kt, en2, mu, dt,
                    gravity=(0.0, 0.0, -9.81), DVerlet=0.2 * bmax, dVerlet=0.1 * bmax, interVerlet=100 * dt,
                    name="rockfall_bonded_%dx%d" % (nclusters, per), wall_shape=0)
    out["bodies"]["cluster"] = np.concatenate([[0], cl]).astype(np.int32)
    out["bodies"]["vel"][1:] = [0.0, 0.0, -v0]
    if eps is None:
        # vertex spheres of grains of one cluster: pairs within eps + Ri + Rj
        V, owner = [], []
        for i in range(1, len(out["bodies"]["mass"])):
            sh = shapes[out["bodies"]["shape"][i]]
            q = out["bodies"]["Q"][i]
            V.append(_qrot_np(q, np.asarray(sh["vertices"])) + out["bodies"]["pos"][i])
            owner += [i] * len(sh["vertices"])
        V = np.concatenate(V)
        owner = np.asarray(owner)
        rad = np.array([shapes[out["bodies"]["shape"][i]]["radius"] for i in owner])
        tree = cKDTree(V)
        pairs = tree.query_pairs(0.004, output_type="ndarray")
        pairs = pairs[(owner[pairs[:, 0]] != owner[pairs[:, 1]]) &
                      (out["bodies"]["cluster"][owner[pairs[:, 0]]] == out["bodies"]["cluster"][owner[pairs[:, 1]]])]
        gaps = np.sort(np.linalg.norm(V[pairs[:, 0]] - V[pairs[:, 1]], axis=1) - rad[pairs[:, 0]] - rad[pairs[:, 1]])
        eps = float(gaps[min(target_bonds, len(gaps)) - 1]) if len(gaps) else 0.001
        eps = max(eps, 1e-6)
    out["pack"] = {"clusters": nclusters, "per_cluster": per, "solid_fraction_bulk": float(np.mean(
        [st["solid_fraction"] for *_, st in blocks])), "coordination": float(np.mean(
        [2.0 * st["touching_pairs"] / per for *_, st in blocks]))}
    out["bond_eps"] = eps
    out["params"].update({"bond_kn": bond_kn, "bond_kt": bond_kt, "fn0_scale": fn0_scale, "fn0_m": fn0_m, "ft0": ft0})
    out["conf_extra"] = ["%s 0 0 %r" % kv for kv in [
        ("knInnerBond", bond_kn), ("ktInnerBond", bond_kt), ("krInnerBond", 0.0), ("en2InnerBond", en2),
        ("fn0InnerBond", fn0_scale), ("ft0InnerBond", ft0), ("mom0InnerBond", 1e10), ("powInnerBond", 2.0)]]
    out["conf_tail"] = ["stickVerticesInClusters %r" % eps,
                        "setVariableStickParams fn0 inner %r %r 0" % (fn0_scale, fn0_m)]
    return out


def _qrot_np(q, v):
    """Rotate the rows of v by the unit quaternion q = (w, x, y, z)."""
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    return v @ R.T


def packing_stats(pos, vol, lo, hi, inset, st):
    """Bulk solid fraction (grain volume with centres inside the packing's
    box shrunk by `inset` on every side, over that box's volume: away from
    the floor, the side walls and the rough top) and mean coordination
    (2 x touching pairs / grains, the floor counted) of a packing."""
    lo = np.asarray(lo, np.float64) + inset
    hi = np.asarray(hi, np.float64) - inset
    inside = np.all((pos >= lo) & (pos <= hi), axis=1)
    st["solid_fraction_bulk"] = float(vol[inside].sum() / np.prod(hi - lo)) if np.all(hi > lo) else 0.0
    st["coordination"] = 2.0 * st["touching_pairs"] / len(pos)
    return st


def column_collapse(n=50000, seed=SEED, nshapes=4096, law="Avalanche", density=2700.0, kn=1e6, kt=1e6,
                    en2=0.25, mu=0.4, dt=1e-6, column=(0.5, 0.5, 1.5), walls=False, semi=(0.005, 0.015), tries=16):
    """Granular column collapse: n hull grains (semi-axes U[0.5, 1.5] cm,
    rounding 5 % of the smallest), each resting on a face, in a random
    packing (sequential deposition with frictionless sliding, each grain
    kept at the lowest of `tries` drop sites, pack()) that fills a
    0.5 x 0.5 m column on a rigid floor plate (body 0) to about 1.1 m; the
    grains touch (within 1e-9 m) but carry no load yet.  With walls, four
    vertical plates (bodies 1-4, listed in
    "walls") confine the column as it was packed, to be removed
    (drop_bodies) when the collapse starts; without, the walls are already
    released (t = 0 of the collapse)."""
    rng = np.random.default_rng(seed)
    shapes = [plate_shape("FLOOR", 1.5, 0.005)]
    shapes += [hull_shape(rng, "G%05d" % k, semi_lo=semi[0], semi_hi=semi[1]) for k in range(nshapes)]
    shape_of = rng.integers(1, nshapes + 1, n)
    Q = stable_face_quaternions(rng, shapes, shape_of)
    vol = np.array([shapes[k]["volume"] for k in shape_of])
    hx, hy = 0.5 * column[0], 0.5 * column[1]
    z0 = 0.005
    pos, st = pack(shapes, shape_of, Q, vol, (-hx, -hy, z0), (hx, hy, column[2]), seed=seed, tries=tries)
    bmax = max(float(shapes[k]["bound"]) for k in np.unique(shape_of))
    packing_stats(pos, vol, (-hx, -hy, z0), (hx, hy, st["top"]), 2.0 * bmax, st)
    wall_pos, wall_Q, wall_shape = [np.zeros(3)], [np.array([1.0, 0, 0, 0])], [0]
    if walls:
        rw = 0.005
        top = st["top"]
        half = max(max(hx, hy) + 0.05, 0.5 * top + 0.05)
        shapes.append(plate_shape("WALL", half, rw))  # after the grain shapes: their indices do not move
        ws = len(shapes) - 1
        s2 = math.sqrt(0.5)
        zc = 0.5 * top
        wall_pos += [np.array([hx + rw, 0, zc]), np.array([-hx - rw, 0, zc]), np.array([0, hy + rw, zc]),
                     np.array([0, -hy - rw, zc])]
        wall_Q += [np.array([s2, 0, s2, 0]), np.array([s2, 0, s2, 0]), np.array([s2, s2, 0, 0]),
                   np.array([s2, s2, 0, 0])]
        wall_shape += [ws] * 4
    out = _assemble(shapes, wall_pos, wall_Q, pos, Q, shape_of, density, law, kn, kt, en2,
                    mu, dt, gravity=(0.0, 0.0, -9.81), DVerlet=0.2 * bmax, dVerlet=0.1 * bmax,
                    interVerlet=100 * dt, name="column_collapse_%d" % n, wall_shape=wall_shape)
    out["pack"] = st
    if walls:
        out["walls"] = [1, 2, 3, 4]
    return out


def iso_compression(n=200000, seed=SEED, nshapes=4096, law="Default", density=2700.0, kn=1e6, kt=1e6, en2=0.25,
                    mu=0.4, dt=5e-7, pressure=1e5, wall_density=None, size=(0.01, 0.03), tries=16):
    """Dense isotropic compression: n hull grains (8-20 vertices, diameters
    uniform in `size`, 1-3 cm: ratio 1:3, by homothety of a library of
    shapes of about 1 cm; dt = 5e-7 s: at 1e-6 s the smallest grains of the
    top layer, squeezed by the incoming walls, spin up without bound), packed (pack(), the lowest of `tries` drop sites per grain)
    in a box about as high as wide, then enclosed by six rigid walls (bodies
    0-5: Xmin, Xmax, Ymin, Ymax, Zmin, Zmax) driven by Rockable's
    tritriIsostaticCompression servo at `pressure` (DrivingSystem.cpp:
    242-268: the min walls are held, the max walls pushed with pressure x
    their face area); no gravity.  The grains touch but carry no load: the
    servo loads them.  The walls have the grains' density by default: heavy
    walls, pushed at the servo's force across the loose top layer, gather a
    momentum that crushes the first grains they meet."""
    rng = np.random.default_rng(seed)
    lib = [hull_shape(rng, "G%05d" % k, semi_lo=0.004, semi_hi=0.006) for k in range(nshapes)]
    shape_of = rng.integers(0, nshapes, n)
    lib_d = np.array([2.0 * s["bound"] for s in lib])
    h = rng.uniform(size[0], size[1], n) / lib_d[shape_of]
    Q = stable_face_quaternions(rng, lib, shape_of)
    vol = np.array([lib[k]["volume"] for k in shape_of]) * h ** 3
    L = float((vol.sum() / 0.5) ** (1.0 / 3.0))  # about a cube at the packing's solid fraction
    pos, st = pack(lib, shape_of, Q, vol, (-0.5 * L, -0.5 * L, 0.0), (0.5 * L, 0.5 * L, 4.0 * L), scale=h,
                   seed=seed, tries=tries)
    top = st["top"]
    bmax = float(np.max(lib_d[shape_of] * h)) * 0.5
    packing_stats(pos, vol, (-0.5 * L, -0.5 * L, 0.0), (0.5 * L, 0.5 * L, top), 2.0 * bmax, st)
    # the box's faces (x, y, z): lo, hi
    faces = np.array([[-0.5 * L, 0.5 * L], [-0.5 * L, 0.5 * L], [0.0, top]])
    centre = faces.mean(axis=1)
    rw = 0.005
    half = 0.5 * max(L, top) + 0.02
    shapes = [plate_shape("WALL", half, rw)] + lib
    s2 = math.sqrt(0.5)
    zc = centre[2]
    wall_pos = [np.array([faces[0, 0] - rw, 0, zc]), np.array([faces[0, 1] + rw, 0, zc]),
                np.array([0, faces[1, 0] - rw, zc]), np.array([0, faces[1, 1] + rw, zc]),
                np.array([0, 0, faces[2, 0] - rw]), np.array([0, 0, faces[2, 1] + rw])]
    wall_Q = [np.array([s2, 0, s2, 0])] * 2 + [np.array([s2, s2, 0, 0])] * 2 + [np.array([1.0, 0, 0, 0])] * 2
    out = _assemble(shapes, wall_pos, wall_Q, pos, Q, shape_of + 1, density, law, kn, kt, en2, mu, dt,
                    gravity=(0.0, 0.0, 0.0), DVerlet=0.2 * bmax, dVerlet=0.1 * bmax, interVerlet=100 * dt,
                    name="iso_compression_%d" % n, wall_shape=0, homothety=h, wall_density=wall_density)
    out["pack"] = st
    # tritriIsostaticCompression: x/y/z velocity controls on the min walls,
    # force controls on the max walls, the servo setting the forces
    out["controls"] = {"type": [0, 6, 1, 7, 2, 8], "body": [0, 1, 2, 3, 4, 5], "value": [0.0] * 6,
                       "vec": [[0.0, 0.0, 0.0]] * 6}
    out["servo"] = {"kind": 1, "icontr": 0, "walls": [0, 1, 2, 3, 4, 5], "pressure": pressure}
    return out


def drop_bodies(scene, drop):
    """The scene without the given bodies (e.g. released walls); the other
    bodies keep their relative order and the entries that involve a dropped
    body are removed (the others keep their key order)."""
    n = len(scene["bodies"]["mass"])
    keep = np.setdiff1d(np.arange(n), np.asarray(drop, np.int64))
    new = -np.ones(n, np.int64)
    new[keep] = np.arange(len(keep))
    out = dict(scene)
    out["bodies"] = {k: np.asarray(v)[keep] for k, v in scene["bodies"].items()}
    out["n_driven"] = int(np.sum(keep < scene["n_driven"]))
    out.pop("walls", None)
    if scene.get("entries") is not None:
        e = scene["entries"]
        ok = (new[e["i"]] >= 0) & (new[e["j"]] >= 0)
        ne = {k: np.asarray(v)[ok] for k, v in e.items()}
        ne["i"] = new[ne["i"]].astype(np.int32)
        ne["j"] = new[ne["j"]].astype(np.int32)
        out["entries"] = ne
    return out


def sphero_cube_box(n_side=8, seed=SEED, dt=1e-6):
    """512 sphero-cubes (side 1 mm, rounding 0.1 mm, density 2700) on an 8x8x8
    lattice of 1.5 mm spacing with uniform-random orientations, in a rigid box
    of 6 plates; Default law kn = 1e6 N/m, e_n^2 = 0.25, mu = 0.4."""
    rng = np.random.default_rng(seed)
    h = 0.4e-3
    r = 0.1e-3
    v = np.array([[sx * h, sy * h, sz * h] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])
    tris = []
    quads = [[0, 1, 3, 2], [4, 6, 7, 5], [0, 4, 5, 1], [2, 3, 7, 6], [0, 2, 6, 4], [1, 5, 7, 3]]
    edges = sorted({(min(a, b), max(a, b)) for q in quads for a, b in zip(q, q[1:] + q[:1])})
    side = 2 * h + 2 * r
    vol = (2 * h) ** 3 + 6 * (2 * h) ** 2 * r + 3 * math.pi * r * r * (2 * h) + 4.0 / 3.0 * math.pi * r ** 3
    cube = {"name": "CUBE", "radius": r, "volume": vol, "I/m": np.full(3, side * side / 6.0), "vertices": v,
            "edges": np.array(edges), "faces": quads, "obb_center": np.zeros(3),
            "obb_extent": np.full(3, h + r), "bound": math.sqrt(3) * h + r}
    bound = math.sqrt(3) * h + r
    sp = max(1.5e-3, 2.0 * bound * 1.01)  # 1.5 sides, widened so that rotated cubes cannot overlap
    L = n_side * sp + 2e-4
    wall = plate_shape("WALL", 0.5 * L + 1e-3, 0.1e-3)
    shapes = [wall, cube]
    c = 0.5 * L
    wpos = [np.array([c, c, 0.0]), np.array([c, c, L]), np.array([c, 0.0, c]), np.array([c, L, c]),
            np.array([0.0, c, c]), np.array([L, c, c])]
    s2 = math.sqrt(0.5)
    wq = [np.array([1.0, 0, 0, 0]), np.array([1.0, 0, 0, 0]), np.array([s2, -s2, 0, 0]), np.array([s2, s2, 0, 0]),
          np.array([s2, 0, -s2, 0]), np.array([s2, 0, s2, 0])]
    g = (np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), np.arange(n_side), indexing="ij"), -1)
         .reshape(-1, 3) + 0.5) * sp + 1e-4
    Q = random_quaternions(rng, len(g))
    return _assemble(shapes, wpos, wq, g, Q, np.ones(len(g), np.int64), 2700.0, "Default", 1e6, 1e6, 0.25, 0.4, dt,
                     gravity=(0.0, 0.0, -9.81), DVerlet=0.2e-3, dVerlet=0.1e-3, interVerlet=1e-4,
                     name="sphero_cubes_%d" % len(g), wall_shape=0)


def _qmul(a, b):
    """Hamilton product of quaternions stored (w, x, y, z), broadcast over rows."""
    aw, ax, ay, az = np.moveaxis(np.asarray(a, np.float64), -1, 0)
    bw, bx, by, bz = np.moveaxis(np.asarray(b, np.float64), -1, 0)
    return np.stack([aw * bw - ax * bx - ay * by - az * bz, aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx, aw * bz + ax * by - ay * bx + az * bw], -1)


def tilt(scene, theta):
    """The scene rotated by theta (radians) about the y axis through the
    origin: positions, orientations and all body vectors (a slope of angle
    theta when the scene was built on a horizontal floor)."""
    c, s_ = math.cos(theta), math.sin(theta)
    R = np.array([[c, 0.0, s_], [0.0, 1.0, 0.0], [-s_, 0.0, c]])
    q = np.array([math.cos(0.5 * theta), 0.0, math.sin(0.5 * theta), 0.0])
    out = dict(scene)
    b = dict(scene["bodies"])
    for k in ["pos", "vel", "acc", "vrot", "arot"]:
        b[k] = np.asarray(b[k]) @ R.T
    Qn = _qmul(q[None, :], b["Q"])
    b["Q"] = Qn / np.linalg.norm(Qn, axis=1)[:, None]
    out["bodies"] = b
    out.pop("entries", None)
    return out


def batch(parts, name=None):
    """Several independent scenes as one: the driven bodies of every part
    first (part order), then the free bodies of every part (part order), so
    that each part keeps the relative order of its bodies.  Returns the
    combined scene with `scene_of` (part index of every body) and
    `index_of` (per part: new index of each of its bodies).  The parts must
    share their parameters (law, table, dt, gravity, Verlet distances); they
    share one shape list when they hold the same list object."""
    p0 = parts[0]
    for p in parts[1:]:
        for k in ["law", "dt", "DVerlet", "dVerlet", "interVerlet", "ngroup"]:
            assert p[k] == p0[k], k
        assert tuple(p["gravity"]) == tuple(p0["gravity"])
        assert np.array_equal(p["table"], p0["table"])
    shared = all(p["shapes"] is p0["shapes"] for p in parts)
    shapes, sofs = (list(p0["shapes"]), [0] * len(parts)) if shared else ([], [])
    if not shared:
        for p in parts:
            sofs.append(len(shapes))
            shapes.extend(p["shapes"])
    nds = [p["n_driven"] for p in parts]
    ns = [len(p["bodies"]["mass"]) for p in parts]
    ND = sum(nds)
    index_of, dstart, fstart = [], 0, ND
    for nd, n in zip(nds, ns):
        idx = np.empty(n, np.int64)
        idx[:nd] = dstart + np.arange(nd)
        idx[nd:] = fstart + np.arange(n - nd)
        dstart += nd
        fstart += n - nd
        index_of.append(idx)
    N = fstart
    keys = list(p0["bodies"].keys())
    bodies = {}
    for k in keys:
        a0 = np.asarray(p0["bodies"][k])
        out = np.zeros((N,) + a0.shape[1:], a0.dtype)
        for p, idx, so in zip(parts, index_of, sofs):
            v = np.asarray(p["bodies"][k])
            out[idx] = v + so if k == "shape" else v
        bodies[k] = out
    scene_of = np.zeros(N, np.int32)
    for s_, idx in enumerate(index_of):
        scene_of[idx] = s_
    out = dict(p0)
    out.pop("entries", None)
    out.update({"name": name or "batch_%d" % len(parts), "shapes": shapes, "n_driven": ND, "bodies": bodies,
                "shape_tables": p0["shape_tables"] if shared else flatten_shapes(shapes), "scene_of": scene_of,
                "index_of": index_of, "free_per_scene": [n - nd for n, nd in zip(ns, nds)]})
    return out


def part_of(batched, k):
    """Part k of a scene built by batch(), as a scene of its own (shared
    shape list, the part's bodies in their original order)."""
    idx = batched["index_of"][k]
    out = dict(batched)
    for key in ["scene_of", "index_of", "free_per_scene", "slope_deg", "entries"]:
        out.pop(key, None)
    out["bodies"] = {key: np.asarray(v)[idx] for key, v in batched["bodies"].items()}
    out["n_driven"] = int(np.sum(idx < batched["n_driven"]))
    out["name"] = "%s_part%d" % (batched["name"], k)
    return out


def slope_batch(nscenes=256, seed=SEED, nmin=200, nmax=5000, nshapes=256, density=2700.0, kn=1e6, kt=1e6,
                en2=0.25, mu=0.4, dt=1e-6):
    """Many independent slope scenes: scene k draws N_k ~ U{nmin..nmax} hull
    grains and a slope angle U[25, 45] degrees from the generator seeded
    seed + 1 + k; its grains are deposited ballistically on a square patch of
    a rigid plate (about 8 layers), and the plate and the pile are tilted by
    the slope angle (gravity stays vertical).  Default law.  All scenes share
    one shape library (a plate and nshapes grain shapes)."""
    rng = np.random.default_rng(seed)
    shapes = [plate_shape("SLOPE", 0.5, 0.005)]
    shapes += [hull_shape(rng, "B%04d" % k) for k in range(nshapes)]
    bound = np.array([s["bound"] for s in shapes])
    bmax = float(bound[1:].max())
    parts, angles = [], []
    for k in range(nscenes):
        rs = np.random.default_rng(seed + 1 + k)
        n = int(rs.integers(nmin, nmax + 1))
        theta = math.radians(float(rs.uniform(25.0, 45.0)))
        shape_of = rs.integers(1, nshapes + 1, n)
        half = 0.5 * math.sqrt(n / 8.0) * 0.0125
        pos = deposit(rs, bound[shape_of], half, half, 0.005 + 1e-5)
        Q = random_quaternions(rs, n)
        sc = _assemble(shapes, [np.zeros(3)], [np.array([1.0, 0, 0, 0])], pos, Q, shape_of, density, "Default", kn,
                       kt, en2, mu, dt, gravity=(0.0, 0.0, -9.81), DVerlet=0.2 * bmax, dVerlet=0.1 * bmax,
                       interVerlet=100 * dt, name="slope_%d" % k)
        sc["shapes"] = shapes
        parts.append(tilt(sc, theta))
        angles.append(math.degrees(theta))
    out = batch(parts, name="slope_batch_%d" % nscenes)
    out["slope_deg"] = angles
    return out


def _assemble(shapes, wall_pos, wall_Q, pos, Q, shape_of, density, law, kn, kt, en2, mu, dt, gravity, DVerlet,
              dVerlet, interVerlet, name, wall_shape=0, homothety=None, wall_density=None):
    """Driven bodies (walls, group 1) first, then the grains (group 0).  Mass
    and inertia follow Rockable::loadConf (Rockable.cpp:918-920): mass =
    h^3 V density(group), inertia = h^2 (I/m) mass, h the homothety."""
    nd = len(wall_pos)
    n = nd + len(pos)
    shape = np.concatenate([np.broadcast_to(np.asarray(wall_shape), (nd,)), shape_of]).astype(np.int32)
    P = np.concatenate([np.array(wall_pos), pos])
    Qa = np.concatenate([np.array(wall_Q), Q])
    group = np.concatenate([np.ones(nd), np.zeros(len(pos))]).astype(np.int32)
    hom = np.ones(n)
    if homothety is not None:
        hom[nd:] = homothety
    wall_density = density if wall_density is None else wall_density
    vol = np.array([shapes[s]["volume"] for s in shape])
    mass = hom ** 3 * vol * np.where(group == 1, wall_density, density)
    im = np.array([shapes[s]["I/m"] for s in shape]) * (hom ** 2)[:, None]
    tab = law_table(kn=kn, kt=kt, en2=en2, mu=mu)
    return {"name": name, "shapes": shapes, "shape_tables": flatten_shapes(shapes), "n_driven": nd,
            "bodies": {"pos": P, "vel": np.zeros((n, 3)), "acc": np.zeros((n, 3)), "Q": Qa,
                       "vrot": np.zeros((n, 3)), "arot": np.zeros((n, 3)), "homothety": hom, "mass": mass,
                       "inertia": im * mass[:, None], "shape": shape, "group": group,
                       "cluster": np.zeros(n, np.int32)},
            "density": {0: density, 1: wall_density}, "law": law, "ngroup": 2, "table": tab, "dt": dt,
            "gravity": gravity, "DVerlet": DVerlet, "dVerlet": dVerlet, "interVerlet": interVerlet,
            "params": {"kn": kn, "kt": kt, "en2": en2, "mu": mu}}


def settle(scene, steps=4000, dt=1e-5, kn=1e4, gboost=20.0, damping=0.5, device=0, report=None, law="Avalanche",
           rebuild_every=10, relax_steps=0):
    """Compact a freshly deposited pile on the GPU: contacts of the given law
    (Avalanche by default) at a soft stiffness, boosted gravity and numerical
    damping, large time step.
    Returns the GpuScene, switched afterwards to the scene's own parameters
    (the Avalanche law's incremental normal force carries the settled contact
    forces across the change of stiffness).  With relax_steps, the pile then
    relaxes under plain gravity with the same soft contacts, which shrinks the
    overlaps before a law without force history (Default) takes over."""
    from .abi import GpuScene, RK_LAW
    g = GpuScene(device=device)
    g.upload_shapes(scene["shape_tables"])
    g.upload_bodies(scene["bodies"], scene["n_driven"])
    if scene.get("scene_of") is not None:
        g.set_scenes(scene["scene_of"])
    p = scene["params"]
    grav = tuple(gboost * x for x in scene["gravity"])
    g.set_params(t=0.0, dt=dt, gravity=grav, DVerlet=scene["DVerlet"], dVerlet=scene["dVerlet"],
                 interVerlet=rebuild_every * dt, interVerletC=0.0, law=RK_LAW[law], ngroup=scene["ngroup"],
                 table=law_table(kn=kn, kt=kn, en2=p["en2"], mu=p["mu"]), numerical_damping=damping)
    g.update_nl()
    done = 0
    while done < steps:
        k = min(500, steps - done)
        g.step(k)
        done += k
        if report is not None:
            st = g.stats()
            report.append((done, st["n_entries"], st["n_active"], st["e_trans"]))
    if relax_steps > 0:
        g.set_params(t=done * dt, dt=dt, gravity=tuple(scene["gravity"]), DVerlet=scene["DVerlet"],
                     dVerlet=scene["dVerlet"], interVerlet=rebuild_every * dt, interVerletC=0.0, law=RK_LAW[law],
                     ngroup=scene["ngroup"], table=law_table(kn=kn, kt=kn, en2=p["en2"], mu=p["mu"]),
                     numerical_damping=damping)
        g.step(relax_steps)
        done += relax_steps
    set_scene_params(g, scene, t=done * dt)
    return g


def set_scene_params(g, scene, t=0.0, numerical_damping=0.0):
    """Law, table, time step and Verlet parameters of the scene, and its
    controls and servo when it has them."""
    from .abi import RK_LAW
    g.set_params(t=t, dt=scene["dt"], gravity=scene["gravity"], DVerlet=scene["DVerlet"], dVerlet=scene["dVerlet"],
                 interVerlet=scene["interVerlet"], interVerletC=0.0, law=RK_LAW[scene["law"]],
                 ngroup=scene["ngroup"], table=scene["table"], numerical_damping=numerical_damping)
    c = scene.get("controls")
    if c is not None:
        g.set_controls(c["type"], c["body"], c["value"], c["vec"], scene.get("servo"))


def loaded(scene, steps, device=0, damping=0.5, form=1, dt_factor=1.0, rebuild_steps=1000, chunk=2000,
           report=None):
    """The scene settled by the DEM itself: `steps` DEM steps with the
    scene's laws, stiffnesses, gravity, walls and servo, a time step
    `dt_factor` times the scene's (kept well inside the contacts' and the
    grains' rotational stability limits by the caller), plus Rockable's
    numerical damping `damping` (Rockable.cpp:3814-3866), in the
    given form (the mixed form by default: the result is only an initial
    state) with a neighbour list rebuilt every `rebuild_steps` steps (the
    damped grains move far less than dVerlet in that time).  The packer's
    grains touch but carry no load and are not in rotational balance: here
    they load their contacts, topple into place and come to rest.  Then the
    walls listed in scene["walls"] are removed (the start of a collapse).
    A servo's pressure is ramped up over the first 60 % of the steps.
    The stiffnesses never change, so the contact forces carried over (with
    their history, "entries") hold the load without the damping.  Returns
    the new scene and a "load" record (steps, damping, simulated time,
    entries and active contacts per free body at the end, kinetic
    energies)."""
    from .abi import GpuScene, RK_LAW
    g = GpuScene(device=device, form=form)
    g.upload_shapes(scene["shape_tables"])
    g.upload_bodies(scene["bodies"], scene["n_driven"])
    if scene.get("scene_of") is not None:
        g.set_scenes(scene["scene_of"])
    dt = scene["dt"] * dt_factor
    g.set_params(t=0.0, dt=dt, gravity=scene["gravity"], DVerlet=scene["DVerlet"], dVerlet=scene["dVerlet"],
                 interVerlet=rebuild_steps * dt, interVerletC=0.0, law=RK_LAW[scene["law"]],
                 ngroup=scene["ngroup"], table=scene["table"], numerical_damping=damping)
    c = scene.get("controls")
    if c is not None:
        g.set_controls(c["type"], c["body"], c["value"], c["vec"], scene.get("servo"))
    if scene.get("entries") is not None:
        g.upload_entries(scene["entries"])
    else:
        g.update_nl()
    g.set_graphs(True)
    done = 0
    nfree = len(scene["bodies"]["mass"]) - scene["n_driven"]
    trace = []
    sv = scene.get("servo")
    while done < steps:
        k = min(chunk, steps - done)
        if sv is not None and c is not None:
            # the servo's pressure raised linearly over the first 60 % of the
            # steps: the full pressure on a loose, rough top layer would push
            # the walls deep into its few highest grains
            ramp = dict(sv)
            ramp["pressure"] = sv["pressure"] * min(1.0, (done + k) / (0.6 * steps))
            g.set_controls(c["type"], c["body"], c["value"], c["vec"], ramp)
        g.step(k)
        done += k
        st = g.stats()
        trace.append((done, round(st["n_active"] / max(1, nfree), 4), float("%.4g" % st["e_trans"])))
    if report is not None:
        report.extend(trace)
    g.update_nl()  # the list for the scene's own schedule, from the final positions
    st = g.stats()
    out = scene_from_gpu(scene, g)
    g.close()
    rec = {"steps": int(steps), "dt": dt, "numerical_damping": damping, "form": "mixed" if form == 1 else "fp64",
           "t": steps * dt, "active_per_free": st["n_active"] / max(1, nfree), "entries": int(st["n_entries"]),
           "e_trans": st["e_trans"], "e_rot": st["e_rot"], "trace": trace}
    if scene.get("walls"):
        out = drop_bodies(out, scene["walls"])
        rec["released_walls"] = [int(w) for w in scene["walls"]]
    out["load"] = rec
    return out


def scene_from_gpu(scene, g):
    """The scene with the bodies and the neighbour list of a running engine
    (for writing a conf that the CPU path can load)."""
    out = dict(scene)
    st = g.bodies()
    b = dict(scene["bodies"])
    for k in ["pos", "vel", "acc", "Q", "vrot", "arot"]:
        b[k] = st[k]
    out["bodies"] = b
    out["entries"] = g.entries(geometry=True)
    return out


def law_table(kn, kt, en2, mu, kr=0.0, mur=0.0, ngroup=2):
    """Parameter table in the RK_P_* slot order (include/rk_gpu.h)."""
    t = np.zeros((22, ngroup, ngroup))
    t[0] = kn
    t[1] = en2
    t[2] = kt
    t[3] = mu
    t[4] = kr
    t[5] = mur
    return t.ravel()


# -------------------------------------------------------------- conf files --
def _f(x):
    return "%.16e" % x


def write_conf(scene, directory, conf_name="input.conf", shape_name="shapes.shp", tmax=None):
    """Write the scene as a Rockable conf + shape library."""
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, shape_name), "w") as f:
        for s in scene["shapes"]:
            f.write("<\nname %s\nradius %s\npreCompDone y\nvolume %s\n" % (s["name"], _f(s["radius"]), _f(s["volume"])))
            f.write("I/m %s\n" % " ".join(_f(x) for x in s["I/m"]))
            f.write("obb.extent %s\nobb.center %s\n" % (" ".join(_f(x) for x in s["obb_extent"]),
                                                        " ".join(_f(x) for x in s["obb_center"])))
            f.write("obb.e1 1 0 0\nobb.e2 0 1 0\nobb.e3 0 0 1\nOBBtreeLevel 0\n")
            f.write("nv %d\n" % len(s["vertices"]))
            for v in s["vertices"]:
                f.write("%s\n" % " ".join(_f(x) for x in v))
            f.write("ne %d\n" % len(s["edges"]))
            for e in s["edges"]:
                f.write("%d %d\n" % (e[0], e[1]))
            f.write("nf %d\n" % len(s["faces"]))
            for fc in s["faces"]:
                f.write("%d %s\n" % (len(fc), " ".join(str(x) for x in fc)))
            f.write(">\n")
    b = scene["bodies"]
    p = scene["params"]
    dt = scene["dt"]
    lines = ["Rockable 29-11-2018", "AddOrRemoveInteractions bruteForce", "UpdateNL linkCells",
             "forceLaw %s" % scene["law"], "t 0", "tmax %s" % (tmax if tmax is not None else 1.0), "dt %r" % dt,
             "interVerlet %r" % scene["interVerlet"], "interConf 1", "DVerlet %r" % scene["DVerlet"],
             "dVerlet %r" % scene["dVerlet"]]
    for g, d in scene["density"].items():
        lines.append("density %d %r" % (g, d))
    lines.append("gravity %r %r %r" % tuple(scene["gravity"]))
    for g1 in range(2):
        for g2 in range(g1, 2):
            lines += ["knContact %d %d %r" % (g1, g2, p["kn"]), "en2Contact %d %d %r" % (g1, g2, p["en2"]),
                      "ktContact %d %d %r" % (g1, g2, p["kt"]), "muContact %d %d %r" % (g1, g2, p["mu"]),
                      "krContact %d %d 0" % (g1, g2), "murContact %d %d 0" % (g1, g2)]
    nd = scene["n_driven"]
    bound = float(np.max(np.array([scene["shapes"][k]["bound"] for k in b["shape"][nd:]]) * b["homothety"][nd:]))
    cs = 2.0 * bound + scene["DVerlet"]
    lines += list(scene.get("conf_extra", []))
    lines += ["cellMinSizes %r %r %r" % (cs, cs, cs), "nDriven %d" % scene["n_driven"],
              "shapeFile %s" % shape_name, "precision 16", "Particles %d" % len(b["mass"])]
    for i in range(len(b["mass"])):
        nm = scene["shapes"][b["shape"][i]]["name"]
        vals = list(b["pos"][i]) + list(b["vel"][i]) + list(b["acc"][i]) + list(b["Q"][i]) + list(b["vrot"][i]) + \
            list(b["arot"][i])
        lines.append("%s %d %d %s %s" % (nm, b["group"][i], b["cluster"][i], _f(b["homothety"][i]),
                                         " ".join(_f(x) for x in vals)))
    e = scene.get("entries")
    if e is None:
        lines += ["Interactions 0"]
    else:  # active entries with their history, like Rockable::saveConf
        act = np.nonzero((e["dn"] < 0.0) | (e["bond"] >= 0))[0]
        lines.append("Interactions %d" % len(act))
        for k in act:
            vals = list(e["n"][k]) + [e["dn"][k]] + list(e["pos"][k]) + list(e["vel"][k]) + [e["fn"][k]] + \
                list(e["ft"][k]) + list(e["mom"][k]) + [e["damp"][k]]
            lines.append("%d %d %d %d %d %s" % (e["i"][k], e["j"][k], e["type"][k], e["isub"][k], e["jsub"][k],
                                                " ".join(_f(x) for x in vals)))
    lines += ["Interfaces 0"] + list(scene.get("conf_tail", [])) + [""]
    with open(os.path.join(directory, conf_name), "w") as f:
        f.write("\n".join(lines))
    sv = scene.get("servo")
    if sv is not None:  # DrivingSystem::read format (DrivingSystem.cpp:188-199)
        with open(os.path.join(directory, "drivingSystem.txt"), "w") as f:
            f.write("Servo tritriIsostaticCompression %s %r\n" % (" ".join(str(int(w)) for w in sv["walls"]),
                                                                   float(sv["pressure"])))
    return os.path.join(directory, conf_name)
