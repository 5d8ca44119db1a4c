"""Data extractors on the device (src/DataExtractors/*.cpp) against a numpy
restatement of each reference record() over the downloaded state: a bonded
rockfall (clusters, bonds, contacts) stepped in both forms.  Extremes,
counts, the picked contact point, the cluster box (vertices placed with the
host's operations) and the tracked body are bit-identical; the means are
tree sums, checked to 1e-12 of their scale."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _glob_vertices(sc, pos, Q, b):
    # Particle::GlobVertex: pos + Q (h v), t = 2 q.v x v; v + s t + q.v x t
    st = sc["shape_tables"]
    shp = sc["bodies"]["shape"][b]
    v0, v1 = st["vert_ofs"][shp], st["vert_ofs"][shp + 1]
    u = sc["bodies"]["homothety"][b] * np.asarray(st["vertices"], dtype=np.float64).reshape(-1, 3)[v0:v1]
    s, x, y, z = Q[b]
    t = np.stack([2.0 * (y * u[:, 2] - z * u[:, 1]), 2.0 * (z * u[:, 0] - x * u[:, 2]),
                  2.0 * (x * u[:, 1] - y * u[:, 0])], axis=1)
    c = np.stack([y * t[:, 2] - z * t[:, 1], z * t[:, 0] - x * t[:, 2], x * t[:, 1] - y * t[:, 0]], axis=1)
    return pos[b] + ((u + s * t) + c)


@pytest.mark.parametrize("form", [0, 1])
def test_device_extractors_match_a_serial_restatement(gpu_lib, tmp_path, form):
    from rockable_gb300 import scenes
    from rockable_gb300.abi import HostScene
    sc = scenes.rockfall_bonded(nclusters=6, per=200, target_bonds=15000)
    conf = scenes.write_conf(sc, str(tmp_path))
    h = HostScene(conf)
    g = h.gpu
    g.set_form(form)
    g.update_nl()
    g.step(300)
    g.set_record_geometry(True)
    g.step(1)
    g.set_record_geometry(False)
    B = g.bodies()
    E = g.entries(geometry=True)

    # MeanVelocity
    speed = np.sqrt(np.sum(B["vel"] ** 2, axis=1))
    ref = np.sum(speed) / len(speed)
    assert abs(g.mean_velocity() - ref) <= 1e-12 * max(abs(ref), 1e-30)

    # dnStat over dn < 0 or bonded, in entry (key) order
    act = (E["dn"] < 0.0) | (E["bond"] >= 0)
    assert act.sum() > 100
    dn = E["dn"][act]
    d = g.dn_stat()
    neg, pos = dn < 0.0, ~(dn < 0.0)
    assert d["dnMin"] == dn.min() and d["dnMax"] == dn.max()
    assert d["nbNeg"] == int(neg.sum()) and d["nbPos"] == int(pos.sum())
    scale = np.abs(dn).max()
    assert abs(d["dnMean"] - dn.mean()) <= 1e-12 * scale
    assert abs(d["dnMeanNeg"] - dn[neg].mean()) <= 1e-12 * scale
    if pos.any():
        assert abs(d["dnMeanPos"] - dn[pos].mean()) <= 1e-12 * scale
    first = np.flatnonzero(act)[np.argmin(dn)]  # argmin: the first of equal minima
    assert np.array_equal(d["pos"], E["pos"][first])

    # ClusterAABB: every cluster, and one that has no body (the zero box)
    clusters = np.asarray(sc["bodies"]["cluster"])
    rad = np.asarray(sc["bodies"]["homothety"]) * np.asarray(sc["shape_tables"]["radius"])[sc["bodies"]["shape"]]
    for cl in sorted(set(clusters.tolist()))[:4] + [int(clusters.max()) + 7]:
        lo, hi = np.full(3, np.inf), np.full(3, -np.inf)
        for b in np.flatnonzero(clusters == cl):
            gv = _glob_vertices(sc, B["pos"], B["Q"], b)
            lo = np.minimum(lo, (gv - rad[b]).min(axis=0))
            hi = np.maximum(hi, (gv + rad[b]).max(axis=0))
        if not np.isfinite(lo).all():
            lo, hi = np.zeros(3), np.zeros(3)
        dlo, dhi = g.cluster_aabb(cl)
        assert np.array_equal(dlo, lo) and np.array_equal(dhi, hi), (cl, dlo - lo, dhi - hi)

    # DuoBalance: the pair with the most touching sub-contacts, and a pair with none
    touching = E["dn"] < 0.0
    pairs = np.minimum(E["i"], E["j"]).astype(np.int64) * (1 << 21) + np.maximum(E["i"], E["j"])
    u, cnt = np.unique(pairs[touching], return_counts=True)
    pi, pj = divmod(int(u[np.argmax(cnt)]), 1 << 21)
    for (a, b) in [(pi, pj), (pj, pi), (0, 0)]:
        sel = touching & (((E["i"] == a) & (E["j"] == b)) | ((E["i"] == b) & (E["j"] == a)))
        want = np.bincount(E["type"][sel], minlength=4)[:4]
        assert np.array_equal(g.duo_balance(a, b), want)

    # TrackBody: the fields of a body, as the full download has them
    for b in [0, 1, len(B["pos"]) // 2, len(B["pos"]) - 1]:
        r = g.body(b)
        for k in ["pos", "vel", "acc", "Q", "vrot", "arot", "force", "moment"]:
            assert np.array_equal(r[k], B[k][b]), (b, k)
    h.close()


def test_host_runner_records_the_device_extractors_like_its_conf(golden_dir, gpu_lib, tmp_path):
    """The C++ runner with a dataExtractors.txt: MeanVelocity, dnStat,
    DuoBalance and TrackBody now reduce on the device; their lines at the
    time of the last conf file agree with that conf's Particles and
    Interactions sections (the data files print 6 significant digits)."""
    import os
    import subprocess
    from conftest import CONF, ROOT
    d = golden_dir / "512_particles"
    conf_in = (d / CONF["512_particles"]).read_text()
    ls = conf_in.split("\nInteractions ")[1].splitlines()
    rows = [l.split() for l in ls[1:] if not l.startswith("#")][:int(ls[0].split()[0])]
    touching = [(int(r[0]), int(r[1])) for r in rows if len(r) > 8 and float(r[8]) < 0.0]
    pi, pj = max(set(touching), key=touching.count)
    (tmp_path / "dataExtractors.txt").write_text(
        "MeanVelocity mv.txt 1\ndnStat dn.txt 1\nDuoBalance %d %d duo.txt 1\nTrackBody 10 tb.txt 1\n" % (pi, pj))
    for f in os.listdir(d):
        if not f.endswith(".conf"):
            (tmp_path / f).write_bytes((d / f).read_bytes())
    cli = os.path.join(ROOT, "rockable_gb300", "_lib", "rockable-gb300")
    (tmp_path / "out").mkdir()
    r = subprocess.run([cli, str(d / CONF["512_particles"]), "-o", str(tmp_path / "out")], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    outs = sorted((p for p in (tmp_path / "out").iterdir() if p.name.startswith("conf")),
                  key=lambda p: int(p.name[4:]))
    last = outs[-1].read_text()
    t = [l.split()[1] for l in last.splitlines() if l.startswith("t ")][0]
    key = "%g" % float(t)

    def line(name):
        ls = [l.split() for l in (tmp_path / name).read_text().splitlines() if l.strip()]
        hit = [l for l in ls if l[0] == key]
        assert hit, (name, key, ls[-3:])
        return [float(x) for x in hit[-1][1:]]

    def section(text, name):  # the N lines of a conf section "name N" (after its column header, if any)
        ls = text.split("\n" + name + " ")[1].splitlines()
        n = int(ls[0].split()[0])
        body = [l for l in ls[1:] if not l.startswith("#")]
        return [l.split() for l in body[:n]]

    P = section(last, "Particles")
    vel = np.array([[float(x) for x in p[7:10]] for p in P])
    mv = line("mv.txt")[0]
    ref = np.mean(np.sqrt(np.sum(vel ** 2, axis=1)))
    assert abs(mv - ref) <= 1e-5 * abs(ref), (mv, ref)
    I = section(last, "Interactions")
    dn = np.array([float(x[8]) for x in I])
    ds = line("dn.txt")
    assert abs(ds[0] - dn.min()) <= 1e-5 * abs(dn.min()) and int(ds[5]) == int(np.sum(dn < 0.0))
    duo = [0, 0, 0, 0]
    for x in I:
        if float(x[8]) < 0.0 and {int(x[0]), int(x[1])} == {pi, pj}:
            duo[int(x[2])] += 1
    assert [int(v) for v in line("duo.txt")[:4]] == duo
    tb = line("tb.txt")
    p10 = np.array([float(x) for x in P[10][4:7]])
    assert np.allclose(tb[0:3], p10, rtol=1e-5, atol=1e-12)
