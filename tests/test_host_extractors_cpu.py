"""The host's DataExtractors (rockable_gb300/host/rk_extractors.cpp) on a hand-
filled host mirror, without a GPU: a C++ harness links librk_host.so, reads a
dataExtractors.txt like Rockable::readDataExtractors, records once, and the
data files are checked against values computed here (the reference's columns,
default stream formatting)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r'''
#include <cstdio>
#include <fstream>
#include <iostream>
#include "rk_host.hpp"
using namespace rkhost;
int main(int argc, char** argv) {
  Rockable box;
  Shape cube;
  cube.name = "cube";
  cube.radius = 1e-4;
  for (int k = 0; k < 8; k++)
    for (int d = 0; d < 3; d++) cube.vertex.push_back(((k >> d) & 1) ? 0.5e-3 : -0.5e-3);
  box.Shapes.push_back(cube);
  Particles& P = box.P;
  const int n = 3;
  P.shape.assign(n, 0); P.group.assign(n, 0); P.cluster = {0, 1, 1}; P.homothety = {1.0, 1.0, 2.0};
  P.mass.assign(n, 1.0); P.inertia.assign(3 * n, 1.0);
  P.pos = {0, 0, 0, 0.01, 0.02, 0.03, 0.013, 0.02, 0.031};
  P.vel = {0, 0, 0, 0.1, -0.2, 0.3, 0.004, 0.005, -0.006};
  P.acc.assign(3 * n, 0.0);
  const double c = 0.8775825618903728, s = 0.479425538604203;  // rotation of 1 rad about z
  P.Q = {1, 0, 0, 0, c, 0, 0, s, 1, 0, 0, 0};
  P.vrot = {0, 0, 0, 1.5, 0, -2.5, 0.001, 0.002, 0.003};
  P.arot.assign(3 * n, 0.0);
  P.force = {0, 0, 0, 0.75, -0.5, 9.25, 0, 0, 0};
  P.moment = {0, 0, 0, 1e-5, 2e-5, -3e-5, 0, 0, 0};
  box.nDriven = 1;
  box.t = 0.5;
  rk_control ctl{};
  ctl.type = RK_X_FOR; ctl.body = 1; ctl.value = 0.25;
  box.controls.push_back(ctl);
  Interactions& I = box.I;
  // (i, j, type, dn, active, pos)
  const double e[][8] = {{1, 2, 0, -1e-6, 1, 0.011, 0.02, 0.03}, {1, 2, 2, -3e-6, 1, 0.012, 0.021, 0.031},
                         {2, 1, 1, -2e-6, 1, 0.0115, 0.02, 0.03}, {1, 2, 3, 5e-6, 0, 0, 0, 0},
                         {0, 1, 2, -4e-7, 1, 0.01, 0.02, 0.0295}, {1, 2, 3, -5e-7, 1, 0.0118, 0.0205, 0.0302}};
  for (auto& r : e) {
    I.i.push_back((int)r[0]); I.j.push_back((int)r[1]); I.type.push_back((int)r[2]); I.isub.push_back(0);
    I.jsub.push_back(0); I.bond.push_back(-1); I.dn.push_back(r[3]); I.active.push_back((uint8_t)r[4]);
    for (int d = 0; d < 3; d++) I.pos.push_back(r[5 + d]);
    I.fn.push_back(0); I.damp.push_back(0);
    for (int d = 0; d < 3; d++) { I.ft.push_back(0); I.mom.push_back(0); I.n.push_back(0); I.vel.push_back(0); }
  }
  box.readDataExtractors(argv[1]);
  std::ofstream doc("extractedDataDoc.txt");
  for (auto& de : box.dataExtractors) { de->generateHelp(doc); de->init(); }
  for (auto& de : box.dataExtractors) de->record();
  for (auto& de : box.dataExtractors) { de->end(); de->recordFile.close(); }
  printf("extractors %zu stop %d\n", box.dataExtractors.size(), box.computationStopAsked);
  return 0;
}
'''

EXTRACTORS = """TrackBody 1 track.txt 10
MeanVelocity mean.txt 20
# a comment line
dnStat dn.txt 10
ClusterAABB 1 aabb.txt 10
DuoBalance 1 2 duo.txt 10
TrackRockfall 2 0.01 0.01 rock.txt 10
NoSuchExtractor
"""


def g(x):
    return "%g" % x


def qrot(q, u):
    s, v = q[0], np.asarray(q[1:])
    t = 2.0 * np.cross(v, u)
    return u + s * t + np.cross(v, t)


@pytest.fixture(scope="module")
def run(tmp_path_factory, gpu_lib):
    lib = os.path.join(ROOT, "rockable_gb300", "_lib")
    d = tmp_path_factory.mktemp("extractors")
    (d / "h.cpp").write_text(HARNESS)
    exe = str(d / "h")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "rockable_gb300", "host"),
                           str(d / "h.cpp"), "-o", exe, "-L" + lib, "-lrk_host", "-lrk_gpu",
                           "-Wl,-rpath," + lib])
    (d / "dataExtractors.txt").write_text(EXTRACTORS)
    p = subprocess.run([exe, "dataExtractors.txt"], cwd=str(d), capture_output=True, text=True, timeout=60)
    assert p.returncode == 0, p.stderr
    return d, p


def test_extractors_read_and_report_unknown(run):
    d, p = run
    assert "extractors 6" in p.stdout
    assert "NoSuchExtractor is unknown" in p.stderr
    doc = (d / "extractedDataDoc.txt").read_text()
    assert doc.count("Data File: ") == 6 and "1:\tTime" in doc and "ibody = 1, nrec = 10" in doc


def test_track_body_subtracts_the_imposed_force(run):
    d, _ = run
    want = ["0.5", "0.01", "0.02", "0.03", "0.1", "-0.2", "0.3", g(0.8775825618903728), "0", "0",
            g(0.479425538604203), "1.5", "0", "-2.5", g(0.75 - 0.25), "-0.5", "9.25", "1e-05", "2e-05", "-3e-05"]
    assert (d / "track.txt").read_text().split() == want


def test_mean_velocity_and_dn_stat(run):
    d, _ = run
    v = np.array([[0, 0, 0], [0.1, -0.2, 0.3], [0.004, 0.005, -0.006]])
    assert (d / "mean.txt").read_text().split() == ["0.5", g(np.linalg.norm(v, axis=1).mean())]
    dns = [-1e-6, -3e-6, -2e-6, -4e-7, -5e-7]  # the active entries
    want = ["0.5", g(min(dns)), g(max(dns)), g(np.mean(dns)), g(np.mean(dns)), "0", "5", "0", "0.012", "0.021", "0.031"]
    assert (d / "dn.txt").read_text().split() == want


def test_cluster_box_and_duo_balance(run):
    d, _ = run
    cube = np.array([[0.5e-3 if (k >> a) & 1 else -0.5e-3 for a in range(3)] for k in range(8)])
    pos = [np.array([0.01, 0.02, 0.03]), np.array([0.013, 0.02, 0.031])]
    Q = [np.array([0.8775825618903728, 0, 0, 0.479425538604203]), np.array([1.0, 0, 0, 0])]
    h = [1.0, 2.0]
    pts, rad = [], []
    for b in range(2):
        for u in cube:
            pts.append(pos[b] + qrot(Q[b], h[b] * u))
            rad.append(h[b] * 1e-4)
    pts, rad = np.array(pts), np.array(rad)[:, None]
    lo, hi = (pts - rad).min(0), (pts + rad).max(0)
    got = [float(x) for x in (d / "aabb.txt").read_text().split()]
    assert got[0] == 0.5
    np.testing.assert_allclose(got[1:], list(lo) + list(hi), rtol=1e-5)
    # bodies 1 and 2, dn < 0: one VV, one VE (stored as 2 -> 1), one VF, one EE (the other EE is separated)
    assert (d / "duo.txt").read_text() == "0.5   1 1 1 1\n\n"


def test_track_rockfall_records_and_asks_to_stop(run):
    d, p = run
    cols = (d / "rock.txt").read_text().split()
    assert cols[:7] == ["0.5", "0.013", "0.02", "0.031", "0.004", "0.005", "-0.006"] and len(cols) == 20
    # at rest (|v| < 0.01, |w| < 0.01 after 0.01 / 9.81 s); with one driven body the reference's
    # computeAABB(0, nDriven - 1) gets the last index 0, which means every body
    # (Rockable.cpp:3926-3928), so the body is inside the box
    assert "stop 1" in p.stdout and "vel = " in p.stdout and "out of box!!" not in p.stdout
