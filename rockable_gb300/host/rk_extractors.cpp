// rk_extractors.cpp -- Rockable's DataExtractors (src/DataExtractors/*.cpp)
// over the host mirror of the state, which consoleRun downloads from the GPU
// engine at their cadence.  Each reads the parameters of its reference
// counterpart from dataExtractors.txt and writes the same columns to its data
// file with the stream's default formatting (the reference sets no precision
// on these files); vectors print as "x y z" and quaternions as "w x y z", as
// the reference's vec3r / quat stream operators do.
#include <cmath>
#include <iostream>
#include <limits>

#include "rk_host.hpp"

namespace rkhost {

void DataExtractor::generateHelp(std::ostream& os) {  // DataExtractor.cpp: generateHelp
  const std::string rule(90, '=');
  os << rule << '\n' << "Data File: " << filename << '\n' << docString.str() << '\n';
  for (size_t k = 0; k < columnDoc.size(); k++) os << k + 1 << ":\t" << columnDoc[k] << '\n';
  os << rule << "\n\n";
}

void Rockable::globVertex(size_t b, size_t v, double out[3]) const {
  // pos + Q (h u): t = 2 q.v x u; u + s t + q.v x t
  const Shape& sh = Shapes[P.shape[b]];
  const double h = P.homothety[b];
  const double u[3] = {h * sh.vertex[3 * v], h * sh.vertex[3 * v + 1], h * sh.vertex[3 * v + 2]};
  const double* q = &P.Q[4 * b];
  const double s = q[0], x = q[1], y = q[2], z = q[3];
  const double t[3] = {2.0 * (y * u[2] - z * u[1]), 2.0 * (z * u[0] - x * u[2]), 2.0 * (x * u[1] - y * u[0])};
  const double c[3] = {y * t[2] - z * t[1], z * t[0] - x * t[2], x * t[1] - y * t[0]};
  for (int d = 0; d < 3; d++) out[d] = P.pos[3 * b + d] + (u[d] + s * t[d] + c[d]);
}

double Rockable::minkowskiRadius(size_t b) const { return P.homothety[b] * Shapes[P.shape[b]].radius; }

bool Rockable::readDataExtractors(const std::string& path) {
  register_builtin_extractors();
  std::ifstream is(path);
  if (!is) return true;  // no file, no extractors
  std::string name;
  while (is >> name) {
    if (name[0] == '/' || name[0] == '#' || name[0] == '!') {
      std::string rest;
      std::getline(is, rest);
      continue;
    }
    DataExtractor* de = Factory<DataExtractor>::instance().create(name);
    if (!de) {
      std::cerr << "[rockable-gb300] the DataExtractor named " << name << " is unknown\n";
      continue;
    }
    de->plug(this);
    de->read(is);
    dataExtractors.emplace_back(de);
  }
  return true;
}

namespace {

void put3(std::ostream& os, const double* v) { os << v[0] << ' ' << v[1] << ' ' << v[2]; }

// the first control acting on body ib and the force components it imposes
// (TrackBody.cpp / TrackRockfall.cpp: init)
struct Imposed {
  size_t ictrl{0};
  bool f[3]{false, false, false};
  void find(const Rockable& box, int ib) {
    ictrl = 0;
    f[0] = f[1] = f[2] = false;
    for (size_t c = 0; c < box.controls.size(); c++) {
      if (box.controls[c].body != ib) continue;
      ictrl = c;
      const int ty = box.controls[c].type;
      if (ty == RK_X_FOR) f[0] = true;
      else if (ty == RK_Y_FOR) f[1] = true;
      else if (ty == RK_Z_FOR) f[2] = true;
      break;
    }
  }
  void subtract(const Rockable& box, double force[3]) const {
    for (int d = 0; d < 3; d++)
      if (f[d]) force[d] -= box.controls[ictrl].value;
  }
};

const char* const kBodyColumns[] = {"Time", "x", "y", "z", "v.x", "v.y", "v.z", "Q.w", "Q.x", "Q.y", "Q.z",
                                    "vrot.x", "vrot.y", "vrot.z", "f.x - imposedForce.x", "f.y - imposedForce.y",
                                    "f.z - imposedForce.z", "m.x", "m.y", "m.z"};

void record_body(const Rockable& box, std::ofstream& f, int ib, const Imposed& imp) {
  const Particles& P = box.P;
  double force[3] = {P.force[3 * ib], P.force[3 * ib + 1], P.force[3 * ib + 2]};
  imp.subtract(box, force);
  f << box.t << ' ';
  put3(f, &P.pos[3 * ib]);
  f << ' ';
  put3(f, &P.vel[3 * ib]);
  f << ' ' << P.Q[4 * ib] << ' ' << P.Q[4 * ib + 1] << ' ' << P.Q[4 * ib + 2] << ' ' << P.Q[4 * ib + 3] << ' ';
  put3(f, &P.vrot[3 * ib]);
  f << ' ';
  put3(f, force);
  f << ' ';
  put3(f, &P.moment[3 * ib]);
  f << std::endl << std::flush;
}

// TrackBody: ibody filename nrec -- one body's kinematics and resultant
// (with a GPU context: that body's fields only, rk_download_body)
class TrackBody : public DataExtractor {
  int ibody{0};
  Imposed imp;

 public:
  void read(std::istream& is) override {
    is >> ibody >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << "ibody = " << ibody << ", nrec = " << nrec;
    columnDoc.assign(std::begin(kBodyColumns), std::end(kBodyColumns));
  }
  void init() override { imp.find(*box, ibody); }
  bool onDevice() const override { return box && box->ctx(); }
  void record() override {
    if (!onDevice()) {
      record_body(*box, recordFile, ibody, imp);
      return;
    }
    double o[25];
    if (rk_download_body(box->ctx(), ibody, o) != RK_OK) return;
    double force[3] = {o[19], o[20], o[21]};
    imp.subtract(*box, force);
    recordFile << box->t << ' ';
    put3(recordFile, o);
    recordFile << ' ';
    put3(recordFile, o + 3);
    recordFile << ' ' << o[9] << ' ' << o[10] << ' ' << o[11] << ' ' << o[12] << ' ';
    put3(recordFile, o + 13);
    recordFile << ' ';
    put3(recordFile, force);
    recordFile << ' ';
    put3(recordFile, o + 22);
    recordFile << std::endl << std::flush;
  }
};

// MeanVelocity: filename nrec -- mean speed over all bodies
class MeanVelocity : public DataExtractor {
 public:
  void read(std::istream& is) override {
    is >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << " nrec = " << nrec;
  }
  bool onDevice() const override { return box && box->ctx(); }
  void record() override {
    double m = 0.0;
    if (onDevice()) {
      if (rk_extract_mean_velocity(box->ctx(), &m) != RK_OK) return;
    } else {
      const Particles& P = box->P;
      for (size_t b = 0; b < P.size(); b++) {
        const double* v = &P.vel[3 * b];
        m += std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      }
      m /= (double)P.size();
    }
    recordFile << box->t << ' ' << m << std::endl << std::flush;
  }
};

// dnStat: filename nrec -- statistics of dn over the active entries and the
// contact point of the smallest
class DnStat : public DataExtractor {
 public:
  void read(std::istream& is) override {
    is >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << "nrec = " << nrec;
    columnDoc = {"Time",    "dnMin", "dnMax",          "dnMean",         "dnMeanNeg",     "dnMeanPos",
                 "nbNeg",   "nbPos", "pos.x of dnMin", "pos.y of dnMin", "pos.z of dnMin"};
  }
  bool needsGeometry() const override { return true; }
  bool onDevice() const override { return box && box->ctx(); }
  void record() override {
    const Interactions& I = box->I;
    double mn = 1e20, mx = -1e20, meanNeg = 0.0, meanPos = 0.0, nNeg = 0.0, nPos = 0.0, mean = 0.0;
    double pmin[3] = {0.0, 0.0, 0.0};
    if (onDevice()) {
      double o[10];
      if (rk_extract_dn_stat(box->ctx(), o) != RK_OK) return;
      recordFile << box->t << ' ' << o[0] << ' ' << o[1] << ' ' << o[2] << ' ' << o[3] << ' ' << o[4] << ' '
                 << (int)o[5] << ' ' << (int)o[6] << ' ';
      put3(recordFile, o + 7);
      recordFile << std::endl << std::flush;
      return;
    }
    for (size_t e = 0; e < I.size(); e++) {
      if (!I.active[e]) continue;
      const double dn = I.dn[e];
      mean += dn;
      if (dn < 0.0) {
        meanNeg += dn;
        nNeg += 1.0;
      } else {
        meanPos += dn;
        nPos += 1.0;
      }
      if (dn < mn) {
        mn = dn;
        for (int d = 0; d < 3; d++) pmin[d] = I.pos[3 * e + d];
      }
      if (dn > mx) mx = dn;
    }
    if (nNeg > 0.0) meanNeg /= nNeg;
    if (nPos > 0.0) meanPos /= nPos;
    if (nNeg > 0.0 || nPos > 0.0) mean /= (nNeg + nPos);
    recordFile << box->t << ' ' << mn << ' ' << mx << ' ' << mean << ' ' << meanNeg << ' ' << meanPos << ' '
               << (int)nNeg << ' ' << (int)nPos << ' ';
    put3(recordFile, pmin);
    recordFile << std::endl << std::flush;
  }
};

// axis-aligned box of points enlarged by r, grown by union
struct Box3 {
  double lo[3], hi[3];
  bool set{false};
  void add(const double p[3], double r) {
    for (int d = 0; d < 3; d++) {
      const double a = p[d] - r, b = p[d] + r;
      if (!set || a < lo[d]) lo[d] = a;
      if (!set || b > hi[d]) hi[d] = b;
    }
    set = true;
  }
  bool contains(const double p[3]) const {
    for (int d = 0; d < 3; d++)
      if (p[d] < lo[d] || p[d] > hi[d]) return false;
    return true;
  }
};

// ClusterAABB: icluster filename nrec -- box of the bodies of one cluster
// (their vertices enlarged by the rounding radius)
class ClusterAABB : public DataExtractor {
  int icluster{0};

 public:
  void read(std::istream& is) override {
    is >> icluster >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << "icluster = " << icluster << ", nrec = " << nrec;
    columnDoc = {"Time", "aabb.min.x", "aabb.min.y", "aabb.min.z", "aabb.max.x", "aabb.max.y", "aabb.max.z"};
  }
  bool onDevice() const override { return box && box->ctx(); }
  void record() override {
    if (onDevice()) {
      double o[7];
      if (rk_extract_cluster_aabb(box->ctx(), icluster, o) != RK_OK) return;
      recordFile << box->t << ' ';
      put3(recordFile, o + 1);
      recordFile << ' ';
      put3(recordFile, o + 4);
      recordFile << std::endl << std::flush;
      return;
    }
    const Particles& P = box->P;
    Box3 bx;
    for (size_t b = 0; b < P.size(); b++) {
      if (P.cluster[b] != icluster) continue;
      const double r = box->minkowskiRadius(b);
      const size_t nv = box->Shapes[P.shape[b]].vertex.size() / 3;
      for (size_t v = 0; v < nv; v++) {
        double g[3];
        box->globVertex(b, v, g);
        bx.add(g, r);
      }
    }
    recordFile << box->t << ' ';
    // the reference starts from a default (zero) box when the cluster is empty
    const double zero[3] = {0.0, 0.0, 0.0};
    put3(recordFile, bx.set ? bx.lo : zero);
    recordFile << ' ';
    put3(recordFile, bx.set ? bx.hi : zero);
    recordFile << std::endl << std::flush;
  }
};

// DuoBalance: i j filename nrec -- sub-contacts in contact (dn < 0) between
// two bodies, by type
class DuoBalance : public DataExtractor {
  int bi{0}, bj{0};

 public:
  void read(std::istream& is) override {
    is >> bi >> bj >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << "first particle = " << bi << ", second particle = " << bj << ", nrec = " << nrec;
    columnDoc = {"Time", "nvv", "nve", "nvf", "nee", "(nvv + nve + nvf + nee) x weight"};
  }
  bool onDevice() const override { return box && box->ctx(); }
  void record() override {
    const Interactions& I = box->I;
    size_t n[4] = {0, 0, 0, 0};
    if (onDevice()) {
      int64_t d[4];
      if (rk_extract_duo_balance(box->ctx(), bi, bj, d) != RK_OK) return;
      for (int k = 0; k < 4; k++) n[k] = (size_t)d[k];
    } else {
      for (size_t e = 0; e < I.size(); e++) {
        const bool pair = (I.i[e] == bi && I.j[e] == bj) || (I.i[e] == bj && I.j[e] == bi);
        if (pair && I.dn[e] < 0.0 && I.type[e] >= 0 && I.type[e] < 4) n[I.type[e]]++;
      }
    }
    // no contact-partnership weights on this engine (ContactPartnership None)
    recordFile << box->t << "   " << n[0] << ' ' << n[1] << ' ' << n[2] << ' ' << n[3] << "\n" << '\n' << std::flush;
  }
};

// TrackRockfall: ibody vStop wStop filename nrec -- TrackBody's columns, and
// a stop request when the body has come to rest (after vStop / 9.81 s) or
// has left the box of the driven bodies
class TrackRockfall : public DataExtractor {
  int ibody{0};
  double vStop{0.0}, wStop{0.0}, tminStop{0.0};
  Imposed imp;
  Box3 aabb;

 public:
  void read(std::istream& is) override {
    is >> ibody >> vStop >> wStop >> filename >> nrec;
    recordFile.open(filename);
    nstep = std::numeric_limits<int>::max();
    docString << "ibody = " << ibody << ", nrec = " << nrec;
    columnDoc.assign(std::begin(kBodyColumns), std::end(kBodyColumns));
  }
  void init() override {
    imp.find(*box, ibody);
    tminStop = vStop / 9.81;
    // Rockable::computeAABB(0, nDriven - 1) (Rockable.cpp:3925-3948): the
    // driven bodies' boxes; a last index of 0 means every body
    const Particles& P = box->P;
    size_t last = box->nDriven > 0 ? box->nDriven - 1 : 0;
    if (last == 0) last = P.size() - 1;
    aabb = Box3();
    for (size_t b = 0; b <= last && b < P.size(); b++) {
      const double r = box->minkowskiRadius(b);
      const size_t nv = box->Shapes[P.shape[b]].vertex.size() / 3;
      Box3 one;
      for (size_t v = 0; v < nv; v++) {
        double g[3];
        box->globVertex(b, v, g);
        one.add(g, 0.0);
      }
      for (int d = 0; d < 3; d++) {
        one.lo[d] -= r;
        one.hi[d] += r;
      }
      aabb.add(one.lo, 0.0);
      aabb.add(one.hi, 0.0);
    }
  }
  void record() override {
    record_body(*box, recordFile, ibody, imp);
    const double* v = &box->P.vel[3 * ibody];
    const double* w = &box->P.vrot[3 * ibody];
    const double vsqr = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double wsqr = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    if (box->t > tminStop && vsqr < vStop * vStop && wsqr < wStop * wStop) {
      std::cout << "t = " << box->t << "\ntminStop = " << tminStop << "\nvel = " << std::sqrt(vsqr)
                << "\nvStop = " << vStop << "\nvrot = " << std::sqrt(wsqr) << "\nwStop = " << wStop << '\n';
      box->computationStopAsked = 1;
    }
    if (!aabb.contains(&box->P.pos[3 * ibody])) {
      std::cout << "out of box!!\n";
      box->computationStopAsked = 1;
    }
  }
};

}  // namespace

void register_builtin_extractors() {
  static bool done = false;
  if (done) return;
  done = true;
  auto& f = Factory<DataExtractor>::instance();
  f.add("TrackBody", [] { return new TrackBody(); });
  f.add("MeanVelocity", [] { return new MeanVelocity(); });
  f.add("dnStat", [] { return new DnStat(); });
  f.add("ClusterAABB", [] { return new ClusterAABB(); });
  f.add("DuoBalance", [] { return new DuoBalance(); });
  f.add("TrackRockfall", [] { return new TrackRockfall(); });
}

}  // namespace rkhost
