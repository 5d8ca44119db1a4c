// rk_host.cpp -- Rockable's host side around the GB300 engine (see rk_host.hpp).
#include "rk_host.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <set>
#include <sstream>

namespace rkhost {

static const char* kParamNames[RK_NPARAM] = {
    "knContact", "en2Contact", "ktContact", "muContact", "krContact", "murContact",
    "knInnerBond", "ktInnerBond", "krInnerBond", "en2InnerBond", "fn0InnerBond", "ft0InnerBond", "mom0InnerBond",
    "powInnerBond", "knOuterBond", "ktOuterBond", "krOuterBond", "en2OuterBond", "fn0OuterBond", "ft0OuterBond",
    "mom0OuterBond", "powOuterBond"};

// ------------------------------------------------------------ force laws ----
// The three laws of the hot path; their arithmetic runs in the narrow-phase
// kernel (rockable_gb300/csrc/rk_step.cu).  init() registers the parameter
// names like ForceLaw_*.cpp init() do.
namespace {
struct LawDefault : ForceLaw {
  void init() override {
    for (const char* n : {"knContact", "en2Contact", "ktContact", "muContact", "krContact", "murContact"})
      box->dataTable[n];
  }
  int device_law() const override { return RK_LAW_DEFAULT; }
};
struct LawAvalanche : LawDefault {
  int device_law() const override { return RK_LAW_AVALANCHE; }
};
struct LawStickedLinks : LawDefault {
  void init() override {
    LawDefault::init();
    for (int k = 6; k < RK_NPARAM; k++) box->dataTable[kParamNames[k]];
  }
  int device_law() const override { return RK_LAW_STICKEDLINKS; }
};
}  // namespace

// ----------------------------------------------------------- body forces ----
// The three BodyForce plugins: read() and write() like the reference's, the
// force itself computed by the GPU step (rk_body.cuh body_force);
// getForceAndMoment() gives the same values on the host state.
namespace {
void normalize3(double v[3]) {  // toofus vec3::normalize: times the inverse norm
  double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (n > 0.0) {
    double inv = 1.0 / n;
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
  }
}
void qrot3(const double* q, const double* u, double* r) {  // body to global frame: u + s t + v x t, t = 2 v x u
  const double s = q[0], vx = q[1], vy = q[2], vz = q[3];
  double t[3] = {2.0 * (vy * u[2] - vz * u[1]), 2.0 * (vz * u[0] - vx * u[2]), 2.0 * (vx * u[1] - vy * u[0])};
  r[0] = u[0] + s * t[0] + (vy * t[2] - vz * t[1]);
  r[1] = u[1] + s * t[1] + (vz * t[0] - vx * t[2]);
  r[2] = u[2] + s * t[2] + (vx * t[1] - vy * t[0]);
}

struct AttractingPoint : BodyForce {  // BodyForce_AttractingPoint.cpp:43-59
  double point[3]{0, 0, 0}, acceleration{0.0};
  void read(std::istream& is) override { is >> point[0] >> point[1] >> point[2] >> acceleration; }
  void write(std::ostream& os) override {
    os << "AttractingPoint " << point[0] << " " << point[1] << " " << point[2] << ' ' << acceleration << '\n';
  }
  void getForceAndMoment(size_t b, double force[3], double moment[3]) override {
    (void)moment;
    const double* p = &box->P.pos[3 * b];
    double d[3] = {point[0] - p[0], point[1] - p[1], point[2] - p[2]};
    double l2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (l2 > 0.0) {
      double inv = 1.0 / std::sqrt(l2);
      double ma = box->P.mass[b] * acceleration;
      for (int k = 0; k < 3; k++) force[k] = ma * (d[k] * inv);
    }
  }
  int device_body_force(std::vector<double>& p) const override {
    p = {point[0], point[1], point[2], acceleration};
    return RK_BF_ATTRACTING_POINT;
  }
};

struct PreferredDirection : BodyForce {  // BodyForce_PreferredDirection.cpp:43-80
  double raw[7]{0, 0, 0, 0, 0, 0, 0};  // as read: axisBody, axis, momentMax
  double axisBody[3]{0, 0, 0}, axis[3]{0, 0, 0}, momentMax{0.0}, Kr{0.0};
  void read(std::istream& is) override {
    for (double& v : raw) is >> v;
    for (int k = 0; k < 3; k++) {
      axisBody[k] = raw[k];
      axis[k] = raw[3 + k];
    }
    momentMax = raw[6];
    normalize3(axisBody);
    normalize3(axis);
    Kr = 2.0 * momentMax / M_PI;
  }
  void write(std::ostream& os) override {
    os << "PreferredDirection " << axisBody[0] << " " << axisBody[1] << " " << axisBody[2] << ' ' << axis[0] << " "
       << axis[1] << " " << axis[2] << ' ' << momentMax << '\n';
  }
  void getForceAndMoment(size_t b, double force[3], double moment[3]) override {
    (void)force;
    double a[3];
    qrot3(&box->P.Q[4 * b], axisBody, a);
    normalize3(a);
    double u[3] = {axis[1] * a[2] - axis[2] * a[1], axis[2] * a[0] - axis[0] * a[2], axis[0] * a[1] - axis[1] * a[0]};
    normalize3(u);
    double cosa = a[0] * axis[0] + a[1] * axis[1] + a[2] * axis[2];
    double angle = std::acos(cosa), sgn = -1.0;
    if (cosa < 0.0) {
      sgn = 1.0;
      angle = M_PI - angle;
    }
    for (int k = 0; k < 3; k++) moment[k] = ((Kr * sgn) * u[k]) * angle;
  }
  int device_body_force(std::vector<double>& p) const override {
    p.assign(raw, raw + 7);
    return RK_BF_PREFERRED_DIRECTION;
  }
};

struct ViscousFluid : BodyForce {  // BodyForce_ViscousFluid.cpp:42-58
  double fluidDensity{0.0};
  void read(std::istream& is) override { is >> fluidDensity; }
  void write(std::ostream& os) override { os << "ViscousFluid " << fluidDensity << '\n'; }
  void getForceAndMoment(size_t b, double force[3], double moment[3]) override {
    (void)moment;
    const double* v = &box->P.vel[3 * b];
    double h = box->P.homothety[b];
    double vol = box->Shapes[box->P.shape[b]].volume * h * h * h;
    double c = (0.5 * 0.47) * fluidDensity * std::pow(vol, 2.0 / 3.0);
    for (int k = 0; k < 3; k++) force[k] = c * (v[k] * v[k]);
  }
  int device_body_force(std::vector<double>& p) const override {
    p = {fluidDensity};
    return RK_BF_VISCOUS_FLUID;
  }
};
}  // namespace

void register_builtin_plugins() {
  static bool done = false;
  if (done) return;
  done = true;
  auto& f = Factory<ForceLaw>::instance();
  f.add("Default", [] { return new LawDefault(); });
  f.add("Avalanche", [] { return new LawAvalanche(); });
  f.add("StickedLinks", [] { return new LawStickedLinks(); });
  auto& b = Factory<BodyForce>::instance();
  b.add("AttractingPoint", [] { return new AttractingPoint(); });
  b.add("PreferredDirection", [] { return new PreferredDirection(); });
  b.add("ViscousFluid", [] { return new ViscousFluid(); });
}

// ------------------------------------------------------------- Rockable ----
Rockable::Rockable() {  // Rockable.cpp:78-127
  register_builtin_plugins();
  optionNames["forceLaw"] = "Default";
  optionNames["AddOrRemoveInteractions"] = "bruteForce";
  optionNames["UpdateNL"] = "bruteForce";
  optionNames["Integrator"] = "velocityVerlet";
  for (const char* n : kParamNames) dataTable[n];
  dataTable["viscTContact"];
  dataTable["gcInnerBond"];
  dataTable["gcOuterBond"];
  forceLaw.reset(Factory<ForceLaw>::instance().create("Default"));
  forceLaw->plug(this);
  forceLaw->init();
}

Rockable::~Rockable() {
  if (ctx_) rk_destroy(ctx_);
}

double Rockable::dataTableGet(const std::string& name, int g1, int g2) const {
  auto it = dataTable.find(name);
  if (it == dataTable.end()) return 0.0;
  auto jt = it->second.find({g1, g2});
  return jt == it->second.end() ? 0.0 : jt->second;
}
void Rockable::dataTableSet(const std::string& name, int g1, int g2, double v) {
  dataTable[name][{g1, g2}] = v;
  dataTable[name][{g2, g1}] = v;
}

bool Rockable::ck(int rc, const char* what) {
  if (rc == RK_OK) return true;
  err_ = std::string(what) + ": " + (ctx_ ? rk_last_error(ctx_) : "no context") + " (code " + std::to_string(rc) + ")";
  return false;
}

static std::string dirname_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string() : p.substr(0, k + 1);
}

static bool read3(std::istream& is, double* v) { return (bool)(is >> v[0] >> v[1] >> v[2]); }

bool Rockable::loadShapes(const std::string& fname) {  // Rockable.cpp:1187-1225, Shape.cpp:69-128
  std::ifstream is(fname);
  if (!is) return fail("cannot open shape library " + fname);
  Shapes.clear();
  shapeId.clear();
  std::string tok;
  while (is >> tok) {
    if (tok != "<") continue;
    Shape s;
    while (is >> tok && tok != ">") {
      if (tok == "name") is >> s.name;
      else if (tok == "radius") is >> s.radius;
      else if (tok == "preCompDone") is >> s.preCompDone;
      else if (tok == "volume") is >> s.volume;
      else if (tok == "I/m") read3(is, s.inertia_mass);
      else if (tok == "obb.extent") read3(is, s.obb + 12);
      else if (tok == "obb.center") read3(is, s.obb);
      else if (tok == "obb.e1") read3(is, s.obb + 3);
      else if (tok == "obb.e2") read3(is, s.obb + 6);
      else if (tok == "obb.e3") read3(is, s.obb + 9);
      else if (tok == "OBBtreeLevel" || tok == "MCnstep" || tok == "fibObbOption") { std::string x; is >> x; }
      else if (tok == "position") { double v[3]; read3(is, v); }
      else if (tok == "orientation") { double v[4]; is >> v[0] >> v[1] >> v[2] >> v[3]; }
      else if (tok == "nv") {
        size_t nv; is >> nv;
        s.vertex.resize(3 * nv);
        for (size_t k = 0; k < 3 * nv; k++) is >> s.vertex[k];
      } else if (tok == "ne") {
        size_t ne; is >> ne;
        s.edge.resize(2 * ne);
        for (size_t k = 0; k < 2 * ne; k++) is >> s.edge[k];
      } else if (tok == "nf") {
        size_t nf; is >> nf;
        for (size_t f = 0; f < nf; f++) {
          size_t k; is >> k;
          std::vector<int> ids(k);
          for (auto& id : ids) is >> id;
          s.face.push_back(ids);
        }
      }
    }
    if (s.preCompDone != 'y') return fail("shape " + s.name + ": mass properties must be precomputed (preCompDone y)");
    shapeId[s.name] = (int)Shapes.size();
    Shapes.push_back(s);
  }
  return true;
}

bool Rockable::parse(std::istream& conf) {  // Rockable.cpp:643-1069
  std::string tok;
  auto law_line = [&](const std::string& name) {
    int g1, g2; double v;
    conf >> g1 >> g2 >> v;
    dataTableSet(name, g1, g2, v);
  };
  std::set<std::string> lawNames(std::begin(kParamNames), std::end(kParamNames));
  lawNames.insert({"viscTContact", "gcInnerBond", "gcOuterBond"});
  while (conf >> tok) {
    if (tok[0] == '/' || tok[0] == '#' || tok[0] == '!') { std::string r; std::getline(conf, r); continue; }
    if (tok == "t") conf >> t;
    else if (tok == "tmax") conf >> tmax;
    else if (tok == "dt") conf >> dt;
    else if (tok == "interVerlet") conf >> interVerlet;
    else if (tok == "interConf") conf >> interConf;
    else if (tok == "DVerlet") conf >> DVerlet;
    else if (tok == "dVerlet") conf >> dVerlet;
    else if (tok == "parallel_mode") conf >> parallel_mode;
    else if (tok == "density") { int g; double d; conf >> g >> d; density[g] = d; }
    else if (tok == "gravity") read3(conf, gravity);
    else if (tok == "ParamsInInterfaces") conf >> paramsInInterfaces;
    else if (tok == "dynamicUpdateNL") conf >> dynamicUpdateNL;
    else if (tok == "dispUpdateNL") conf >> dispUpdateNL;
    else if (tok == "angleUpdateNL") { conf >> angleUpdateNL; angleUpdateNL *= M_PI / 180.0; }
    else if (tok == "numericalDampingCoeff") conf >> numericalDampingCoeff;
    else if (tok == "VelocityBarrier" || tok == "velocityBarrier" || tok == "AngularVelocityBarrier" ||
             tok == "angularVelocityBarrier") {
      double v; conf >> v;
      if (v > 0.0) return fail(tok + " > 0 is not supported by the GPU engine");
    } else if (tok == "VelocityBarrierExponent" || tok == "AngularVelocityBarrierExponent") { double v; conf >> v; }
    else if (tok == "forceLaw") {  // Rockable.cpp:763-781
      std::string name; conf >> name;
      ForceLaw* fl = Factory<ForceLaw>::instance().create(name);
      if (!fl) {
        std::cerr << "[rockable-gb300] ForceLaw " << name << " is unknown -> Default\n";
        name = "Default";
        fl = Factory<ForceLaw>::instance().create(name);
      }
      forceLaw.reset(fl);
      forceLaw->plug(this);
      forceLaw->init();
      optionNames["forceLaw"] = name;
    } else if (tok == "AddOrRemoveInteractions") {
      std::string n; conf >> n;
      if (n == "bruteForce" || n == "OBBtree") optionNames["AddOrRemoveInteractions"] = n;
      // the GPU list update tests every sub-element pair of a visited body pair
      // (AddOrRemoveInteractions_bruteForce, Rockable.cpp:1309-1432); the tree
      // variant (1440-1541) tests only the pairs whose leaf boxes overlap
      if (n == "OBBtree")
        std::cerr << "[rockable-gb300] AddOrRemoveInteractions OBBtree runs the bruteForce sub-element test\n";
    } else if (tok == "UpdateNL") {
      std::string n; conf >> n;
      if (n == "bruteForce" || n == "linkCells") optionNames["UpdateNL"] = n;
    } else if (tok == "Integrator") {
      std::string n; conf >> n;
      if (n != "velocityVerlet") return fail("integrator " + n + " is not provided by the GPU engine");
      optionNames["Integrator"] = n;
    } else if (tok == "cellMinSizes") read3(conf, cellMinSizes);
    else if (tok == "boxForLinkCellsOpt") conf >> boxForLinkCellsOpt;
    else if (tok == "ContactPartnership") {
      std::string n; conf >> n;
      if (n != "None") return fail("ContactPartnership " + n + " is not supported by the GPU engine");
    } else if (lawNames.count(tok)) law_line(tok);
    else if (tok == "iconf") conf >> iconf;
    else if (tok == "nDriven") conf >> nDriven;
    else if (tok == "shapeFile") {
      std::string name; conf >> name;
      std::string want = path_ + name;
      if (want != shapeFile) {
        shapeFile = want;
        if (!loadShapes(want)) return false;
      }
    } else if (tok == "precision") conf >> precision;
    else if (tok == "Particles") {  // Rockable.cpp:886-931
      size_t nb; conf >> nb;
      P = Particles();
      for (size_t k = 0; k < nb; k++) {
        std::string name; conf >> name;
        if (name[0] == '#') { std::string r; std::getline(conf, r); --k; continue; }
        if (name[0] == '!') { std::string r; std::getline(conf, r); --k; --nb; continue; }
        auto it = shapeId.find(name);
        if (it == shapeId.end()) return fail("unknown shape " + name);
        int g, c; double h, v[19];
        conf >> g >> c >> h;
        for (double& x : v) conf >> x;
        const Shape& S = Shapes[it->second];
        double dens = density.count(g) ? density[g] : 0.0;
        double mass = (h * h * h * S.volume) * dens;
        P.shape.push_back(it->second); P.group.push_back(g); P.cluster.push_back(c); P.homothety.push_back(h);
        P.mass.push_back(mass);
        for (int d = 0; d < 3; d++) P.inertia.push_back((h * h * S.inertia_mass[d]) * mass);
        P.pos.insert(P.pos.end(), v, v + 3); P.vel.insert(P.vel.end(), v + 3, v + 6);
        P.acc.insert(P.acc.end(), v + 6, v + 9); P.Q.insert(P.Q.end(), v + 9, v + 13);
        P.vrot.insert(P.vrot.end(), v + 13, v + 16); P.arot.insert(P.arot.end(), v + 16, v + 19);
      }
      P.force.assign(3 * P.size(), 0.0);
      P.moment.assign(3 * P.size(), 0.0);
    } else if (tok == "Interactions") {  // Rockable.cpp:932-955 (keyed set: first copy wins)
      size_t nb; conf >> nb;
      std::map<std::array<int64_t, 5>, std::array<double, 18>> rows;
      for (size_t k = 0; k < nb; k++) {
        std::array<int64_t, 5> key;
        std::array<double, 18> st;  // n3 dn pos3 vel3 fn ft3 mom3 damp
        for (auto& x : key) conf >> x;
        for (auto& x : st) conf >> x;
        rows.emplace(key, st);
      }
      I = Interactions();
      for (auto& kv : rows) {
        const auto& k = kv.first;
        const auto& s = kv.second;
        I.i.push_back((int)k[0]); I.j.push_back((int)k[1]); I.type.push_back((int)k[2]);
        I.isub.push_back((int)k[3]); I.jsub.push_back((int)k[4]); I.bond.push_back(-1);
        I.n.insert(I.n.end(), s.begin(), s.begin() + 3); I.dn.push_back(s[3]);
        I.pos.insert(I.pos.end(), s.begin() + 4, s.begin() + 7); I.vel.insert(I.vel.end(), s.begin() + 7, s.begin() + 10);
        I.fn.push_back(s[10]); I.ft.insert(I.ft.end(), s.begin() + 11, s.begin() + 14);
        I.mom.insert(I.mom.end(), s.begin() + 14, s.begin() + 17); I.damp.push_back(s[17]);
      }
    } else if (tok == "Interfaces") {  // Rockable.cpp:956-1002
      size_t nb; conf >> nb;
      F = Interfaces();
      for (size_t k = 0; k < nb; k++) {
        int bi, bj; size_t nbonds; double dn0;
        conf >> bi >> bj >> nbonds >> dn0;
        double par[8] = {0, 0, 0, 0, 0, 0, 2.0, 0};
        if (paramsInInterfaces == 1) for (double& x : par) conf >> x;
        std::vector<std::array<int32_t, 3>> bonds(nbonds);
        for (auto& b : bonds) conf >> b[0] >> b[1] >> b[2];
        F.i.push_back(bi); F.j.push_back(bj); F.nbonds.push_back((int)nbonds); F.dn0.push_back(dn0);
        F.params.insert(F.params.end(), par, par + 8); F.is_inner.push_back(1); F.bonds.push_back(bonds);
        F.live.emplace_back(bonds.size(), 1);
      }
    } else if (tok == "stickVerticesInClusters") {
      double eps; conf >> eps;
      stickVerticesInClusters(eps);
    } else if (tok == "setVariableStickParams") {
      std::string par, io; double lambda, m; int ts;
      conf >> par >> io >> lambda >> m >> ts;
      setVariableStickParams(par, io, lambda, m);
    } else if (tok == "BodyForce") {
      std::string name; conf >> name;
      BodyForce* bf = Factory<BodyForce>::instance().create(name);
      if (!bf) return fail("BodyForce " + name + " is unknown");
      bf->plug(this);
      bf->read(conf);
      bodyForce.reset(bf);
    } else if (tok == "DataExtractor") {  // Rockable.cpp:1003-1022 (kept for compatibility)
      std::string name; conf >> name;
      register_builtin_extractors();
      std::cerr << "[rockable-gb300] the DataExtractor named " << name
                << " is defined in the input file; dataExtractors.txt is the place for it\n";
      DataExtractor* de = Factory<DataExtractor>::instance().create(name);
      if (!de) {
        std::cerr << "[rockable-gb300] the DataExtractor named " << name << " is unknown\n";
      } else {
        de->plug(this);
        de->read(conf);
        dataExtractors.emplace_back(de);
      }
    } else if (tok == "usePeriodicCell" || tok == "initSpringJoint" || tok == "useSoftParticles") {
      return fail("keyword " + tok + " is outside the GPU engine (periodic cells, spring joints, soft particles)");
    }
    // other tokens: skipped like the reference's kwParser does with unknown keywords
  }
  return true;
}

// PreproCommand_stickVerticesInClusters.cpp:56-141 is a load-time pass; the
// engine's bond creation needs the placed vertices, so it is evaluated here on
// the host in FP64 with the same arithmetic as the step (quaternion rotation
// u + s t + v x t with t = 2 v x u).
static void rot(const double* q, const double* u, double* out) {
  const double s = q[0], vx = q[1], vy = q[2], vz = q[3];
  double t0 = 2.0 * (vy * u[2] - vz * u[1]), t1 = 2.0 * (vz * u[0] - vx * u[2]), t2 = 2.0 * (vx * u[1] - vy * u[0]);
  out[0] = u[0] + s * t0 + (vy * t2 - vz * t1);
  out[1] = u[1] + s * t1 + (vz * t0 - vx * t2);
  out[2] = u[2] + s * t2 + (vx * t1 - vy * t0);
}

void Rockable::stickVerticesInClusters(double eps) {
  // Bodies are compared by bounding spheres before the vertex test (the
  // reference compares enlarged OBBs; the vertex test below decides).
  const size_t n = P.size();
  std::vector<double> gv;
  std::vector<size_t> ofs(n + 1, 0);
  for (size_t b = 0; b < n; b++) ofs[b + 1] = ofs[b] + Shapes[P.shape[b]].vertex.size() / 3;
  gv.resize(3 * ofs[n]);
  std::vector<double> bound(n, 0.0);
  for (size_t b = 0; b < n; b++) {
    const Shape& S = Shapes[P.shape[b]];
    for (size_t v = 0; v < S.vertex.size() / 3; v++) {
      double u[3] = {P.homothety[b] * S.vertex[3 * v], P.homothety[b] * S.vertex[3 * v + 1],
                     P.homothety[b] * S.vertex[3 * v + 2]};
      double r[3];
      rot(&P.Q[4 * b], u, r);
      for (int d = 0; d < 3; d++) gv[3 * (ofs[b] + v) + d] = P.pos[3 * b + d] + r[d];
      bound[b] = std::max(bound[b], std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
    }
    bound[b] += P.homothety[b] * S.radius;
  }
  std::map<std::pair<int, int>, size_t> iface_of;
  for (size_t k = 0; k < F.i.size(); k++) iface_of[{F.i[k], F.j[k]}] = k;
  std::map<std::array<int64_t, 5>, size_t> entry_of;
  for (size_t k = 0; k < I.size(); k++) entry_of[{I.i[k], I.j[k], I.type[k], I.isub[k], I.jsub[k]}] = k;
  std::vector<std::array<int64_t, 5>> newkeys;
  for (size_t i = nDriven; i < n; i++)
    for (size_t j = i + 1; j < n; j++) {
      if (P.cluster[i] != P.cluster[j]) continue;
      double dx = P.pos[3 * j] - P.pos[3 * i], dy = P.pos[3 * j + 1] - P.pos[3 * i + 1], dz = P.pos[3 * j + 2] - P.pos[3 * i + 2];
      double lim = bound[i] + bound[j] + DVerlet + eps;
      if (dx * dx + dy * dy + dz * dz > lim * lim) continue;
      double Ri = P.homothety[i] * Shapes[P.shape[i]].radius, Rj = P.homothety[j] * Shapes[P.shape[j]].radius;
      for (size_t iv = ofs[i]; iv < ofs[i + 1]; iv++)
        for (size_t jv = ofs[j]; jv < ofs[j + 1]; jv++) {
          double ex = gv[3 * jv] - gv[3 * iv], ey = gv[3 * jv + 1] - gv[3 * iv + 1], ez = gv[3 * jv + 2] - gv[3 * iv + 2];
          double distSqr = ex * ex + ey * ey + ez * ez;
          double dMax = eps + (Ri + Rj);
          dMax *= dMax;
          if (distSqr < dMax) {
            int g1 = P.group[i], g2 = P.group[j];
            auto it = iface_of.find({(int)i, (int)j});
            size_t fk;
            if (it == iface_of.end()) {
              fk = F.i.size();
              iface_of[{(int)i, (int)j}] = fk;
              F.i.push_back((int)i); F.j.push_back((int)j); F.nbonds.push_back(0); F.dn0.push_back(0.0);
              double par[8] = {dataTableGet("knInnerBond", g1, g2), dataTableGet("ktInnerBond", g1, g2),
                               dataTableGet("krInnerBond", g1, g2), dataTableGet("fn0InnerBond", g1, g2),
                               dataTableGet("ft0InnerBond", g1, g2), dataTableGet("mom0InnerBond", g1, g2),
                               dataTableGet("powInnerBond", g1, g2), 0.0};
              F.params.insert(F.params.end(), par, par + 8);
              F.is_inner.push_back(1);
              F.bonds.emplace_back();
              F.live.emplace_back();
            } else {
              fk = it->second;
            }
            int isub = (int)(iv - ofs[i]), jsub = (int)(jv - ofs[j]);
            F.bonds[fk].push_back({0, isub, jsub});
            // PreproCommand_stickVerticesInClusters.cpp:127-133: the bonded
            // interaction goes into a std::set, where an existing one with
            // the same key stays as it was (without the bond)
            F.live[fk].push_back(entry_of.count({(int64_t)i, (int64_t)j, 0, isub, jsub}) ? 0 : 1);
            F.nbonds[fk]++;
            newkeys.push_back({(int64_t)i, (int64_t)j, 0, isub, jsub});
          }
        }
    }
  // new bonded vertex-vertex entries: fresh history, damping from the
  // inner-bond parameters (the device narrow phase computes their geometry)
  for (auto& k : newkeys) {
    if (entry_of.count(k)) continue;
    size_t i = (size_t)k[0], j = (size_t)k[1];
    double en2 = dataTableGet("en2InnerBond", P.group[i], P.group[j]);
    double kn = dataTableGet("knInnerBond", P.group[i], P.group[j]);
    double meff = (P.mass[i] * P.mass[j]) / (P.mass[i] + P.mass[j]);
    double damp = 0.0;
    if (en2 > 0.0 && en2 < 1.0) {
      double logen = 0.5 * std::log(en2);
      double dampRate = -logen / std::sqrt(logen * logen + M_PI * M_PI);
      damp = dampRate * 2.0 * std::sqrt(kn * meff);
    } else if (en2 <= 0.0) {
      damp = 2.0 * std::sqrt(kn * meff);
    }
    entry_of[k] = (size_t)-1;
    I.i.push_back((int)k[0]); I.j.push_back((int)k[1]); I.type.push_back(0); I.isub.push_back((int)k[3]);
    I.jsub.push_back((int)k[4]); I.bond.push_back(-1);
    for (int d = 0; d < 3; d++) { I.n.push_back(0); I.pos.push_back(0); I.vel.push_back(0); I.ft.push_back(0); I.mom.push_back(0); }
    I.dn.push_back(0.0); I.fn.push_back(0.0); I.damp.push_back(damp);
  }
}

// PreproCommand_setVariableStickParams.cpp:57-94 (libstdc++ engine and
// Weibull distribution with the default seed, interfaces in (i, j) order)
void Rockable::setVariableStickParams(const std::string& par, const std::string& io, double lambda, double m) {
  std::default_random_engine gen;
  std::weibull_distribution<> dist(m, lambda);
  int shift = 0;
  if (par == "kt") shift = 1;
  else if (par == "kr") shift = 2;
  else if (par == "fn0") shift = 3;
  else if (par == "ft0") shift = 4;
  else if (par == "mom0") shift = 5;
  int inner = io == "inner" ? 1 : 0;
  std::vector<size_t> order(F.i.size());
  for (size_t k = 0; k < order.size(); k++) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return F.i[a] != F.i[b] ? F.i[a] < F.i[b] : F.j[a] < F.j[b];
  });
  for (size_t k : order) {
    int ic = P.cluster[F.i[k]], jc = P.cluster[F.j[k]];
    if (inner == 0 && ic == jc) continue;
    if (inner == 1 && ic != jc) continue;
    F.params[8 * k + shift] = dist(gen);
  }
  paramsInInterfaces = 1;
}

bool Rockable::loadConf(const std::string& name) {  // Rockable.cpp:1085-1145
  std::ifstream conf(name);
  if (!conf) return fail("cannot read " + name);
  std::string prog;
  conf >> prog;
  if (prog == "redirection") {
    std::string sub, nn;
    conf >> sub >> nn;
    path_ = dirname_of(name) + sub;
    return loadConf(path_ + nn);
  }
  if (path_.empty()) path_ = dirname_of(name);
  std::string date;
  conf >> date;
  if (!parse(conf)) return false;
  if (!upload()) return false;
  // the load-time step (Rockable.cpp:1137) also fills the contact geometry
  // written by the first saveConf
  if (!ck(rk_set_record_geometry(ctx_, 1), "rk_set_record_geometry")) return false;
  if (!ck(rk_accelerations(ctx_), "rk_accelerations")) return false;
  return ck(rk_set_record_geometry(ctx_, 0), "rk_set_record_geometry");
}

bool Rockable::readDrivingSystem(const std::string& fname) {  // DrivingSystem.cpp:44-268
  std::ifstream is(fname);
  if (!is) return fail("cannot open " + fname);
  static const std::map<std::string, int> types = {
      {"_x_Vel_", RK_X_VEL}, {"_y_Vel_", RK_Y_VEL}, {"_z_Vel_", RK_Z_VEL}, {"_xrot_Vel_", RK_XROT_VEL},
      {"_yrot_Vel_", RK_YROT_VEL}, {"_zrot_Vel_", RK_ZROT_VEL}, {"_x_For_", RK_X_FOR}, {"_y_For_", RK_Y_FOR},
      {"_z_For_", RK_Z_FOR}, {"_xrot_Mom_", RK_XROT_MOM}, {"_yrot_Mom_", RK_YROT_MOM}, {"_zrot_Mom_", RK_ZROT_MOM},
      {"_xyzrot_Vel_", RK_XYZROT_VEL}, {"_xyzrot_Mom_", RK_XYZROT_MOM}};
  controls.clear();
  servo = rk_servo{};
  std::string tok;
  while (is >> tok) {
    if (tok[0] == '/' || tok[0] == '#' || tok[0] == '!') { std::string r; std::getline(is, r); continue; }
    if (tok == "Control") {
      std::string ts; rk_control c{}; is >> ts >> c.body;
      auto it = types.find(ts);
      c.type = it == types.end() ? 0 : it->second;
      if (c.type >= 100) read3(is, c.vec); else is >> c.value;
      controls.push_back(c);
    } else if (tok == "Servo") {
      std::string name; is >> name;
      if (name != "tritriIsostaticCompression") return fail("servo " + name + " is not supported by the GPU engine");
      int w[6];
      for (int& x : w) is >> x;
      servo.kind = 1;
      servo.icontr = (int)controls.size();
      for (int k = 0; k < 6; k++) servo.walls[k] = w[k];
      is >> servo.pressure;
      const int types6[6] = {RK_X_VEL, RK_X_FOR, RK_Y_VEL, RK_Y_FOR, RK_Z_VEL, RK_Z_FOR};
      for (int k = 0; k < 6; k++) {
        rk_control c{};
        c.type = types6[k];
        c.body = w[k];
        controls.push_back(c);
      }
    }
  }
  if (!ctx_) return true;
  return ck(rk_set_controls(ctx_, controls.data(), (int32_t)controls.size(), &servo), "rk_set_controls");
}

bool Rockable::upload() {
  if (P.size() == 0 || Shapes.empty()) return fail("no particles or no shapes");
  if (!ctx_) {
    rk_config cfg{0, RK_FORM_FP64, (int64_t)std::max<size_t>(I.size() * 2, 1024)};
    int rc = rk_create(&ctx_, &cfg);
    if (rc != RK_OK) return fail("rk_create failed (code " + std::to_string(rc) + "): a CUDA device is required");
  }
  // shapes
  std::vector<int32_t> vo{0}, eo{0}, fo{0}, fvo{0}, ed, fv;
  std::vector<double> vx, rad, obb;
  for (auto& s : Shapes) {
    vx.insert(vx.end(), s.vertex.begin(), s.vertex.end());
    ed.insert(ed.end(), s.edge.begin(), s.edge.end());
    for (auto& f : s.face) {
      fv.insert(fv.end(), f.begin(), f.end());
      fvo.push_back((int32_t)fv.size());
    }
    vo.push_back(vo.back() + (int32_t)(s.vertex.size() / 3));
    eo.push_back(eo.back() + (int32_t)(s.edge.size() / 2));
    fo.push_back(fo.back() + (int32_t)s.face.size());
    rad.push_back(s.radius);
    obb.insert(obb.end(), s.obb, s.obb + 15);
  }
  if (ed.empty()) ed.push_back(0);
  if (fv.empty()) fv.push_back(0);
  rk_shapes sh{(int32_t)Shapes.size(), vo.data(), vx.data(), eo.data(), ed.data(), fo.data(), fvo.data(), fv.data(),
               rad.data(), obb.data()};
  if (!ck(rk_upload_shapes(ctx_, &sh), "rk_upload_shapes")) return false;
  {  // for the device-formatted conf text
    std::vector<const char*> names;
    for (auto& sp : Shapes) names.push_back(sp.name.c_str());
    if (!ck(rk_set_shape_names(ctx_, names.data(), (int32_t)names.size()), "rk_set_shape_names")) return false;
  }
  rk_bodies b{(int64_t)P.size(), (int64_t)nDriven, P.pos.data(), P.vel.data(), P.acc.data(), P.Q.data(),
              P.vrot.data(), P.arot.data(), P.homothety.data(), P.mass.data(), P.inertia.data(), P.shape.data(),
              P.group.data(), P.cluster.data()};
  if (!ck(rk_upload_bodies(ctx_, &b), "rk_upload_bodies")) return false;
  int ngroup = 1;
  for (int g : P.group) ngroup = std::max(ngroup, g + 1);
  for (auto& kv : dataTable)
    for (auto& e : kv.second) ngroup = std::max(ngroup, std::max(e.first.first, e.first.second) + 1);
  std::vector<double> table((size_t)RK_NPARAM * ngroup * ngroup, 0.0);
  for (int p = 0; p < RK_NPARAM; p++)
    for (int g1 = 0; g1 < ngroup; g1++)
      for (int g2 = 0; g2 < ngroup; g2++)
        table[((size_t)p * ngroup + g1) * ngroup + g2] = dataTableGet(kParamNames[p], g1, g2);
  rk_params prm{};
  prm.t = t;
  prm.dt = dt;
  for (int d = 0; d < 3; d++) prm.gravity[d] = gravity[d];
  prm.DVerlet = DVerlet;
  prm.dVerlet = dVerlet;
  prm.interVerlet = interVerlet;
  prm.interVerletC = 0.0;
  prm.numerical_damping = numericalDampingCoeff;
  prm.law = forceLaw->device_law();
  prm.params_in_interfaces = paramsInInterfaces;
  prm.dynamic_update_nl = dynamicUpdateNL;
  prm.disp_update_nl = dispUpdateNL;
  prm.angle_update_nl = angleUpdateNL;
  prm.ngroup = ngroup;
  prm.table = table.data();
  if (!ck(rk_set_params(ctx_, &prm), "rk_set_params")) return false;
  // interfaces sorted by (i, j); bond index of each bonded entry
  std::vector<size_t> order(F.i.size());
  for (size_t k = 0; k < order.size(); k++) order[k] = k;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t c) {
    return F.i[a] != F.i[c] ? F.i[a] < F.i[c] : F.j[a] < F.j[c];
  });
  Interfaces Fs;
  for (size_t k : order) {
    Fs.i.push_back(F.i[k]); Fs.j.push_back(F.j[k]); Fs.nbonds.push_back(F.nbonds[k]); Fs.dn0.push_back(F.dn0[k]);
    Fs.params.insert(Fs.params.end(), F.params.begin() + 8 * k, F.params.begin() + 8 * k + 8);
    Fs.is_inner.push_back(F.is_inner[k]); Fs.bonds.push_back(F.bonds[k]); Fs.live.push_back(F.live[k]);
  }
  F = Fs;
  // entries sorted by key
  std::vector<size_t> eorder(I.size());
  for (size_t k = 0; k < eorder.size(); k++) eorder[k] = k;
  auto key = [&](size_t k) { return std::array<int64_t, 5>{I.i[k], I.j[k], I.type[k], I.isub[k], I.jsub[k]}; };
  std::sort(eorder.begin(), eorder.end(), [&](size_t a, size_t c) { return key(a) < key(c); });
  Interactions Is;
  for (size_t k : eorder) {
    Is.i.push_back(I.i[k]); Is.j.push_back(I.j[k]); Is.type.push_back(I.type[k]); Is.isub.push_back(I.isub[k]);
    Is.jsub.push_back(I.jsub[k]); Is.bond.push_back(-1); Is.dn.push_back(I.dn[k]); Is.fn.push_back(I.fn[k]);
    Is.damp.push_back(I.damp[k]);
    for (int d = 0; d < 3; d++) {
      Is.n.push_back(I.n[3 * k + d]); Is.pos.push_back(I.pos[3 * k + d]); Is.vel.push_back(I.vel[3 * k + d]);
      Is.ft.push_back(I.ft[3 * k + d]); Is.mom.push_back(I.mom[3 * k + d]);
    }
  }
  I = Is;
  std::map<std::array<int64_t, 5>, size_t> pos_of;
  for (size_t k = 0; k < I.size(); k++) pos_of[key(k)] = k;
  for (size_t f = 0; f < F.i.size(); f++)
    for (size_t q = 0; q < F.bonds[f].size(); q++) {
      if (q < F.live[f].size() && !F.live[f][q]) continue;  // an interaction that kept no bond
      const auto& b = F.bonds[f][q];
      auto it = pos_of.find({F.i[f], F.j[f], b[0], b[1], b[2]});
      if (it != pos_of.end()) I.bond[it->second] = (int32_t)f;
    }
  if (!F.i.empty()) {
    rk_interfaces fi{(int64_t)F.i.size(), F.i.data(), F.j.data(), F.dn0.data(), F.params.data(), F.is_inner.data()};
    if (!ck(rk_upload_interfaces(ctx_, &fi), "rk_upload_interfaces")) return false;
  }
  rk_entries en{(int64_t)I.size(), I.i.data(), I.j.data(), I.type.data(), I.isub.data(), I.jsub.data(), I.dn.data(),
                I.fn.data(), I.ft.data(), I.mom.data(), I.damp.data(), I.bond.data()};
  if (!ck(rk_upload_entries(ctx_, &en), "rk_upload_entries")) return false;
  if (!controls.empty() || servo.kind)
    if (!ck(rk_set_controls(ctx_, controls.data(), (int32_t)controls.size(), &servo), "rk_set_controls")) return false;
  if (bodyForce) {
    std::vector<double> bp;
    const int kind = bodyForce->device_body_force(bp);
    if (kind < 0) return fail("this BodyForce plugin has no GPU form");
    const size_t n = P.size();
    std::vector<double> vol(n);
    for (size_t b = 0; b < n; b++) {
      double h = P.homothety[b];
      vol[b] = Shapes[P.shape[b]].volume * h * h * h;
    }
    if (!ck(rk_set_body_force(ctx_, kind, bp.data(), (int32_t)bp.size(), vol.data()), "rk_set_body_force"))
      return false;
  }
  uploaded_ = true;
  return true;
}

bool Rockable::updateNL() { return ck(rk_update_nl(ctx_), "rk_update_nl"); }

bool Rockable::syncFromDevice(bool geometry) {
  const size_t n = P.size();
  if (!ck(rk_download_bodies(ctx_, P.pos.data(), P.vel.data(), P.acc.data(), P.Q.data(), P.vrot.data(),
                             P.arot.data(), P.force.data(), P.moment.data()), "rk_download_bodies"))
    return false;
  (void)n;
  const int64_t ne = rk_num_entries(ctx_);
  I.i.resize(ne); I.j.resize(ne); I.type.resize(ne); I.isub.resize(ne); I.jsub.resize(ne); I.bond.resize(ne);
  I.dn.resize(ne); I.fn.resize(ne); I.damp.resize(ne); I.active.resize(ne);
  I.ft.resize(3 * ne); I.mom.resize(3 * ne); I.n.resize(3 * ne); I.pos.resize(3 * ne); I.vel.resize(3 * ne);
  if (!ck(rk_download_entries(ctx_, I.i.data(), I.j.data(), I.type.data(), I.isub.data(), I.jsub.data(), I.dn.data(),
                              I.fn.data(), I.ft.data(), I.mom.data(), I.damp.data(), I.bond.data(), I.active.data(),
                              geometry ? I.n.data() : nullptr, geometry ? I.pos.data() : nullptr,
                              geometry ? I.vel.data() : nullptr), "rk_download_entries"))
    return false;
  if (!F.i.empty()) {
    F.broken.resize(F.i.size());
    if (!ck(rk_download_interfaces(ctx_, nullptr, nullptr, F.broken.data()), "rk_download_interfaces")) return false;
  }
  return true;
}

bool Rockable::saveConf(const std::string& fname) {  // Rockable.cpp:440-610
  std::ostringstream h;
  h << "Rockable 21-08-2022\n";
  for (auto& kv : optionNames) h << kv.first << " " << kv.second << '\n';
  h << "t " << t << "\ntmax " << tmax << "\ndt " << dt << "\ninterVerlet " << interVerlet << "\ninterConf "
    << interConf << "\nDVerlet " << DVerlet << "\ndVerlet " << dVerlet << "\nparallel_mode " << parallel_mode << '\n';
  for (auto& kv : density)
    if (kv.second > 0.0) h << "density " << kv.first << " " << kv.second << '\n';
  h << "gravity " << gravity[0] << " " << gravity[1] << " " << gravity[2] << '\n';
  if (bodyForce) {  // Rockable.cpp:470-473
    h << "BodyForce ";
    bodyForce->write(h);
  }
  h << "ParamsInInterfaces " << paramsInInterfaces << "\ndynamicUpdateNL " << dynamicUpdateNL << '\n';
  if (dynamicUpdateNL) h << "dispUpdateNL " << dispUpdateNL << "\nangleUpdateNL " << angleUpdateNL * 180.0 / M_PI << '\n';
  h << "numericalDampingCoeff " << numericalDampingCoeff << "\nVelocityBarrier 0\nAngularVelocityBarrier 0\n"
    << "VelocityBarrierExponent 1\nAngularVelocityBarrierExponent 1\n";
  for (auto& kv : dataTable) {
    std::set<std::pair<int, int>> seen;
    for (auto& e : kv.second)
      if (e.first.first <= e.first.second && !seen.count(e.first)) {
        seen.insert(e.first);
        h << kv.first << ' ' << e.first.first << ' ' << e.first.second << ' ' << e.second << '\n';
      }
  }
  h << "ContactPartnership None\ncellMinSizes " << cellMinSizes[0] << " " << cellMinSizes[1] << " "
    << cellMinSizes[2] << "\nboxForLinkCellsOpt " << boxForLinkCellsOpt << "\niconf " << iconf << "\nnDriven "
    << nDriven << '\n';
  std::string shp = shapeFile;
  size_t sl = shp.find_last_of('/');
  if (sl != std::string::npos) shp = shp.substr(sl + 1);
  h << "shapeFile " << shp << "\nprecision " << precision << '\n';
  std::string o = h.str();
  // the Particles and Interactions sections are formatted on the device from
  // its own state (rk_format_conf: the same printf rounding, the contact
  // normal toward zero), one copy of text instead of the state
  int64_t lp = 0, li = 0, na = 0;
  if (!ck(rk_format_conf(ctx_, precision, nullptr, 0, &lp, &li, &na), "rk_format_conf")) return false;
  std::string txt((size_t)(lp + li), '\0');
  if (!ck(rk_format_conf(ctx_, precision, &txt[0], lp + li, &lp, &li, &na), "rk_format_conf")) return false;
  o += "Particles " + std::to_string(P.size()) + "\n";
  o += "#name group cluster homothety pos.x pos.y pos.z vel.x vel.y vel.z acc.x acc.y acc.z Q.w Q.x Q.y Q.z vrot.x vrot.y vrot.z arot.x arot.y arot.z\n";
  o.append(txt, 0, (size_t)lp);
  o += "Interactions " + std::to_string(na) + "\n";
  o.append(txt, (size_t)lp, (size_t)li);
  size_t nf = 0;
  for (size_t f = 0; f < F.i.size(); f++) nf += !(F.broken.size() > f && F.broken[f]);
  o += "Interfaces " + std::to_string(nf) + "\n";
  char b[64];
  for (size_t f = 0; f < F.i.size(); f++) {
    if (F.broken.size() > f && F.broken[f]) continue;
    o += std::to_string(F.i[f]) + ' ' + std::to_string(F.j[f]) + "  " + std::to_string(F.bonds[f].size()) + ' ';
    snprintf(b, sizeof b, "%.6f", F.dn0[f]);
    o += b;
    if (paramsInInterfaces == 1) {
      for (int q = 0; q < 8; q++) { snprintf(b, sizeof b, " %.6f", F.params[8 * f + q]); o += b; }
      o += ' ';
    }
    for (auto& bd : F.bonds[f])
      o += "  " + std::to_string(bd[0]) + ' ' + std::to_string(bd[1]) + ' ' + std::to_string(bd[2]);
    o += '\n';
  }
  std::ofstream out(fname);
  if (!out) return fail("cannot write " + fname);
  out << o;
  return true;
}

bool Rockable::run(long nsteps) {
  rk_step_report rep{};
  for (long s = 0; s < nsteps; s++) t += dt;
  if (nsteps <= 0) return true;
  // the last step records the contact geometry that a saveConf writes
  if (nsteps > 1 && !ck(rk_step(ctx_, nsteps - 1, &rep), "rk_step")) return false;
  if (!ck(rk_set_record_geometry(ctx_, 1), "rk_set_record_geometry")) return false;
  const bool ok = ck(rk_step(ctx_, 1, &rep), "rk_step");
  return ck(rk_set_record_geometry(ctx_, 0), "rk_set_record_geometry") && ok;
}

long Rockable::consoleRun(const std::string& outdir, long max_steps) {  // run.cpp + Rockable.cpp:2538-2746
  if (!uploaded_) { fail("load a conf first"); return -1; }
  if (!updateNL()) return -1;
  // the data extractors of ./dataExtractors.txt (Rockable.cpp:1152-1180,
  // 1241-1250), documented in extractedDataDoc.txt, then initialised
  if (!extractorsRead_) {
    extractorsRead_ = true;
    readDataExtractors("dataExtractors.txt");
  }
  if (!dataExtractors.empty()) {
    std::ofstream doc("extractedDataDoc.txt");
    for (auto& de : dataExtractors) de->generateHelp(doc);
  }
  bool geo_extractor = false;
  for (auto& de : dataExtractors) {
    de->init();
    geo_extractor = geo_extractor || de->needsGeometry();
  }
  // the reference's step counter: (size_t)(t / dt) at the start, compared
  // with nstep / nrec after the step's body, then incremented
  auto due = [&](long s, bool geometry_only) {
    for (auto& de : dataExtractors) {
      if (geometry_only && !de->needsGeometry()) continue;
      if ((!geometry_only && de->nstep > 0 && s % de->nstep == 0) || (de->nrec > 0 && s % de->nrec == 0)) return true;
    }
    return false;
  };
  const double dt_2 = 0.5 * dt;
  if (!syncFromDevice(true) || !saveConf(outdir + "/conf" + std::to_string(iconf))) return -1;
  step_ = (long)(t / dt);
  long steps = 0;
  while (t <= tmax && (max_steps <= 0 || steps < max_steps)) {
    // steps until the next conf output or extractor call (same accumulation
    // as the reference)
    long n = 0;
    double tt = t, cc = interConfC_;
    bool save = false;
    while (true) {
      if (!(tt <= tmax)) break;
      if (max_steps > 0 && steps + n >= max_steps) break;
      tt += dt;
      cc += dt;
      n++;
      if (cc >= interConf - dt_2) { save = true; break; }
      if (!dataExtractors.empty() && due(step_ + n - 1, false)) break;
    }
    if (n == 0) break;
    const long s_last = step_ + n - 1;
    const bool geo = save || (geo_extractor && due(s_last, true));
    if (n > 1) {
      rk_step_report rep{};
      if (!ck(rk_step(ctx_, n - 1, &rep), "rk_step")) return -1;
    }
    if (!ck(rk_set_record_geometry(ctx_, geo ? 1 : 0), "rk_set_record_geometry")) return -1;
    rk_step_report rep{};
    if (!ck(rk_step(ctx_, 1, &rep), "rk_step")) return -1;
    if (geo) rk_set_record_geometry(ctx_, 0);
    t = tt;
    interConfC_ = cc;
    steps += n;
    step_ += n;
    if (save) {
      iconf++;
      if (!syncFromDevice(true) || !saveConf(outdir + "/conf" + std::to_string(iconf))) return -1;
      interConfC_ = 0.0;
    }
    if (!dataExtractors.empty() && due(s_last, false)) {
      bool mirror = false;  // the extractors that read the host mirror need it downloaded
      for (auto& de : dataExtractors) mirror = mirror || !de->onDevice();
      if (!save && mirror && !syncFromDevice(geo)) return -1;
      for (auto& de : dataExtractors) {
        if (de->nstep > 0 && s_last % de->nstep == 0) de->exec();
        if (de->nrec > 0 && s_last % de->nrec == 0) de->record();
      }
    }
    if (computationStopAsked > 0) {
      // the reference's loop makes one more step before it sees the request
      // (Rockable.cpp:2586-2595)
      rk_step_report r2{};
      if (!ck(rk_step(ctx_, 1, &r2), "rk_step")) return -1;
      t += dt;
      interConfC_ += dt;
      steps++;
      step_++;
      break;
    }
  }
  for (auto& de : dataExtractors) de->end();
  return steps;
}

}  // namespace rkhost

// =============================================================== C API ====
static std::string g_err;
struct rkh_sim {
  rkhost::Rockable R;
};

extern "C" {
rkh_sim* rkh_open(const char* conf_path) {
  rkh_sim* s = new rkh_sim();
  if (!s->R.loadConf(conf_path)) {
    g_err = s->R.error();
    delete s;
    return nullptr;
  }
  return s;
}
const char* rkh_error(void) { return g_err.c_str(); }
void rkh_close(rkh_sim* s) { delete s; }
int rkh_read_driving(rkh_sim* s, const char* path) {
  if (!s->R.readDrivingSystem(path)) { g_err = s->R.error(); return -1; }
  return 0;
}
long rkh_console_run(rkh_sim* s, const char* outdir, long max_steps) {
  long n = s->R.consoleRun(outdir, max_steps);
  if (n < 0) g_err = s->R.error();
  return n;
}
int rkh_run(rkh_sim* s, long nsteps) {
  if (!s->R.run(nsteps)) { g_err = s->R.error(); return -1; }
  return 0;
}
rk_ctx* rkh_context(rkh_sim* s) { return s ? s->R.ctx() : nullptr; }
int rkh_save_conf(rkh_sim* s, const char* path) {
  if (!s->R.syncFromDevice(true) || !s->R.saveConf(path)) { g_err = s->R.error(); return -1; }
  return 0;
}
}
