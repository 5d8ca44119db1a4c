// rk_oracle.cpp -- CPU restatement of Rockable's DEM hot path (TEST INFRASTRUCTURE).
//
// This file is the checker for the CUDA path, not part of the product.  Each
// function cites the reference file:line it restates (paths are relative to
// the Rockable source tree).  The arithmetic of the unvendored `toofus`
// library (vec3 / quat / OBB / linkCells) is restated from the mathematics;
// where several operation orders are possible, the pinned one is variant 0
// (selected by reproducing the reference's regression goldens bit for bit).
//
// Build with -ffp-contract=off: fused multiply-adds would change results.

#include "rk_oracle.h"

#include <algorithm>
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

namespace orc {

// Pinned choice: reproduces the 512_particles and 518_poly goldens bit for bit.
static orc_variant g_var = {1, 0, 0, 3, 1, 1};
static std::string g_err;

// ---------------------------------------------------------------- vec3 ----
struct V3 {
  double x{0.0}, y{0.0}, z{0.0};
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double& operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
  double operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
  void reset() { x = y = z = 0.0; }
};
static inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
static inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline double operator*(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3& operator+=(V3& a, const V3& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
static inline V3& operator-=(V3& a, const V3& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
static inline V3& operator*=(V3& a, double s) { a.x *= s; a.y *= s; a.z *= s; return a; }
static inline V3 vdiv(const V3& a, double s) {
  if (g_var.vdiv == 0) return V3(a.x / s, a.y / s, a.z / s);
  double inv = 1.0 / s;
  return V3(a.x * inv, a.y * inv, a.z * inv);
}
static inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double norm2(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double norm(const V3& a) { return sqrt(norm2(a)); }
// Normalise in place and return the norm before normalisation.
static inline double normalize(V3& a) {
  double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  if (g_var.vnorm == 0) {
    if (n > 0.0) { a.x /= n; a.y /= n; a.z /= n; }
  } else {
    if (n > 0.0) { double inv = 1.0 / n; a.x *= inv; a.y *= inv; a.z *= inv; }
  }
  return n;
}

// ---------------------------------------------------------------- quat ----
// Unit quaternion (s, v) mapping body-frame vectors to the global frame.
struct Quat {
  double s{1.0};
  V3 v;
  void reset() { s = 1.0; v.reset(); }
};
static inline Quat qconj(const Quat& q) { Quat r; r.s = q.s; r.v = -q.v; return r; }
// Hamilton product a (x) b
static inline Quat qmul(const Quat& a, const Quat& b) {
  Quat r;
  r.s = a.s * b.s - a.v * b.v;
  r.v = a.s * b.v + b.s * a.v + cross(a.v, b.v);
  return r;
}
// Rotate u by q: q (0,u) q*
static inline V3 qrot(const Quat& q, const V3& u) {
  switch (g_var.qrot) {
    default:
    case 0: {  // rotation-matrix form
      double xx = q.v.x * q.v.x, yy = q.v.y * q.v.y, zz = q.v.z * q.v.z;
      double xy = q.v.x * q.v.y, xz = q.v.x * q.v.z, yz = q.v.y * q.v.z;
      double sx = q.s * q.v.x, sy = q.s * q.v.y, sz = q.s * q.v.z;
      return V3(u.x * (1.0 - 2.0 * (yy + zz)) + u.y * 2.0 * (xy - sz) + u.z * 2.0 * (xz + sy),
                u.x * 2.0 * (xy + sz) + u.y * (1.0 - 2.0 * (xx + zz)) + u.z * 2.0 * (yz - sx),
                u.x * 2.0 * (xz - sy) + u.y * 2.0 * (yz + sx) + u.z * (1.0 - 2.0 * (xx + yy)));
    }
    case 1: {  // t = 2 v x u ; u' = u + s t + v x t
      V3 t = 2.0 * cross(q.v, u);
      return u + q.s * t + cross(q.v, t);
    }
    case 2: {  // u' = u + 2s (v x u) + 2 v x (v x u)
      V3 c = cross(q.v, u);
      return u + 2.0 * q.s * c + 2.0 * cross(q.v, c);
    }
    case 3: {  // explicit q (0,u) q*
      Quat p; p.s = 0.0; p.v = u;
      return qmul(qmul(q, p), qconj(q)).v;
    }
    case 4: {  // (s^2 - v.v) u + 2 (v.u) v + 2 s (v x u)
      return (q.s * q.s - q.v * q.v) * u + 2.0 * (q.v * u) * q.v + 2.0 * q.s * cross(q.v, u);
    }
    case 5: {  // matrix with diagonal s^2 + x^2 - y^2 - z^2
      double ss = q.s * q.s, xx = q.v.x * q.v.x, yy = q.v.y * q.v.y, zz = q.v.z * q.v.z;
      double xy = q.v.x * q.v.y, xz = q.v.x * q.v.z, yz = q.v.y * q.v.z;
      double sx = q.s * q.v.x, sy = q.s * q.v.y, sz = q.s * q.v.z;
      return V3((ss + xx - yy - zz) * u.x + 2.0 * (xy - sz) * u.y + 2.0 * (xz + sy) * u.z,
                2.0 * (xy + sz) * u.x + (ss - xx + yy - zz) * u.y + 2.0 * (yz - sx) * u.z,
                2.0 * (xz - sy) * u.x + 2.0 * (yz + sx) * u.y + (ss - xx - yy + zz) * u.z);
    }
    case 6: {  // q (x) ((0,u) (x) q*)
      Quat p; p.s = 0.0; p.v = u;
      return qmul(q, qmul(p, qconj(q))).v;
    }
    case 7: {  // (2 s^2 - 1) u + 2 (v.u) v + 2 s (v x u)
      return (2.0 * q.s * q.s - 1.0) * u + 2.0 * (q.v * u) * q.v + 2.0 * q.s * cross(q.v, u);
    }
    case 8: {  // u + 2 s (v x u) + 2 (v (v.u) - u (v.v))
      return u + 2.0 * q.s * cross(q.v, u) + 2.0 * ((q.v * u) * q.v - (q.v * q.v) * u);
    }
    case 9: {  // (u + 2 v x (v x u)) + 2 s (v x u)
      V3 c = cross(q.v, u);
      return (u + 2.0 * cross(q.v, c)) + 2.0 * q.s * c;
    }
    case 10: {  // u + (2 s c + 2 v x c) with c = v x u
      V3 c = cross(q.v, u);
      return u + (2.0 * q.s * c + 2.0 * cross(q.v, c));
    }
    case 11: {  // u + 2 (s c + v x c)
      V3 c = cross(q.v, u);
      return u + 2.0 * (q.s * c + cross(q.v, c));
    }
    case 12: {  // explicit products written out: t = q (x) (0,u) ; r = t (x) q*
      double tw = -(q.v.x * u.x + q.v.y * u.y + q.v.z * u.z);
      double tx = q.s * u.x + q.v.y * u.z - q.v.z * u.y;
      double ty = q.s * u.y + q.v.z * u.x - q.v.x * u.z;
      double tz = q.s * u.z + q.v.x * u.y - q.v.y * u.x;
      return V3(-tw * q.v.x + tx * q.s - ty * q.v.z + tz * q.v.y,
                -tw * q.v.y + ty * q.s - tz * q.v.x + tx * q.v.z,
                -tw * q.v.z + tz * q.s - tx * q.v.y + ty * q.v.x);
    }
  }
}
// dQ/dt for a global-frame angular velocity w: 1/2 (0,w) (x) Q
static inline Quat qdot(const Quat& q, const V3& w) {
  Quat r;
  switch (g_var.qdot) {
    default:
    case 0:
      r.s = -0.5 * (w * q.v);
      r.v = 0.5 * (q.s * w + cross(w, q.v));
      break;
    case 1:
      r.s = -0.5 * (q.v.x * w.x + q.v.y * w.y + q.v.z * w.z);
      r.v.x = 0.5 * (q.s * w.x - q.v.z * w.y + q.v.y * w.z);
      r.v.y = 0.5 * (q.v.z * w.x + q.s * w.y - q.v.x * w.z);
      r.v.z = 0.5 * (-q.v.y * w.x + q.v.x * w.y + q.s * w.z);
      break;
    case 2: {  // body-frame convention 1/2 Q (x) (0,w)
      Quat p; p.s = 0.0; p.v = w;
      r = qmul(q, p);
      r.s *= 0.5; r.v *= 0.5;
    } break;
    case 3: {
      Quat p; p.s = 0.0; p.v = w;
      r = qmul(p, q);
      r.s *= 0.5; r.v *= 0.5;
    } break;
  }
  return r;
}
// d2Q/dt2 = 1/2 (0,a) (x) Q + 1/2 (0,w) (x) dQ/dt
static inline Quat qddot(const Quat& q, const V3& w, const V3& a) {
  Quat r;
  switch (g_var.qddot) {
    default:
    case 0: {  // 1/2 a(x)Q - 1/4 |w|^2 Q
      double w2 = w * w;
      r.s = -0.5 * (a * q.v) - 0.25 * w2 * q.s;
      r.v = 0.5 * (q.s * a + cross(a, q.v)) - 0.25 * w2 * q.v;
    } break;
    case 1: {  // through the first derivative
      Quat d = qdot(q, w);
      Quat pa; pa.s = 0.0; pa.v = a;
      Quat pw; pw.s = 0.0; pw.v = w;
      Quat t1 = qmul(pa, q), t2 = qmul(pw, d);
      r.s = 0.5 * (t1.s + t2.s);
      r.v = 0.5 * (t1.v + t2.v);
    } break;
    case 2: {  // body-frame convention
      Quat d = qdot(q, w);
      Quat pa; pa.s = 0.0; pa.v = a;
      Quat pw; pw.s = 0.0; pw.v = w;
      Quat t1 = qmul(q, pa), t2 = qmul(d, pw);
      r.s = 0.5 * (t1.s + t2.s);
      r.v = 0.5 * (t1.v + t2.v);
    } break;
    case 3: {
      double w2 = w * w;
      r.s = -0.5 * (q.v * a) - 0.25 * w2 * q.s;
      r.v.x = 0.5 * (q.s * a.x - q.v.z * a.y + q.v.y * a.z) - 0.25 * w2 * q.v.x;
      r.v.y = 0.5 * (q.v.z * a.x + q.s * a.y - q.v.x * a.z) - 0.25 * w2 * q.v.y;
      r.v.z = 0.5 * (-q.v.y * a.x + q.v.x * a.y + q.s * a.z) - 0.25 * w2 * q.v.z;
    } break;
  }
  return r;
}
static inline void qadd(Quat& a, const Quat& b) { a.s += b.s; a.v += b.v; }
static inline Quat qscale(Quat a, double f) { a.s *= f; a.v *= f; return a; }
static inline void qnormalize(Quat& q) {
  switch (g_var.qnorm) {
    default:
    case 0: {
      double n = sqrt(q.s * q.s + q.v.x * q.v.x + q.v.y * q.v.y + q.v.z * q.v.z);
      if (n > 0.0) { q.s /= n; q.v.x /= n; q.v.y /= n; q.v.z /= n; }
    } break;
    case 1: {
      double n = sqrt(q.s * q.s + q.v.x * q.v.x + q.v.y * q.v.y + q.v.z * q.v.z);
      if (n > 0.0) { double f = 1.0 / n; q.s *= f; q.v *= f; }
    } break;
    case 2: {
      double n = sqrt(q.v.x * q.v.x + q.v.y * q.v.y + q.v.z * q.v.z + q.s * q.s);
      if (n > 0.0) { q.s /= n; q.v.x /= n; q.v.y /= n; q.v.z /= n; }
    } break;
    case 3: {
      double n = sqrt(q.v * q.v + q.s * q.s);
      if (n > 0.0) { double f = 1.0 / n; q.s *= f; q.v *= f; }
    } break;
  }
}
// Rotation angle of a quaternion increment (used by the dynamic NL guard).
static inline double qangle(const Quat& q) {
  double s = q.s;
  if (s > 1.0) s = 1.0;
  if (s < -1.0) s = -1.0;
  return 2.0 * acos(s);
}

// ----------------------------------------------------------------- OBB ----
struct Obb {
  V3 center;
  V3 e[3]{V3(1, 0, 0), V3(0, 1, 0), V3(0, 0, 1)};
  V3 extent;
  void enlarge(double d) { extent.x += d; extent.y += d; extent.z += d; }
  void translate(const V3& t) { center += t; }
  void rotate(const Quat& q) {
    e[0] = qrot(q, e[0]);
    e[1] = qrot(q, e[1]);
    e[2] = qrot(q, e[2]);
    center = qrot(q, center);
  }
};
// Separating-axis test of two oriented boxes (15 axes).
static bool obb_intersect(const Obb& a, const Obb& b) {
  const double eps = 1e-12;
  double R[3][3], AR[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R[i][j] = a.e[i] * b.e[j];
      AR[i][j] = fabs(R[i][j]) + eps;
    }
  V3 d = b.center - a.center;
  double t[3] = {d * a.e[0], d * a.e[1], d * a.e[2]};
  double ra, rb;
  for (int i = 0; i < 3; i++) {
    ra = a.extent[i];
    rb = b.extent.x * AR[i][0] + b.extent.y * AR[i][1] + b.extent.z * AR[i][2];
    if (fabs(t[i]) > ra + rb) return false;
  }
  for (int j = 0; j < 3; j++) {
    ra = a.extent.x * AR[0][j] + a.extent.y * AR[1][j] + a.extent.z * AR[2][j];
    rb = b.extent[j];
    if (fabs(t[0] * R[0][j] + t[1] * R[1][j] + t[2] * R[2][j]) > ra + rb) return false;
  }
  for (int i = 0; i < 3; i++) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    for (int j = 0; j < 3; j++) {
      int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      ra = a.extent[i1] * AR[i2][j] + a.extent[i2] * AR[i1][j];
      rb = b.extent[j1] * AR[i][j2] + b.extent[j2] * AR[i][j1];
      double tt = t[i2] * R[i1][j] - t[i1] * R[i2][j];
      if (fabs(tt) > ra + rb) return false;
    }
  }
  return true;
}

// --------------------------------------------------------------- shape ----
// Shape.hpp:58-111 (the fields the hot path reads)
struct Shape {
  std::string name;
  double radius{0.0}, volume{0.0};
  char preCompDone{'n'};
  V3 inertia_mass;
  Obb obb;
  std::vector<V3> vertex;
  std::vector<std::pair<size_t, size_t>> edge;
  std::vector<std::vector<size_t>> face;
};

// ---------------------------------------------------------- data table ----
struct DataTable {
  std::map<std::string, size_t> id;
  std::vector<std::map<std::pair<int, int>, double>> tab;
  size_t ngroup{0};
  size_t add(const std::string& name) {
    auto it = id.find(name);
    if (it != id.end()) return it->second;
    size_t k = tab.size();
    id[name] = k;
    tab.emplace_back();
    return k;
  }
  void set(size_t k, int g1, int g2, double v) {
    tab[k][{g1, g2}] = v;
    tab[k][{g2, g1}] = v;
    ngroup = std::max(ngroup, (size_t)std::max(g1, g2) + 1);
  }
  double get(size_t k, int g1, int g2) const {
    auto it = tab[k].find({g1, g2});
    return it == tab[k].end() ? 0.0 : it->second;
  }
  bool defined(size_t k, int g1, int g2) const { return tab[k].count({g1, g2}) != 0; }
};

// -------------------------------------------------------- body, contact ----
struct Body {  // Particle.hpp:77-127
  int group{0}, cluster{0};
  V3 pos, vel, acc;
  Quat Q;
  V3 vrot, arot;
  Shape* shape{nullptr};
  size_t shape_id{0};
  double homothety{1.0};
  V3 inertia;
  double mass{0.0};
  V3 force, moment;
  Obb obb;
  double R() const { return homothety * shape->radius; }  // Particle.cpp:71
  V3 glob_vertex(size_t v) const { return pos + qrot(Q, homothety * shape->vertex[v]); }  // Particle.cpp:55-57
  V3 glob_face_vertex(size_t f, size_t v) const {  // Particle.cpp:63-65
    return pos + qrot(Q, homothety * shape->vertex[shape->face[f][v]]);
  }
  void update_obb() {  // Particle.cpp:78-86
    obb = shape->obb;
    obb.rotate(Q);
    obb.extent = homothety * obb.extent;
    obb.center = homothety * obb.center;
    obb.center += pos;
  }
};

enum { VV = 0, VE = 1, VF = 2, EE = 3 };

struct Key {  // lexicographic order of Interaction.hpp:106-122
  size_t i, j;
  int type;
  size_t isub, jsub;
  bool operator<(const Key& o) const {
    if (i != o.i) return i < o.i;
    if (j != o.j) return j < o.j;
    if (type != o.type) return type < o.type;
    if (isub != o.isub) return isub < o.isub;
    return jsub < o.jsub;
  }
};

struct Iface;
struct Contact {  // Interaction.hpp:57-100
  Key k;
  V3 prev_n, n;
  double dn{0.0}, prev_dn{0.0};
  V3 pos, vel;
  double fn{0.0};
  V3 ft, mom;
  double damp{0.0};
  Iface* stick{nullptr};
  void deactivate() {  // Interaction.cpp:123-128
    dn = prev_dn = 0.0;
    fn = 0.0;
    ft.reset();
    mom.reset();
  }
};

struct Iface {  // BreakableInterface.hpp:48-77
  size_t i{0}, j{0};
  double kn{0}, kt{0}, kr{0}, fn0{0}, ft0{0}, mom0{0}, power{2.0}, Gc{0};
  double dn0{0.0}, area{0.0};
  int isInner{1};
  std::vector<Contact*> bonds;
};

struct Control {  // DrivingSystem.hpp:70-75
  int type;
  size_t i;
  double value;
  V3 vec;
};
enum {
  X_VEL = 0, Y_VEL = 1, Z_VEL = 2, XROT_VEL = 3, YROT_VEL = 4, ZROT_VEL = 5,
  X_FOR = 6, Y_FOR = 7, Z_FOR = 8, XROT_MOM = 9, YROT_MOM = 10, ZROT_MOM = 11,
  XYZROT_VEL = 100, XYZROT_MOM = 101
};

static const double kPi = 3.14159265358979323846;

struct Sim {
  std::vector<Shape> shapes;
  std::map<std::string, size_t> shape_id;
  std::string shape_file{"noShapeFile"};
  std::string path;
  std::vector<Body> bodies;
  std::vector<std::map<Key, Contact>> inter;   // Rockable.hpp:107
  std::vector<std::map<size_t, Iface>> ifaces;  // Rockable.hpp:108 (keyed by j)
  std::vector<Contact*> active;
  std::vector<Contact*> flat;  // every entry in key order (Rockable.cpp:1598-1608)
  bool flat_dirty{true};
  std::vector<Iface*> to_break;
  std::map<std::string, std::string> options;
  DataTable table;
  std::map<int, double> density;
  // time
  double t{0.0}, tmax{1.0}, dt{1e-6};
  double dt_2{0.5e-6}, dt2_2{0.5e-12}, dt2{1e-12};
  double interVerlet{0.01}, interConf{0.25};
  double DVerlet{0.0}, dVerlet{0.0};
  V3 gravity{0.0, -9.81, 0.0};
  // BodyForce plugin (Rockable.cpp:1026-1040): 0 none, 1 AttractingPoint,
  // 2 PreferredDirection, 3 ViscousFluid, with their read() members
  // (BodyForce_AttractingPoint.cpp:43-45, BodyForce_PreferredDirection.cpp:
  // 43-48, BodyForce_ViscousFluid.cpp:42)
  int bf_kind{0};
  V3 bf_point;
  double bf_acceleration{0.0};
  V3 bf_axisBody, bf_axis;
  double bf_momentMax{0.0}, bf_Kr{0.0};
  double bf_fluidDensity{0.0};
  std::vector<double> bf_raw;  // the plugin's conf values as read
  int paramsInInterfaces{0};
  int dynamicUpdateNL{0};
  double dispUpdateNL{1.0}, angleUpdateNL{1.0};
  double numDamp{0.0};
  double velBarrier{0.0}, angVelBarrier{0.0}, velBarrierExp{1.0}, angVelBarrierExp{1.0};
  V3 cellMinSizes{1.0, 1.0, 1.0};
  int boxForLinkCellsOpt{0};
  int iconf{0};
  size_t nDriven{0};
  int precision{16};
  int law{0};  // 0 Default 1 Avalanche 2 StickedLinks
  bool nl_linkcells{false};
  std::string parallel_mode{"DefaultParallelMode"};
  // law parameter ids
  size_t idKn, idEn2, idKt, idMu, idKr, idMur, idViscT;
  size_t idKnI, idKtI, idKrI, idEn2I, idFn0I, idFt0I, idMom0I, idPowI;
  size_t idKnO, idKtO, idKrO, idEn2O, idFn0O, idFt0O, idMom0O, idPowO, idGcI, idGcO;
  // driving
  std::vector<Control> controls;
  bool servo{false};
  size_t servo_icontr{0}, sXmin{0}, sXmax{0}, sYmin{0}, sYmax{0}, sZmin{0}, sZmax{0};
  double servo_p{0.0};
  // flow
  double interVerletC{0.0}, interConfC{0.0};
  bool needUpdate{false};
  double maxDeltaPos{0.0}, maxDeltaRot{0.0};
  std::vector<V3> deltaPos;
  std::vector<Quat> deltaQ;
  double totalBrokenArea{0.0};
  long nbroken{0};

  Sim() {  // Rockable.cpp:78-127 (parameter ids)
    idKn = table.add("knContact"); idEn2 = table.add("en2Contact"); idKt = table.add("ktContact");
    idMu = table.add("muContact"); idKr = table.add("krContact"); idMur = table.add("murContact");
    idViscT = table.add("viscTContact");
    idKnI = table.add("knInnerBond"); idKtI = table.add("ktInnerBond"); idKrI = table.add("krInnerBond");
    idEn2I = table.add("en2InnerBond"); idFn0I = table.add("fn0InnerBond"); idFt0I = table.add("ft0InnerBond");
    idMom0I = table.add("mom0InnerBond"); idPowI = table.add("powInnerBond");
    idKnO = table.add("knOuterBond"); idKtO = table.add("ktOuterBond"); idKrO = table.add("krOuterBond");
    idEn2O = table.add("en2OuterBond"); idFn0O = table.add("fn0OuterBond"); idFt0O = table.add("ft0OuterBond");
    idMom0O = table.add("mom0OuterBond"); idPowO = table.add("powOuterBond");
    idGcI = table.add("gcInnerBond"); idGcO = table.add("gcOuterBond");
    options["forceLaw"] = "Default";
    options["AddOrRemoveInteractions"] = "bruteForce";
    options["UpdateNL"] = "bruteForce";
    options["Integrator"] = "velocityVerlet";
  }
  void set_dt(double v) {  // Rockable.cpp:645-654 and 2559-2565
    dt = v;
    dt_2 = 0.5 * dt;
    dt2_2 = dt_2 * dt;
    dt2 = dt * dt;
  }
};

// ------------------------------------------------------ narrow phase ----
// Interaction.cpp:143-326 (UpdateDispatcher).  Returns false when the
// sub-contact was deactivated.
static inline void contact_velocity(Contact& I, const Body& Pi, const Body& Pj) {
  I.vel = (Pj.vel - cross(I.pos - Pj.pos, Pj.vrot)) - (Pi.vel - cross(I.pos - Pi.pos, Pi.vrot));
}
static bool update_vv(Contact& I, const Body& Pi, const Body& Pj) {  // Interaction.cpp:147-165
  V3 posi = Pi.glob_vertex(I.k.isub);
  V3 posj = Pj.glob_vertex(I.k.jsub);
  double Ri = Pi.R(), Rj = Pj.R();
  I.prev_n = I.n;
  I.n = posi - posj;
  I.prev_dn = I.dn;
  I.dn = normalize(I.n) - (Ri + Rj);
  I.pos = posi - I.n * (Ri + 0.5 * I.dn);
  contact_velocity(I, Pi, Pj);
  return true;
}
static bool update_ve(Contact& I, const Body& Pi, const Body& Pj) {  // Interaction.cpp:169-198
  size_t v1 = Pj.shape->edge[I.k.jsub].first, v2 = Pj.shape->edge[I.k.jsub].second;
  V3 posj1 = Pj.glob_vertex(v1), posj2 = Pj.glob_vertex(v2);
  V3 posi = Pi.glob_vertex(I.k.isub);
  V3 E = posj2 - posj1;
  V3 v = posi - posj1;
  double r = (v * E) / (E * E);
  if (r <= 0.0 || r >= 1.0) { I.deactivate(); return false; }
  double Ri = Pi.R(), Rj = Pj.R();
  I.prev_n = I.n;
  I.n = posi - (posj1 + r * E);
  I.prev_dn = I.dn;
  I.dn = normalize(I.n) - (Ri + Rj);
  I.pos = posi - I.n * (Ri + 0.5 * I.dn);
  contact_velocity(I, Pi, Pj);
  return true;
}
static bool update_vf(Contact& I, const Body& Pi, const Body& Pj) {  // Interaction.cpp:202-271
  size_t nbv = Pj.shape->face[I.k.jsub].size();
  V3 A = Pj.glob_face_vertex(I.k.jsub, 0);
  V3 B = Pj.glob_face_vertex(I.k.jsub, 1);
  V3 C = Pj.glob_face_vertex(I.k.jsub, nbv - 1);
  V3 posi = Pi.glob_vertex(I.k.isub);
  V3 v = posi - A;
  V3 v1 = B - A;
  normalize(v1);
  V3 v2 = C - A;
  I.prev_n = I.n;
  I.n = cross(v1, v2);
  normalize(I.n);
  double dist = v * I.n;
  if (dist < 0.0) { I.n = -I.n; dist = -dist; }
  V3 P = posi - dist * I.n;
  int odd = 0;
  v2 = cross(I.n, v1);
  double ori1 = P * v1, ori2 = P * v2;
  for (size_t iva = 0; iva < nbv; ++iva) {
    size_t ivb = iva + 1;
    if (ivb == nbv) ivb = 0;
    V3 pa = Pj.glob_face_vertex(I.k.jsub, iva);
    V3 pb = Pj.glob_face_vertex(I.k.jsub, ivb);
    double pa1 = pa * v1, pb1 = pb * v1, pa2 = pa * v2, pb2 = pb * v2;
    if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
      if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
    }
  }
  if (odd) {
    double Ri = Pi.R(), Rj = Pj.R();
    I.prev_dn = I.dn;
    I.dn = dist - (Ri + Rj);
    I.pos = posi - I.n * (Ri + 0.5 * I.dn);
    contact_velocity(I, Pi, Pj);
    return true;
  }
  I.deactivate();
  return false;
}
static bool update_ee(Contact& I, const Body& Pi, const Body& Pj) {  // Interaction.cpp:275-326
  V3 pi1 = Pi.glob_vertex(Pi.shape->edge[I.k.isub].first);
  V3 pi2 = Pi.glob_vertex(Pi.shape->edge[I.k.isub].second);
  V3 pj1 = Pj.glob_vertex(Pj.shape->edge[I.k.jsub].first);
  V3 pj2 = Pj.glob_vertex(Pj.shape->edge[I.k.jsub].second);
  V3 Ei = pi2 - pi1, Ej = pj2 - pj1, v = pi1 - pj1;
  double c = Ei * Ei, d = Ej * Ej, e = Ei * Ej;
  double f = (c * d) - (e * e);
  double s, t;
  if (fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    double a = Ei * v, b = Ej * v;
    s = (e * b - a * d) * f;
    t = (c * b - e * a) * f;
    if (s <= 0.0 || s >= 1.0 || t <= 0.0 || t >= 1.0) { I.deactivate(); return false; }
    I.prev_n = I.n;
    I.n = (pi1 + s * Ei) - (pj1 + t * Ej);
  } else {
    I.deactivate();
    return false;
  }
  double Ri = Pi.R(), Rj = Pj.R();
  I.prev_dn = I.dn;
  I.dn = normalize(I.n) - (Ri + Rj);
  I.pos = pi1 + s * Ei - I.n * (Ri + 0.5 * I.dn);
  contact_velocity(I, Pi, Pj);
  return true;
}
static bool update_contact(Contact& I, const Body& Pi, const Body& Pj) {
  switch (I.k.type) {
    case VV: return update_vv(I, Pi, Pj);
    case VE: return update_ve(I, Pi, Pj);
    case VF: return update_vf(I, Pi, Pj);
    default: return update_ee(I, Pi, Pj);
  }
}

// ------------------------------------------------------ NEAR predicates ----
// Particle.cpp:88-209 (no periodic shift)
static bool near_vv(const Body& Pi, const Body& Pj, size_t isub, size_t jsub, double dmax) {
  V3 a = Pi.glob_vertex(isub), b = Pj.glob_vertex(jsub);
  double sum = Pi.R() + Pj.R() + dmax;
  return norm2(b - a) <= sum * sum;
}
static bool near_ve(const Body& Pi, const Body& Pj, size_t isub, size_t jsub, double dmax) {
  V3 piv = Pi.glob_vertex(isub);
  V3 p0 = Pj.glob_vertex(Pj.shape->edge[jsub].first), p1 = Pj.glob_vertex(Pj.shape->edge[jsub].second);
  V3 E = p1 - p0, v = piv - p0;
  double r = (v * E) / (E * E);
  if (r < -dmax) return false;
  if (r > 1.0 + dmax) return false;
  double sum = Pi.R() + Pj.R() + dmax;
  return norm2(piv - (p0 + r * E)) <= sum * sum;
}
static bool near_vf(const Body& Pi, const Body& Pj, size_t isub, size_t jsub, double dmax) {
  size_t nbv = Pj.shape->face[jsub].size();
  V3 A = Pj.glob_face_vertex(jsub, 0), B = Pj.glob_face_vertex(jsub, 1), C = Pj.glob_face_vertex(jsub, nbv - 1);
  V3 piv = Pi.glob_vertex(isub);
  V3 v = piv - A;
  V3 v1 = B - A;
  normalize(v1);
  V3 v2 = C - A;
  V3 n = cross(v1, v2);
  normalize(n);
  double dist = v * n;
  if (dist < 0.0) { n = -n; dist = -dist; }
  V3 P = piv - dist * n;
  int odd = 0;
  v2 = cross(n, v1);
  double ori1 = P * v1, ori2 = P * v2;
  for (size_t iva = 0; iva < nbv; ++iva) {
    size_t ivb = iva + 1;
    if (ivb == nbv) ivb = 0;
    V3 pa = Pj.glob_face_vertex(jsub, iva), pb = Pj.glob_face_vertex(jsub, ivb);
    double pa1 = pa * v1, pb1 = pb * v1, pa2 = pa * v2, pb2 = pb * v2;
    if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
      if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
    }
  }
  if (odd == 1) {
    dist -= (Pi.R() + Pj.R());
    if (dist <= dmax) return true;
  }
  return false;
}
static bool near_ee(const Body& Pi, const Body& Pj, size_t isub, size_t jsub, double dmax) {
  V3 pj0 = Pj.glob_vertex(Pj.shape->edge[jsub].first), pj1 = Pj.glob_vertex(Pj.shape->edge[jsub].second);
  V3 pi0 = Pi.glob_vertex(Pi.shape->edge[isub].first), pi1 = Pi.glob_vertex(Pi.shape->edge[isub].second);
  V3 Ei = pi1 - pi0, Ej = pj1 - pj0, v = pi0 - pj0;
  double c = Ei * Ei, d = Ej * Ej, e = Ei * Ej;
  double f = (c * d) - (e * e);
  if (fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    double a = Ei * v, b = Ej * v;
    double s = (e * b - a * d) * f;
    double t = (c * b - e * a) * f;
    if (s >= 0.0 && s <= 1.0 && t >= 0.0 && t <= 1.0) {
      V3 n = (pi0 + s * Ei) - (pj0 + t * Ej);
      double sum = Pi.R() + Pj.R() + dmax;
      return norm2(n) <= sum * sum;
    }
  }
  return false;
}

// ------------------------------------------------------------- damping ----
// Rockable.cpp:1356-1376: damping from en2 = e_n^2 and the effective mass.
static double contact_damping(const Sim& S, size_t i, size_t j, size_t idEn2, size_t idKn) {
  const Body& Pi = S.bodies[i];
  const Body& Pj = S.bodies[j];
  double en2 = S.table.get(idEn2, Pi.group, Pj.group);
  double kn = S.table.get(idKn, Pi.group, Pj.group);
  double meff;
  if (i < S.nDriven) meff = Pj.mass;
  else if (j < S.nDriven) meff = Pi.mass;
  else meff = (Pi.mass * Pj.mass) / (Pi.mass + Pj.mass);
  if (en2 > 0.0 && en2 < 1.0) {
    double logen = 0.5 * log(en2);
    double dampRate = -logen / sqrt(logen * logen + kPi * kPi);
    return dampRate * 2.0 * sqrt(kn * meff);
  } else if (en2 <= 0.0) {
    return 2.0 * sqrt(kn * meff);
  }
  return 0.0;
}

// --------------------------------------------------- neighbour list ----
typedef bool (*NearFn)(const Body&, const Body&, size_t, size_t, double);

// Rockable.cpp:1309-1432 (AddOrRemoveInteractions_bruteForce), in two
// phases so that the NEAR predicates of many body pairs can run in parallel
// (like the reference's OpenMP loop over link cells, Rockable.cpp:1697):
// eval_pair tests the pair's sub-element candidates against the geometry
// only and records the NEAR keys and which vertex-owned candidates were
// tested; apply_pair then inserts the new NEAR keys and erases the tested
// ones that are no longer NEAR.  A key belongs to one body pair only, so
// applying the pairs in visit order gives exactly the sets of the serial
// loop.
struct PairWork {
  size_t i, j;
  bool visit{false};        // the enlarged OBBs intersect
  double damp{0.0};
  std::vector<Key> near;    // NEAR keys, in key order
  std::vector<char> cull_i, cull_j;  // vertex-owned candidates of i (j) tested
};

static void eval_pair(const Sim& S, PairWork& w, double dmax) {
  const size_t i = w.i, j = w.j;
  w.damp = contact_damping(S, i, j, S.idEn2, S.idKn);
  auto single = [&](size_t i_, size_t j_, size_t isub, int type, size_t nbj, NearFn fn) {
    for (size_t jsub = 0; jsub < nbj; ++jsub)
      if (fn(S.bodies[i_], S.bodies[j_], isub, jsub, dmax)) w.near.push_back(Key{i_, j_, type, isub, jsub});
  };
  const Body& Pi = S.bodies[i];
  const Body& Pj = S.bodies[j];
  size_t nvi = Pi.shape->vertex.size(), nvj = Pj.shape->vertex.size();
  size_t nei = Pi.shape->edge.size(), nej = Pj.shape->edge.size();
  size_t nfi = Pi.shape->face.size(), nfj = Pj.shape->face.size();
  w.cull_i.assign(nvi, 0);
  w.cull_j.assign(nvj, 0);
  for (size_t isub = 0; isub < nvi; ++isub) {
    Obb sub;
    sub.center = Pi.glob_vertex(isub);
    sub.enlarge(Pi.R() + dmax);
    Obb obbj = Pj.obb;
    obbj.enlarge(dmax);
    if (!obb_intersect(obbj, sub)) continue;
    w.cull_i[isub] = 1;
    single(i, j, isub, VV, nvj, near_vv);
    single(i, j, isub, VE, nej, near_ve);
    single(i, j, isub, VF, nfj, near_vf);
  }
  for (size_t jsub = 0; jsub < nvj; ++jsub) {
    Obb sub;
    sub.center = Pj.glob_vertex(jsub);
    sub.enlarge(Pj.R() + dmax);
    Obb obbi = Pi.obb;
    obbi.enlarge(dmax);
    if (!obb_intersect(obbi, sub)) continue;
    w.cull_j[jsub] = 1;
    single(j, i, jsub, VE, nei, near_ve);
    single(j, i, jsub, VF, nfi, near_vf);
  }
  for (size_t isub = 0; isub < nei; ++isub) single(i, j, isub, EE, nej, near_ee);
  std::sort(w.near.begin(), w.near.end());  // key order, for apply_pair's lookups
}

static void apply_pair(Sim& S, const PairWork& w) {
  auto sweep = [&](size_t a, size_t b, const std::vector<char>& cull) {
    auto& set = S.inter[a];
    auto it = set.lower_bound(Key{a, b, 0, 0, 0});
    while (it != set.end() && it->first.i == a && it->first.j == b) {
      const Key& k = it->first;
      bool tested = (k.type == EE && a == w.i) || (k.isub < cull.size() && cull[k.isub] &&
                                                   (a == w.i ? (k.type == VV || k.type == VE || k.type == VF)
                                                             : (k.type == VE || k.type == VF)));
      bool isNear = tested && std::binary_search(w.near.begin(), w.near.end(), k);
      if (tested && !isNear) it = set.erase(it);
      else ++it;
    }
  };
  sweep(w.i, w.j, w.cull_i);
  sweep(w.j, w.i, w.cull_j);
  for (const Key& k : w.near) {
    auto& set = S.inter[k.i];
    if (set.find(k) == set.end()) {
      Contact c;
      c.k = k;
      c.damp = w.damp;
      set.emplace(k, c);
    }
  }
}

// The visited pairs of one list update: OBB test and NEAR predicates in
// parallel, the list changes in visit order.
static void process_pairs(Sim& S, std::vector<PairWork>& work) {
  const long np = (long)work.size();
#pragma omp parallel for schedule(dynamic, 16)
  for (long p = 0; p < np; ++p) {
    PairWork& w = work[p];
    Obb obbi = S.bodies[w.i].obb;
    obbi.enlarge(0.5 * S.DVerlet);
    Obb obbj = S.bodies[w.j].obb;
    obbj.enlarge(0.5 * S.DVerlet);
    w.visit = obb_intersect(obbi, obbj);
    if (w.visit) eval_pair(S, w, S.dVerlet);
  }
  for (long p = 0; p < np; ++p)
    if (work[p].visit) apply_pair(S, work[p]);
}

static bool has_iface(const Sim& S, size_t i, size_t j) {
  return S.ifaces[i].count(j) != 0;
}

// Rockable.cpp:1614-1662 (UpdateNL_bruteForce)
static void update_nl_bruteforce(Sim& S) {
  size_t N = S.bodies.size();
#pragma omp parallel for
  for (long i = 0; i < (long)N; ++i) S.bodies[i].update_obb();
  std::vector<PairWork> work;
  for (size_t i = 0; i < N; ++i) {
    size_t jnext = i + 1;
    if (jnext < S.nDriven) jnext = S.nDriven;
    for (size_t j = jnext; j < N; j++) {
      if (has_iface(S, i, j)) continue;
      PairWork w;
      w.i = i;
      w.j = j;
      work.push_back(std::move(w));
    }
  }
  process_pairs(S, work);
}

// Rockable.cpp:1667-1809 (UpdateNL_linkCells).  The cell grid follows the
// reference's use of toofus linkCells: the box is the AABB of all bodies
// (or of the free ones), the number of cells per axis is floor(L / minSize)
// (at least 1), bodies whose AABB is larger than a cell are "oversized" and
// tested against every cell, and each cell's neighbour list holds the 27
// surrounding cells (itself included).
static void compute_aabb(Sim& S, size_t first, std::vector<V3>& bmin, std::vector<V3>& bmax, V3& smin, V3& smax) {
  size_t N = S.bodies.size();
  bmin.resize(N);
  bmax.resize(N);
  for (size_t i = 0; i < N; i++) {  // Rockable.cpp:3925-3948
    const Body& P = S.bodies[i];
    double r = P.R();
    V3 a = P.glob_vertex(0), b = a;
    for (size_t v = 1; v < P.shape->vertex.size(); v++) {
      V3 g = P.glob_vertex(v);
      a.x = std::min(a.x, g.x); a.y = std::min(a.y, g.y); a.z = std::min(a.z, g.z);
      b.x = std::max(b.x, g.x); b.y = std::max(b.y, g.y); b.z = std::max(b.z, g.z);
    }
    a -= V3(r, r, r);
    b += V3(r, r, r);
    bmin[i] = a;
    bmax[i] = b;
  }
  smin = bmin[first];
  smax = bmax[first];
  for (size_t i = first + 1; i < N; i++) {
    smin.x = std::min(smin.x, bmin[i].x); smin.y = std::min(smin.y, bmin[i].y); smin.z = std::min(smin.z, bmin[i].z);
    smax.x = std::max(smax.x, bmax[i].x); smax.y = std::max(smax.y, bmax[i].y); smax.z = std::max(smax.z, bmax[i].z);
  }
}
static void update_nl_linkcells(Sim& S) {
  size_t N = S.bodies.size();
#pragma omp parallel for
  for (long i = 0; i < (long)N; ++i) S.bodies[i].update_obb();
  std::vector<V3> bmin, bmax;
  V3 smin, smax;
  compute_aabb(S, S.boxForLinkCellsOpt == 1 ? S.nDriven : 0, bmin, bmax, smin, smax);
  int n[3];
  double cs[3];
  for (int d = 0; d < 3; d++) {
    double L = smax[d] - smin[d];
    n[d] = (int)floor(L / S.cellMinSizes[d]);
    if (n[d] < 1) n[d] = 1;
    cs[d] = L / n[d];
    if (!(cs[d] > 0.0)) cs[d] = 1.0;
  }
  std::vector<std::vector<size_t>> cells((size_t)n[0] * n[1] * n[2]);
  std::vector<size_t> oversized;
  for (size_t i = 0; i < N; i++) {
    bool big = false;
    for (int d = 0; d < 3; d++)
      if (bmax[i][d] - bmin[i][d] > cs[d]) big = true;
    if (big) { oversized.push_back(i); continue; }
    int c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (int)floor((S.bodies[i].pos[d] - smin[d]) / cs[d]);
      if (c[d] < 0) c[d] = 0;
      if (c[d] >= n[d]) c[d] = n[d] - 1;
    }
    cells[((size_t)c[0] * n[1] + c[1]) * n[2] + c[2]].push_back(i);
  }
  std::vector<PairWork> work;
  auto visit = [&](size_t i, size_t j) {
    if (j < S.nDriven && i < S.nDriven) return;
    if (j <= i) return;
    if (has_iface(S, i, j)) return;
    PairWork w;
    w.i = i;
    w.j = j;
    work.push_back(std::move(w));
  };
  for (int ix = 0; ix < n[0]; ix++)
    for (int iy = 0; iy < n[1]; iy++)
      for (int iz = 0; iz < n[2]; iz++) {
        auto& Cc = cells[((size_t)ix * n[1] + iy) * n[2] + iz];
        for (int dx = -1; dx <= 1; dx++)
          for (int dy = -1; dy <= 1; dy++)
            for (int dz = -1; dz <= 1; dz++) {
              int jx = ix + dx, jy = iy + dy, jz = iz + dz;
              if (jx < 0 || jy < 0 || jz < 0 || jx >= n[0] || jy >= n[1] || jz >= n[2]) continue;
              auto& Cv = cells[((size_t)jx * n[1] + jy) * n[2] + jz];
              for (size_t a : Cc)
                for (size_t b : Cv) visit(a, b);
            }
      }
  for (auto& Cv : cells)
    for (size_t a : oversized)
      for (size_t b : Cv) visit(a, b);
  process_pairs(S, work);
}

static void update_nl(Sim& S) {
  if (S.nl_linkcells) update_nl_linkcells(S);
  else update_nl_bruteforce(S);
  S.flat_dirty = true;
}

// ----------------------------------------------------------- force laws ----
// ForceLaw_Default.cpp:57-131
static void law_default(Sim& S, Contact& I) {
  if (I.dn > 0.0) { I.fn = 0.0; I.ft.reset(); I.mom.reset(); return; }
  const Body& Pi = S.bodies[I.k.i];
  const Body& Pj = S.bodies[I.k.j];
  int g1 = Pi.group, g2 = Pj.group;
  double kn = S.table.get(S.idKn, g1, g2), kt = S.table.get(S.idKt, g1, g2);
  double mu = S.table.get(S.idMu, g1, g2), kr = S.table.get(S.idKr, g1, g2);
  double mur = S.table.get(S.idMur, g1, g2);
  double damp = I.damp;
  double vn = I.vel * I.n;
  double fne = -kn * I.dn;
  double fnv = damp * vn;
  I.fn = fne + fnv;
  if (I.fn < 0.0) I.fn = 0.0;
  V3 vt = I.vel - vn * I.n;
  I.ft += kt * (vt * S.dt);
  double threshold = fabs(mu * fne);
  double ft_square = I.ft * I.ft;
  if (ft_square > 0.0 && ft_square >= threshold * threshold) I.ft *= threshold / sqrt(ft_square);
  if (kr > 0.0) {
    I.mom += kr * (Pj.vrot - Pi.vrot) * S.dt;
    double threshold_mom = fabs(mur * I.fn);
    double mom_square = I.mom * I.mom;
    if (mom_square > 0.0 && mom_square >= threshold_mom * threshold_mom) I.mom *= threshold_mom / sqrt(mom_square);
  }
}
// ForceLaw_Avalanche.cpp:57-136
static void law_avalanche(Sim& S, Contact& I) {
  if (I.dn > 0.0) { I.fn = 0.0; I.ft.reset(); I.mom.reset(); return; }
  const Body& Pi = S.bodies[I.k.i];
  const Body& Pj = S.bodies[I.k.j];
  int g1 = Pi.group, g2 = Pj.group;
  double kn = S.table.get(S.idKn, g1, g2), en2 = S.table.get(S.idEn2, g1, g2);
  double kt = S.table.get(S.idKt, g1, g2), mu = S.table.get(S.idMu, g1, g2);
  double kr = S.table.get(S.idKr, g1, g2), mur = S.table.get(S.idMur, g1, g2);
  if (I.prev_dn > 0.0) I.prev_dn = 0.0;
  double delta_Dn = I.dn - I.prev_dn;
  if (delta_Dn > 0.0) I.fn = -kn * en2 * I.dn;
  else if (delta_Dn < 0.0) I.fn += -kn * delta_Dn;
  if (I.fn < 0.0) I.fn = 0.0;
  V3 vt = I.vel - (I.vel * I.n) * I.n;
  I.ft += kt * (S.dt * vt);
  double threshold_ft = fabs(mu * I.fn);
  double ft_square = I.ft * I.ft;
  if (ft_square > 0.0 && ft_square > threshold_ft * threshold_ft) I.ft *= threshold_ft / sqrt(ft_square);
  I.mom += kr * (Pj.vrot - Pi.vrot) * S.dt;
  V3 branch;
  if (I.k.i < S.nDriven) {
    branch = I.pos - Pj.pos;
    double r = (branch * Pj.vrot) / (Pj.vrot * Pj.vrot);
    branch -= r * Pj.vrot;
  } else {
    branch = I.pos - Pi.pos;
    double r = (branch * Pi.vrot) / (Pi.vrot * Pi.vrot);
    branch -= r * Pi.vrot;
  }
  double threshold_mom = fabs(mur * norm(branch) * I.fn);
  double mom_square = I.mom * I.mom;
  if (mom_square > 0.0 && mom_square > threshold_mom * threshold_mom) I.mom *= threshold_mom / sqrt(mom_square);
}
// ForceLaw_StickedLinks.cpp:75-215
static void law_sticked(Sim& S, Contact& I, std::vector<Iface*>& to_break) {
  const Body& Pi = S.bodies[I.k.i];
  const Body& Pj = S.bodies[I.k.j];
  if (I.stick != nullptr) {
    double kn = 0, kt = 0, kr = 0, fn0 = 1, ft0 = 1, mom0 = 1, power = 1;
    double dn0 = I.stick->dn0;
    bool isInner = (Pi.cluster == Pj.cluster);
    if (S.paramsInInterfaces == 1) {
      kn = I.stick->kn; kt = I.stick->kt; kr = I.stick->kr;
      fn0 = I.stick->fn0; ft0 = I.stick->ft0; mom0 = I.stick->mom0; power = I.stick->power;
    } else {
      int g1 = Pi.group, g2 = Pj.group;
      if (isInner) {
        kn = S.table.get(S.idKnI, g1, g2); kt = S.table.get(S.idKtI, g1, g2); kr = S.table.get(S.idKrI, g1, g2);
        fn0 = S.table.get(S.idFn0I, g1, g2); ft0 = S.table.get(S.idFt0I, g1, g2);
        mom0 = S.table.get(S.idMom0I, g1, g2); power = S.table.get(S.idPowI, g1, g2);
        dn0 = 0.0;
      } else {
        kn = S.table.get(S.idKnO, g1, g2); kt = S.table.get(S.idKtO, g1, g2); kr = S.table.get(S.idKrO, g1, g2);
        fn0 = S.table.get(S.idFn0O, g1, g2); ft0 = S.table.get(S.idFt0O, g1, g2);
        mom0 = S.table.get(S.idMom0O, g1, g2); power = S.table.get(S.idPowO, g1, g2);
      }
    }
    double vn = I.vel * I.n;
    double fne = -kn * (I.dn - dn0);
    double fnv = I.damp * vn;
    I.fn = fne + fnv;
    V3 vt = (I.vel - (vn * I.n));
    I.ft += kt * (vt * S.dt);
    V3 ftv = I.damp * vt;
    I.ft += ftv;
    I.mom += kr * (Pj.vrot - Pi.vrot) * S.dt;
    double yield = pow(norm(I.ft) / ft0, power) + pow(norm(I.mom) / mom0, power) - I.fn / fn0 - 1.0;
    if (yield > 0.0) to_break.push_back(I.stick);
  } else {
    if (I.dn > 0.0) { I.fn = 0.0; I.ft.reset(); I.mom.reset(); return; }
    int g1 = Pi.group, g2 = Pj.group;
    double kn = S.table.get(S.idKn, g1, g2), kt = S.table.get(S.idKt, g1, g2);
    double mu = S.table.get(S.idMu, g1, g2), kr = S.table.get(S.idKr, g1, g2);
    double mur = S.table.get(S.idMur, g1, g2);
    double damp = I.damp;
    double vn = I.vel * I.n;
    double fne = -kn * I.dn;
    double fnv = damp * vn;
    I.fn = fne + fnv;
    if (I.fn < 0.0) I.fn = 0.0;
    V3 vt = I.vel - vn * I.n;
    I.ft += kt * (vt * S.dt);
    double threshold = fabs(mu * I.fn);
    double ft_square = I.ft * I.ft;
    if (ft_square > 0.0 && ft_square >= threshold * threshold) I.ft *= threshold / sqrt(ft_square);
    I.mom += kr * (Pj.vrot - Pi.vrot) * S.dt;
    double threshold_mom = fabs(mur * I.fn);
    double mom_square = I.mom * I.mom;
    if (mom_square > 0.0 && mom_square >= threshold_mom * threshold_mom) I.mom *= threshold_mom / sqrt(mom_square);
  }
}

// --------------------------------------------------------- accelerations ----
// The BodyForce plugins' getForceAndMoment (force and moment start at zero,
// each plugin sets one of them)
static void body_force(const Sim& S, const Body& P, V3& force, V3& moment) {
  if (S.bf_kind == 1) {  // BodyForce_AttractingPoint.cpp:51-59
    V3 direction = S.bf_point - P.pos;
    double l2 = norm2(direction);
    if (l2 > 0.0) {
      direction *= 1.0 / sqrt(l2);
      force = P.mass * S.bf_acceleration * direction;
    }
  } else if (S.bf_kind == 2) {  // BodyForce_PreferredDirection.cpp:58-80
    V3 axisB = qrot(P.Q, S.bf_axisBody);
    normalize(axisB);
    V3 u = cross(S.bf_axis, axisB);
    normalize(u);
    double cosa = axisB * S.bf_axis;
    double angle = acos(cosa);
    double sgn = -1.0;
    if (cosa < 0.0) {
      sgn = 1.0;
      angle = kPi - angle;
    }
    moment = S.bf_Kr * sgn * u * angle;
  } else if (S.bf_kind == 3) {  // BodyForce_ViscousFluid.cpp:47-58
    const double two_thirds = 2.0 / 3.0, half_cx_sphere = 0.5 * 0.47;
    V3 velSqr(P.vel.x * P.vel.x, P.vel.y * P.vel.y, P.vel.z * P.vel.z);
    double h = P.homothety;
    double pVolume = P.shape->volume * h * h * h;
    double pSurface = pow(pVolume, two_thirds);
    force = half_cx_sphere * S.bf_fluidDensity * pSurface * velSqr;
  }
}

// Rockable.cpp:2869-2929
static void init_forces(Sim& S) {
  for (size_t i = 0; i < S.nDriven && i < S.bodies.size(); ++i) {
    Body& P = S.bodies[i];
    P.force.reset(); P.acc.reset(); P.moment.reset(); P.arot.reset();
  }
  for (size_t i = S.nDriven; i < S.bodies.size(); ++i) {
    S.bodies[i].force.reset();
    S.bodies[i].moment.reset();
    if (S.bf_kind != 0) {
      V3 force_more, moment_more;
      body_force(S, S.bodies[i], force_more, moment_more);
      S.bodies[i].force += force_more;
      S.bodies[i].moment += moment_more;
    }
  }
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    switch (c.type) {
      case X_FOR: P.force.x = c.value; break;
      case Y_FOR: P.force.y = c.value; break;
      case Z_FOR: P.force.z = c.value; break;
      case XROT_MOM: P.moment.x = c.value; break;
      case YROT_MOM: P.moment.y = c.value; break;
      case ZROT_MOM: P.moment.z = c.value; break;
      case XYZROT_MOM: P.moment = c.vec; break;
      default: break;
    }
  }
}

// Rockable.cpp:2752-2789
static void increment_resultants(Sim& S, const Contact& I) {
  V3 f = I.fn * I.n + I.ft;
  Body& Pi = S.bodies[I.k.i];
  Body& Pj = S.bodies[I.k.j];
  Pi.force += f;
  Pj.force -= f;
  V3 Ci = (I.pos - Pi.pos);
  V3 Cj = (I.pos - Pj.pos);
  Pi.moment += cross(Ci, f) + I.mom;
  Pj.moment += cross(Cj, -f) - I.mom;
}

static inline V3 euler_domega(const Body& P, const V3& omega, const V3& M) {
  return V3((M[0] - (P.inertia[2] - P.inertia[1]) * omega[1] * omega[2]) / P.inertia[0],
            (M[1] - (P.inertia[0] - P.inertia[2]) * omega[2] * omega[0]) / P.inertia[1],
            (M[2] - (P.inertia[1] - P.inertia[0]) * omega[0] * omega[1]) / P.inertia[2]);
}

// Rockable.cpp:3419-3552 (non-periodic part)
static void accelerations_from_resultants(Sim& S) {
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    switch (c.type) {
      case X_FOR: P.acc.x = P.force.x / P.mass; break;
      case Y_FOR: P.acc.y = P.force.y / P.mass; break;
      case Z_FOR: P.acc.z = P.force.z / P.mass; break;
      case XROT_MOM: case YROT_MOM: case ZROT_MOM: case XYZROT_MOM: {
        Quat Qinv = qconj(P.Q);
        V3 w;
        if (c.type == XROT_MOM) w = V3(P.vrot.x, 0, 0);
        else if (c.type == YROT_MOM) w = V3(0, P.vrot.y, 0);
        else if (c.type == ZROT_MOM) w = V3(0, 0, P.vrot.z);
        else w = P.vrot;
        V3 omega = qrot(Qinv, w);
        V3 M = qrot(Qinv, P.moment);
        V3 dw = qrot(P.Q, euler_domega(P, omega, M));
        if (c.type == XROT_MOM) P.arot.x = dw.x;
        else if (c.type == YROT_MOM) P.arot.y = dw.y;
        else if (c.type == ZROT_MOM) P.arot.z = dw.z;
        else P.arot = dw;
      } break;
      default: break;
    }
  }
  const long nb = (long)S.bodies.size();
#pragma omp parallel for schedule(static)
  for (long i = (long)S.nDriven; i < nb; ++i) {
    Body& P = S.bodies[i];
    P.acc = vdiv(P.force, P.mass) + S.gravity;
    Quat Qinv = qconj(P.Q);
    V3 omega = qrot(Qinv, P.vrot);
    V3 M = qrot(Qinv, P.moment);
    P.arot = qrot(P.Q, euler_domega(P, omega, M));
  }
}

// Rockable.cpp:3806-3868 (not component-wise)
static void numerical_damping(Sim& S) {
  double fm = 1.0 - S.numDamp, fp = 1.0 + S.numDamp;
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    double factor;
    switch (c.type) {
      case X_FOR: factor = (P.force.x * P.vel.x > 0.0) ? fm : fp; P.force.x *= factor; break;
      case Y_FOR: factor = (P.force.y * P.vel.y > 0.0) ? fm : fp; P.force.y *= factor; break;
      case Z_FOR: factor = (P.force.z * P.vel.z > 0.0) ? fm : fp; P.force.z *= factor; break;
      default: break;
    }
  }
  for (size_t i = S.nDriven; i < S.bodies.size(); ++i) {
    Body& P = S.bodies[i];
    double factor = (P.force * P.vel > 0.0) ? fm : fp;
    P.force *= factor;
    factor = (P.moment * P.vrot > 0.0) ? fm : fp;
    P.moment *= factor;
  }
}

// Rockable.cpp:3350-3413
static void breakage(Sim& S) {
  // interfacesToBreak is a std::set ordered by (i, j)
  std::sort(S.to_break.begin(), S.to_break.end(), [](const Iface* a, const Iface* b) {
    if (a->i != b->i) return a->i < b->i;
    return a->j < b->j;
  });
  S.to_break.erase(std::unique(S.to_break.begin(), S.to_break.end()), S.to_break.end());
  for (Iface* BI : S.to_break) {
    int g1 = S.bodies[BI->i].group, g2 = S.bodies[BI->j].group;
    for (Contact* c : BI->bonds) {
      c->stick = nullptr;
      if (c->dn >= 0.0) {
        c->fn = 0.0;
        c->ft.reset();
      } else {
        V3 T = c->ft;
        double FT = normalize(T);
        double mu = S.table.get(S.idMu, g1, g2);
        double thr = fabs(mu * c->fn);
        if (FT > thr) c->ft = thr * T;
      }
    }
    S.totalBrokenArea += BI->area;
    S.nbroken++;
    size_t bi = BI->i, bj = BI->j;
    S.ifaces[bi].erase(bj);
    S.needUpdate = true;
  }
}

// Rockable.cpp:3562-3719 (DefaultParallelMode)
static void accelerations(Sim& S) {
  init_forces(S);
  S.active.clear();
  S.to_break.clear();
  if (S.flat_dirty) {
    S.flat.clear();
    for (size_t k = 0; k < S.inter.size(); ++k)
      for (auto& kv : S.inter[k]) S.flat.push_back(&kv.second);
    S.flat_dirty = false;
  }
  // update_interactions (2934-2977): every NL entry (independent per entry)
  const long nflat = (long)S.flat.size();
#pragma omp parallel for schedule(static)
  for (long k = 0; k < nflat; ++k) {
    Contact& c = *S.flat[k];
    update_contact(c, S.bodies[c.k.i], S.bodies[c.k.j]);
  }
  // build_activeInteractions (3005-3029), in key order
  for (Contact* c : S.flat)
    if (c->dn < 0.0 || c->stick != nullptr) S.active.push_back(c);
  // compute_forces_and_moments (3035-3046): independent per entry; the
  // rupture requests are collected per thread and merged (sorted later)
  const long nact = (long)S.active.size();
#pragma omp parallel
  {
    std::vector<Iface*> mine;
#pragma omp for schedule(static)
    for (long k = 0; k < nact; ++k) {
      Contact* I = S.active[k];
      if (I->dn < 0.0 || I->stick != nullptr) {
        if (S.law == 1) law_avalanche(S, *I);
        else if (S.law == 2) law_sticked(S, *I, mine);
        else law_default(S, *I);
      }
    }
#pragma omp critical
    S.to_break.insert(S.to_break.end(), mine.begin(), mine.end());
  }
  // compute_resultants (3220-3275)
  for (Contact* I : S.active)
    if (I->dn < 0.0 || I->stick != nullptr) increment_resultants(S, *I);
  breakage(S);
  if (S.numDamp > 0.0) numerical_damping(S);
  accelerations_from_resultants(S);
  if (S.velBarrier > 0.0) {  // Rockable.cpp:3879-3893
    for (auto& P : S.bodies) {
      double rx = pow(fabs(P.vel.x / S.velBarrier), S.velBarrierExp);
      P.acc.x *= (1.0 - rx) / (1.0 + rx);
      double ry = pow(fabs(P.vel.y / S.velBarrier), S.velBarrierExp);
      P.acc.y *= (1.0 - ry) / (1.0 + ry);
      double rz = pow(fabs(P.vel.z / S.velBarrier), S.velBarrierExp);
      P.acc.z *= (1.0 - rz) / (1.0 + rz);
    }
  }
  if (S.angVelBarrier > 0.0) {  // Rockable.cpp:3899-3911
    for (auto& P : S.bodies) {
      double rx = pow(fabs(P.vrot.x / S.angVelBarrier), S.angVelBarrierExp);
      P.arot.x *= (1.0 - rx) / (1.0 + rx);
      double ry = pow(fabs(P.vrot.y / S.angVelBarrier), S.angVelBarrierExp);
      P.arot.y *= (1.0 - ry) / (1.0 + ry);
      double rz = pow(fabs(P.vrot.z / S.angVelBarrier), S.angVelBarrierExp);
      P.arot.z *= (1.0 - rz) / (1.0 + rz);
    }
  }
}

// ------------------------------------------------------- velocity Verlet ----
// DrivingSystem.cpp:251-268 (tritriIsostaticCompression)
static void servo(Sim& S) {
  if (!S.servo) return;
  const Body& a = S.bodies[S.sXmin]; const Body& b = S.bodies[S.sXmax];
  const Body& c = S.bodies[S.sYmin]; const Body& d = S.bodies[S.sYmax];
  const Body& e = S.bodies[S.sZmin]; const Body& f = S.bodies[S.sZmax];
  const double Xmin = a.pos.x + a.R(), Xmax = b.pos.x - b.R();
  const double Ymin = c.pos.y + c.R(), Ymax = d.pos.y - d.R();
  const double Zmin = e.pos.z + e.R(), Zmax = f.pos.z - f.R();
  const double dX = fabs(Xmax - Xmin), dY = fabs(Ymax - Ymin), dZ = fabs(Zmax - Zmin);
  const double surfX = dY * dZ, surfY = dX * dZ, surfZ = dY * dX;
  S.controls[S.servo_icontr + 1].value = -S.servo_p * surfX;
  S.controls[S.servo_icontr + 3].value = -S.servo_p * surfY;
  S.controls[S.servo_icontr + 5].value = -S.servo_p * surfZ;
}

// Rockable.cpp:1856-1900
static void velocity_controlled_drive(Sim& S) {
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    switch (c.type) {
      case X_VEL: P.vel.x = c.value; P.pos.x += S.dt * c.value; break;
      case Y_VEL: P.vel.y = c.value; P.pos.y += S.dt * c.value; break;
      case Z_VEL: P.vel.z = c.value; P.pos.z += S.dt * c.value; break;
      case XROT_VEL: case YROT_VEL: case ZROT_VEL: case XYZROT_VEL: {
        V3 w;
        if (c.type == XROT_VEL) w = V3(c.value, 0, 0);
        else if (c.type == YROT_VEL) w = V3(0, c.value, 0);
        else if (c.type == ZROT_VEL) w = V3(0, 0, c.value);
        else w = c.vec;
        qadd(P.Q, qscale(qdot(P.Q, w), S.dt));
        qnormalize(P.Q);
      } break;
      default: break;
    }
  }
}

// Rockable.cpp:1979-2158 (non-periodic)
static void verlet_step(Sim& S) {
  servo(S);
  velocity_controlled_drive(S);
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    switch (c.type) {
      case X_FOR: P.pos.x += S.dt * P.vel.x + S.dt2_2 * P.acc.x; P.vel.x += S.dt_2 * P.acc.x; break;
      case Y_FOR: P.pos.y += S.dt * P.vel.y + S.dt2_2 * P.acc.y; P.vel.y += S.dt_2 * P.acc.y; break;
      case Z_FOR: P.pos.z += S.dt * P.vel.z + S.dt2_2 * P.acc.z; P.vel.z += S.dt_2 * P.acc.z; break;
      case XROT_MOM: case YROT_MOM: case ZROT_MOM: case XYZROT_MOM: {
        V3 w;
        if (c.type == XROT_MOM) w = P.vrot.x * V3(1, 0, 0);
        else if (c.type == YROT_MOM) w = P.vrot.y * V3(0, 1, 0);
        else if (c.type == ZROT_MOM) w = P.vrot.z * V3(0, 0, 1);
        else w = P.vrot;
        qadd(P.Q, qscale(qdot(P.Q, w), S.dt));
        qnormalize(P.Q);
        if (c.type == XROT_MOM) P.vrot.x += S.dt_2 * P.arot.x;
        else if (c.type == YROT_MOM) P.vrot.y += S.dt_2 * P.arot.y;
        else if (c.type == ZROT_MOM) P.vrot.z += S.dt_2 * P.arot.z;
        else P.vrot += S.dt_2 * P.arot;
      } break;
      default: break;
    }
  }
  const long nb = (long)S.bodies.size();
#pragma omp parallel for schedule(static)
  for (long i = (long)S.nDriven; i < nb; ++i) {
    Body& P = S.bodies[i];
    P.pos += S.dt * P.vel + S.dt2_2 * P.acc;
    P.vel += S.dt_2 * P.acc;
    qadd(P.Q, qscale(qdot(P.Q, P.vrot), S.dt));
    qadd(P.Q, qscale(qddot(P.Q, P.vrot, P.arot), S.dt2_2));
    qnormalize(P.Q);
    P.vrot += S.dt_2 * P.arot;
  }
  accelerations(S);
  for (auto& c : S.controls) {
    Body& P = S.bodies[c.i];
    switch (c.type) {
      case X_FOR: P.vel.x += S.dt_2 * P.acc.x; break;
      case Y_FOR: P.vel.y += S.dt_2 * P.acc.y; break;
      case Z_FOR: P.vel.z += S.dt_2 * P.acc.z; break;
      case XROT_MOM: P.vrot.x += S.dt_2 * P.arot.x; break;
      case YROT_MOM: P.vrot.y += S.dt_2 * P.arot.y; break;
      case ZROT_MOM: P.vrot.z += S.dt_2 * P.arot.z; break;
      case XYZROT_MOM: P.vrot += S.dt_2 * P.arot; break;
      default: break;
    }
  }
#pragma omp parallel for schedule(static)
  for (long i = (long)S.nDriven; i < nb; ++i) {
    Body& P = S.bodies[i];
    P.vel += S.dt_2 * P.acc;
    P.vrot += S.dt_2 * P.arot;
  }
}

// Rockable.cpp:1571-1596
static void dynamic_check(Sim& S) {
  for (size_t i = 0; i < S.deltaPos.size(); ++i) {
    S.deltaPos[i] += S.bodies[i].vel * S.dt;
    double t1 = norm2(S.deltaPos[i]);
    if (t1 > S.maxDeltaPos * S.maxDeltaPos) S.maxDeltaPos = sqrt(t1);
    qadd(S.deltaQ[i], qscale(qdot(S.bodies[i].Q, S.bodies[i].vrot), S.dt));
    double t2 = qangle(S.deltaQ[i]);
    if (t2 > S.maxDeltaRot) S.maxDeltaRot = t2;
  }
  if (S.maxDeltaPos >= S.dispUpdateNL || S.maxDeltaRot >= S.angleUpdateNL) {
    S.needUpdate = true;
    for (size_t i = 0; i < S.deltaPos.size(); ++i) { S.deltaPos[i].reset(); S.deltaQ[i].reset(); }
    S.maxDeltaPos = 0.0;
    S.maxDeltaRot = 0.0;
  }
}

// ------------------------------------------------------------- parsing ----
static bool read_v3(std::istream& is, V3& v) { return (bool)(is >> v.x >> v.y >> v.z); }
static bool read_q(std::istream& is, Quat& q) { return (bool)(is >> q.s >> q.v.x >> q.v.y >> q.v.z); }

static std::string dirname_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string("") : p.substr(0, k + 1);
}
static bool file_exists(const std::string& p) {
  std::ifstream f(p);
  return f.good();
}

// Shape.cpp:69-128 and Rockable.cpp:1187-1225
static bool load_shapes(Sim& S, const std::string& fname) {
  std::ifstream is(fname);
  if (!is) { g_err = "cannot open shape file " + fname; return false; }
  S.shapes.clear();
  S.shape_id.clear();
  std::string tok;
  while (is >> tok) {
    if (tok != "<") continue;
    Shape sh;
    while (is >> tok) {
      if (tok == ">") break;
      if (tok == "name") is >> sh.name;
      else if (tok == "radius") is >> sh.radius;
      else if (tok == "preCompDone") is >> sh.preCompDone;
      else if (tok == "volume") is >> sh.volume;
      else if (tok == "I/m") read_v3(is, sh.inertia_mass);
      else if (tok == "obb.extent") read_v3(is, sh.obb.extent);
      else if (tok == "obb.center") read_v3(is, sh.obb.center);
      else if (tok == "obb.e1") read_v3(is, sh.obb.e[0]);
      else if (tok == "obb.e2") read_v3(is, sh.obb.e[1]);
      else if (tok == "obb.e3") read_v3(is, sh.obb.e[2]);
      else if (tok == "OBBtreeLevel" || tok == "MCnstep" || tok == "fibObbOption") { std::string x; is >> x; }
      else if (tok == "position") { V3 p; read_v3(is, p); }
      else if (tok == "orientation") { Quat q; read_q(is, q); }
      else if (tok == "isSurface") {}
      else if (tok == "nv") {
        size_t nv; is >> nv;
        for (size_t v = 0; v < nv; ++v) { V3 p; read_v3(is, p); sh.vertex.push_back(p); }
      } else if (tok == "ne") {
        size_t ne; is >> ne;
        for (size_t e = 0; e < ne; ++e) { size_t a, b; is >> a >> b; sh.edge.push_back({a, b}); }
      } else if (tok == "nf") {
        size_t nf; is >> nf;
        for (size_t f = 0; f < nf; ++f) {
          size_t k; is >> k;
          std::vector<size_t> ids(k);
          for (size_t n = 0; n < k; ++n) is >> ids[n];
          sh.face.push_back(ids);
        }
      }
    }
    if (sh.preCompDone != 'y') {
      g_err = "shape " + sh.name + " has preCompDone n (mass properties must be precomputed)";
      return false;
    }
    S.shapes.push_back(sh);
  }
  for (size_t s = 0; s < S.shapes.size(); ++s) S.shape_id[S.shapes[s].name] = s;
  return true;
}

// drivingSystem.txt: DrivingSystem.cpp:44-497 (Control lines and the
// tritriIsostaticCompression servo)
static bool read_driving(Sim& S, const std::string& fname) {
  std::ifstream is(fname);
  if (!is) { g_err = "cannot open " + fname; return false; }
  static const std::map<std::string, int> types = {
      {"_x_Vel_", X_VEL}, {"_y_Vel_", Y_VEL}, {"_z_Vel_", Z_VEL}, {"_xrot_Vel_", XROT_VEL},
      {"_yrot_Vel_", YROT_VEL}, {"_zrot_Vel_", ZROT_VEL}, {"_x_For_", X_FOR}, {"_y_For_", Y_FOR},
      {"_z_For_", Z_FOR}, {"_xrot_Mom_", XROT_MOM}, {"_yrot_Mom_", YROT_MOM}, {"_zrot_Mom_", ZROT_MOM},
      {"_xyzrot_Vel_", XYZROT_VEL}, {"_xyzrot_Mom_", XYZROT_MOM}};
  S.controls.clear();
  S.servo = false;
  std::string tok;
  while (is >> tok) {
    if (tok[0] == '/' || tok[0] == '#' || tok[0] == '!') { std::string rest; std::getline(is, rest); continue; }
    if (tok == "Control") {
      std::string ts; Control c{}; is >> ts >> c.i;
      auto it = types.find(ts);
      c.type = it == types.end() ? 0 : it->second;
      if (c.type >= 100) read_v3(is, c.vec); else is >> c.value;
      S.controls.push_back(c);
    } else if (tok == "Servo") {
      std::string name; is >> name;
      if (name.substr(0, 6) == "tritri") {
        is >> S.sXmin >> S.sXmax >> S.sYmin >> S.sYmax >> S.sZmin >> S.sZmax;
        size_t ic = S.controls.size();
        Control c{}; c.value = 0.0;
        c.i = S.sXmin; c.type = X_VEL; S.controls.push_back(c);
        c.i = S.sXmax; c.type = X_FOR; S.controls.push_back(c);
        c.i = S.sYmin; c.type = Y_VEL; S.controls.push_back(c);
        c.i = S.sYmax; c.type = Y_FOR; S.controls.push_back(c);
        c.i = S.sZmin; c.type = Z_VEL; S.controls.push_back(c);
        c.i = S.sZmax; c.type = Z_FOR; S.controls.push_back(c);
        if (name == "tritriIsostaticCompression") {
          is >> S.servo_p;
          S.servo = true;
          S.servo_icontr = ic;
        } else {
          g_err = "servo " + name + " is not supported";
          return false;
        }
      } else {
        g_err = "servo " + name + " is not supported";
        return false;
      }
    }
  }
  return true;
}

static void read_law(Sim& S, std::istream& is, size_t id) {  // Rockable.cpp:619-624
  int g1, g2; double v;
  is >> g1 >> g2 >> v;
  S.table.set(id, g1, g2, v);
}

static void prepro_stick_vertices(Sim& S, double eps);  // below
static void prepro_variable_params(Sim& S, const std::string& par, const std::string& io, double lambda, double m,
                                   int timeSeeded);

// Rockable.cpp:643-1069 and 1085-1145
static bool parse_conf(Sim& S, std::istream& conf) {
  std::string tok;
  while (conf >> tok) {
    if (tok[0] == '/' || tok[0] == '#' || tok[0] == '!') { std::string rest; std::getline(conf, rest); continue; }
    if (tok == "t") conf >> S.t;
    else if (tok == "tmax") conf >> S.tmax;
    else if (tok == "dt") { double v; conf >> v; S.set_dt(v); }
    else if (tok == "interVerlet") conf >> S.interVerlet;
    else if (tok == "interConf") conf >> S.interConf;
    else if (tok == "DVerlet") conf >> S.DVerlet;
    else if (tok == "dVerlet") conf >> S.dVerlet;
    else if (tok == "parallel_mode") conf >> S.parallel_mode;
    else if (tok == "density") { int g; double d; conf >> g >> d; S.density[g] = d; }
    else if (tok == "gravity") read_v3(conf, S.gravity);
    else if (tok == "ParamsInInterfaces") conf >> S.paramsInInterfaces;
    else if (tok == "dynamicUpdateNL") conf >> S.dynamicUpdateNL;
    else if (tok == "dispUpdateNL") conf >> S.dispUpdateNL;
    else if (tok == "angleUpdateNL") { conf >> S.angleUpdateNL; S.angleUpdateNL *= kPi / 180.0; }
    else if (tok == "numericalDampingCoeff") conf >> S.numDamp;
    else if (tok == "VelocityBarrier" || tok == "velocityBarrier") conf >> S.velBarrier;
    else if (tok == "AngularVelocityBarrier" || tok == "angularVelocityBarrier") conf >> S.angVelBarrier;
    else if (tok == "VelocityBarrierExponent") conf >> S.velBarrierExp;
    else if (tok == "AngularVelocityBarrierExponent") conf >> S.angVelBarrierExp;
    else if (tok == "forceLaw") {  // Rockable.cpp:763-781: unknown names fall back to Default
      std::string name; conf >> name;
      if (name == "Default") { S.law = 0; S.options["forceLaw"] = name; }
      else if (name == "Avalanche") { S.law = 1; S.options["forceLaw"] = name; }
      else if (name == "StickedLinks") { S.law = 2; S.options["forceLaw"] = name; }
      else { S.law = 0; S.options["forceLaw"] = "Default"; }
    } else if (tok == "AddOrRemoveInteractions") {
      std::string n; conf >> n;
      if (n == "bruteForce" || n == "OBBtree") S.options["AddOrRemoveInteractions"] = n;
    } else if (tok == "UpdateNL") {
      std::string n; conf >> n;
      if (n == "bruteForce") { S.nl_linkcells = false; S.options["UpdateNL"] = n; }
      else if (n == "linkCells") { S.nl_linkcells = true; S.options["UpdateNL"] = n; }
    } else if (tok == "Integrator") {
      std::string n; conf >> n;
      if (n == "velocityVerlet") S.options["Integrator"] = n;
      else if (n == "Euler" || n == "Beeman" || n == "RungeKutta4") { g_err = "integrator " + n + " is out of scope"; return false; }
    } else if (tok == "cellMinSizes") read_v3(conf, S.cellMinSizes);
    else if (tok == "boxForLinkCellsOpt") conf >> S.boxForLinkCellsOpt;
    else if (tok == "ContactPartnership") {
      std::string n; conf >> n;
      if (n != "None") { g_err = "ContactPartnership " + n + " is out of scope"; return false; }
    } else if (tok == "knContact") read_law(S, conf, S.idKn);
    else if (tok == "en2Contact") read_law(S, conf, S.idEn2);
    else if (tok == "en2ContactFromViscRate") {
      int g1, g2; double vr; conf >> g1 >> g2 >> vr;
      S.table.set(S.idEn2, g1, g2, exp(-vr * kPi / sqrt(1.0 - vr * vr)));
    } else if (tok == "ktContact") read_law(S, conf, S.idKt);
    else if (tok == "muContact") read_law(S, conf, S.idMu);
    else if (tok == "krContact") read_law(S, conf, S.idKr);
    else if (tok == "murContact") read_law(S, conf, S.idMur);
    else if (tok == "viscTContact") read_law(S, conf, S.idViscT);
    else if (tok == "knInnerBond") read_law(S, conf, S.idKnI);
    else if (tok == "ktInnerBond") read_law(S, conf, S.idKtI);
    else if (tok == "krInnerBond") read_law(S, conf, S.idKrI);
    else if (tok == "fn0InnerBond") read_law(S, conf, S.idFn0I);
    else if (tok == "ft0InnerBond") read_law(S, conf, S.idFt0I);
    else if (tok == "mom0InnerBond") read_law(S, conf, S.idMom0I);
    else if (tok == "powInnerBond") read_law(S, conf, S.idPowI);
    else if (tok == "en2InnerBond") read_law(S, conf, S.idEn2I);
    else if (tok == "knOuterBond") read_law(S, conf, S.idKnO);
    else if (tok == "ktOuterBond") read_law(S, conf, S.idKtO);
    else if (tok == "krOuterBond") read_law(S, conf, S.idKrO);
    else if (tok == "fn0OuterBond") read_law(S, conf, S.idFn0O);
    else if (tok == "ft0OuterBond") read_law(S, conf, S.idFt0O);
    else if (tok == "mom0OuterBond") read_law(S, conf, S.idMom0O);
    else if (tok == "powOuterBond") read_law(S, conf, S.idPowO);
    else if (tok == "en2OuterBond") read_law(S, conf, S.idEn2O);
    else if (tok == "gcInnerBond") read_law(S, conf, S.idGcI);
    else if (tok == "gcOuterBond") read_law(S, conf, S.idGcO);
    else if (tok == "iconf") conf >> S.iconf;
    else if (tok == "nDriven") conf >> S.nDriven;
    else if (tok == "shapeFile") {
      std::string name; conf >> name;
      std::string want = S.path + name;
      if (want != S.shape_file) {
        S.shape_file = want;
        if (!load_shapes(S, want)) return false;
      }
    } else if (tok == "precision") conf >> S.precision;
    else if (tok == "Particles") {  // Rockable.cpp:886-931
      size_t nb; conf >> nb;
      S.bodies.clear();
      for (size_t i = 0; i < nb; i++) {
        std::string shp; conf >> shp;
        if (shp[0] == '#') { std::string rest; std::getline(conf, rest); --i; continue; }
        if (shp[0] == '!') { std::string rest; std::getline(conf, rest); --i; --nb; continue; }
        Body P;
        conf >> P.group >> P.cluster >> P.homothety;
        read_v3(conf, P.pos); read_v3(conf, P.vel); read_v3(conf, P.acc);
        read_q(conf, P.Q); read_v3(conf, P.vrot); read_v3(conf, P.arot);
        auto it = S.shape_id.find(shp);
        if (it == S.shape_id.end()) { g_err = "unknown shape " + shp; return false; }
        P.shape_id = it->second;
        P.shape = &S.shapes[it->second];
        double h = P.homothety;
        double dens = S.density.count(P.group) ? S.density[P.group] : 0.0;
        P.mass = (h * h * h * P.shape->volume) * dens;
        P.inertia = (h * h * P.shape->inertia_mass) * P.mass;
        S.bodies.push_back(P);
      }
      S.inter.assign(S.bodies.size(), {});
      S.ifaces.assign(S.bodies.size(), {});
    } else if (tok == "Interactions") {  // Rockable.cpp:932-955
      size_t nb; conf >> nb;
      for (auto& m : S.inter) m.clear();
      S.active.clear();
      Contact I;  // reused across lines like the reference
      for (size_t k = 0; k < nb; ++k) {
        conf >> I.k.i >> I.k.j >> I.k.type >> I.k.isub >> I.k.jsub;
        read_v3(conf, I.n);
        conf >> I.dn;
        read_v3(conf, I.pos); read_v3(conf, I.vel);
        conf >> I.fn;
        read_v3(conf, I.ft); read_v3(conf, I.mom);
        conf >> I.damp;
        if (I.k.i >= S.inter.size()) { g_err = "interaction body index out of range"; return false; }
        S.inter[I.k.i].emplace(I.k, I);  // std::set::insert keeps the first
      }
      S.flat_dirty = true;
    } else if (tok == "Interfaces") {  // Rockable.cpp:956-1002
      size_t nbi; conf >> nbi;
      for (auto& m : S.ifaces) m.clear();
      for (size_t k = 0; k < nbi; ++k) {
        Iface BI;
        size_t nbonds;
        conf >> BI.i >> BI.j >> nbonds >> BI.dn0;
        if (S.paramsInInterfaces == 1)
          conf >> BI.kn >> BI.kt >> BI.kr >> BI.fn0 >> BI.ft0 >> BI.mom0 >> BI.power >> BI.Gc;
        std::vector<Contact*> bonds;
        bool missed = false;
        for (size_t u = 0; u < nbonds; ++u) {
          Key kf{BI.i, BI.j, 0, 0, 0};
          conf >> kf.type >> kf.isub >> kf.jsub;
          auto it = S.inter[BI.i].find(kf);
          if (it != S.inter[BI.i].end()) bonds.push_back(&it->second);
          else missed = true;
        }
        if (!missed) {
          auto res = S.ifaces[BI.i].emplace(BI.j, BI);
          Iface* p = &res.first->second;
          if (res.second) {
            p->bonds = bonds;
            for (Contact* c : bonds) c->stick = p;
          }
        }
      }
    } else if (tok == "stickVerticesInClusters") {
      double eps; conf >> eps;
      prepro_stick_vertices(S, eps);
    } else if (tok == "setVariableStickParams") {
      std::string par, io; double lambda, m; int ts;
      conf >> par >> io >> lambda >> m >> ts;
      prepro_variable_params(S, par, io, lambda, m, ts);
    } else if (tok == "BodyForce") {
      std::string name; conf >> name;
      if (name == "AttractingPoint") {
        S.bf_kind = 1;
        read_v3(conf, S.bf_point);
        conf >> S.bf_acceleration;
        S.bf_raw = {S.bf_point.x, S.bf_point.y, S.bf_point.z, S.bf_acceleration};
      } else if (name == "PreferredDirection") {
        S.bf_kind = 2;
        read_v3(conf, S.bf_axisBody);
        read_v3(conf, S.bf_axis);
        conf >> S.bf_momentMax;
        S.bf_raw = {S.bf_axisBody.x, S.bf_axisBody.y, S.bf_axisBody.z, S.bf_axis.x, S.bf_axis.y, S.bf_axis.z,
                    S.bf_momentMax};
        normalize(S.bf_axisBody);
        normalize(S.bf_axis);
        S.bf_Kr = 2.0 * S.bf_momentMax / kPi;
      } else if (name == "ViscousFluid") {
        S.bf_kind = 3;
        conf >> S.bf_fluidDensity;
        S.bf_raw = {S.bf_fluidDensity};
      } else {
        g_err = "BodyForce " + name + " is unknown";
        return false;
      }
    } else if (tok == "DataExtractor" || tok == "initSpringJoint" || tok == "Tempo" ||
               tok == "usePeriodicCell" || tok == "useSoftParticles") {
      g_err = "keyword " + tok + " is out of the oracle's scope";
      return false;
    }
    // any other token is skipped like an unknown keyword (kwParser warns)
  }
  return true;
}

// PreproCommand_stickVerticesInClusters.cpp:56-141
static void prepro_stick_vertices(Sim& S, double eps) {
  for (auto& P : S.bodies) P.update_obb();
  for (size_t i = S.nDriven; i < S.bodies.size(); i++) {
    Obb obbi = S.bodies[i].obb;
    obbi.enlarge(0.5 * S.DVerlet);
    for (size_t j = i + 1; j < S.bodies.size(); j++) {
      if (S.bodies[i].cluster != S.bodies[j].cluster) continue;
      Obb obbj = S.bodies[j].obb;
      obbj.enlarge(0.5 * S.DVerlet);
      if (!obb_intersect(obbi, obbj)) continue;
      Body& Pi = S.bodies[i];
      Body& Pj = S.bodies[j];
      for (size_t iv = 0; iv < Pi.shape->vertex.size(); iv++) {
        V3 Vi = Pi.glob_vertex(iv);
        double Ri = Pi.R();
        for (size_t jv = 0; jv < Pj.shape->vertex.size(); jv++) {
          V3 Vj = Pj.glob_vertex(jv);
          double Rj = Pj.R();
          double distSqr = norm2(Vj - Vi);
          double dMaxSqr = eps + (Ri + Rj);
          dMaxSqr *= dMaxSqr;
          if (distSqr < dMaxSqr) {
            double Damp = contact_damping(S, i, j, S.idEn2I, S.idKnI);
            int g1 = Pi.group, g2 = Pj.group;
            Iface BI;
            BI.i = i; BI.j = j; BI.isInner = 1;
            BI.kn = S.table.get(S.idKnI, g1, g2); BI.kt = S.table.get(S.idKtI, g1, g2);
            BI.kr = S.table.get(S.idKrI, g1, g2); BI.fn0 = S.table.get(S.idFn0I, g1, g2);
            BI.ft0 = S.table.get(S.idFt0I, g1, g2); BI.mom0 = S.table.get(S.idMom0I, g1, g2);
            BI.power = S.table.get(S.idPowI, g1, g2);
            auto res = S.ifaces[i].emplace(j, BI);
            Iface* p = &res.first->second;
            Contact I;
            I.k = Key{i, j, VV, iv, jv};
            I.damp = Damp;
            I.stick = p;
            update_vv(I, Pi, Pj);
            auto ins = S.inter[i].emplace(I.k, I);
            p->bonds.push_back(&ins.first->second);
            S.flat_dirty = true;
          }
        }
      }
    }
  }
}

// PreproCommand_setVariableStickParams.cpp:57-94 (libstdc++ engine and
// Weibull distribution, as the reference uses them)
static void prepro_variable_params(Sim& S, const std::string& par, const std::string& io, double lambda, double m,
                                   int timeSeeded) {
  std::default_random_engine gen;
  (void)timeSeeded;  // time seeding is not reproducible: always the default seed here
  std::weibull_distribution<> dist(m, lambda);
  int inner = (io == "inner") ? 1 : 0;
  for (size_t i = 0; i < S.ifaces.size(); i++)
    for (auto& kv : S.ifaces[i]) {
      Iface& BI = kv.second;
      int ic = S.bodies[BI.i].cluster, jc = S.bodies[BI.j].cluster;
      if (inner == 0 && ic == jc) continue;
      if (inner == 1 && ic != jc) continue;
      double v = dist(gen);
      if (par == "kn") BI.kn = v;
      else if (par == "kt") BI.kt = v;
      else if (par == "kr") BI.kr = v;
      else if (par == "fn0") BI.fn0 = v;
      else if (par == "ft0") BI.ft0 = v;
      else if (par == "mom0") BI.mom0 = v;
      else BI.kn = v;
    }
  S.paramsInInterfaces = 1;
}

static bool load_conf(Sim& S, const std::string& name) {  // Rockable.cpp:1085-1145
  std::ifstream conf(name);
  if (!conf) { g_err = "cannot read " + name; return false; }
  std::string prog;
  conf >> prog;
  if (prog == "redirection") {
    std::string sub, newName;
    conf >> sub >> newName;
    S.path = dirname_of(name) + sub;
    return load_conf(S, S.path + newName);
  }
  if (S.path.empty()) S.path = dirname_of(name);
  std::string date;
  conf >> date;
  if (!parse_conf(S, conf)) return false;
  accelerations(S);  // the load-time "fake step" (Rockable.cpp:1137-1138)
  return true;
}

// ---------------------------------------------------------------- output ----
static int g_prec = 16;  // CommBox().precision: the conf's "precision" keyword
static void put_d(std::string& o, double v) {
  char b[64];
  snprintf(b, sizeof b, "%.*e", g_prec, v);
  o += b;
}
static void put_v3(std::string& o, const V3& v) {
  put_d(o, v.x); o += ' '; put_d(o, v.y); o += ' '; put_d(o, v.z);
}
static void put_g(std::ostringstream& os, double v) { os << v; }

// Rockable.cpp:440-610
static bool save_conf(Sim& S, const std::string& fname) {
  std::ostringstream head;
  head << "Rockable 21-08-2022\n";
  for (auto& kv : S.options) head << kv.first << " " << kv.second << '\n';
  head << "t "; put_g(head, S.t); head << "\ntmax "; put_g(head, S.tmax);
  head << "\ndt "; put_g(head, S.dt); head << "\ninterVerlet "; put_g(head, S.interVerlet);
  head << "\ninterConf "; put_g(head, S.interConf); head << "\nDVerlet "; put_g(head, S.DVerlet);
  head << "\ndVerlet "; put_g(head, S.dVerlet);
  head << "\nparallel_mode " << S.parallel_mode << '\n';
  for (auto& kv : S.density)
    if (kv.second > 0.0) { head << "density " << kv.first << " "; put_g(head, kv.second); head << '\n'; }
  head << "gravity " << S.gravity.x << " " << S.gravity.y << " " << S.gravity.z << '\n';
  if (S.bf_kind == 1)  // Rockable.cpp:470-473 with BodyForce_*.cpp write()
    head << "BodyForce AttractingPoint " << S.bf_point.x << " " << S.bf_point.y << " " << S.bf_point.z << ' '
         << S.bf_acceleration << '\n';
  else if (S.bf_kind == 2)
    head << "BodyForce PreferredDirection " << S.bf_axisBody.x << " " << S.bf_axisBody.y << " " << S.bf_axisBody.z
         << ' ' << S.bf_axis.x << " " << S.bf_axis.y << " " << S.bf_axis.z << ' ' << S.bf_momentMax << '\n';
  else if (S.bf_kind == 3)
    head << "BodyForce ViscousFluid " << S.bf_fluidDensity << '\n';
  head << "ParamsInInterfaces " << S.paramsInInterfaces << '\n';
  head << "dynamicUpdateNL " << S.dynamicUpdateNL << '\n';
  if (S.dynamicUpdateNL != 0) {
    head << "dispUpdateNL " << S.dispUpdateNL << '\n';
    head << "angleUpdateNL " << S.angleUpdateNL * 180.0 / kPi << '\n';
  }
  head << "numericalDampingCoeff " << S.numDamp << '\n';
  head << "VelocityBarrier " << S.velBarrier << '\n';
  head << "AngularVelocityBarrier " << S.angVelBarrier << '\n';
  head << "VelocityBarrierExponent " << S.velBarrierExp << '\n';
  head << "AngularVelocityBarrierExponent " << S.angVelBarrierExp << '\n';
  const char* names[] = {"knContact", "en2Contact", "ktContact", "muContact", "krContact", "murContact",
                         "viscTContact", "knInnerBond", "ktInnerBond", "krInnerBond", "fn0InnerBond",
                         "ft0InnerBond", "mom0InnerBond", "powInnerBond", "en2InnerBond", "knOuterBond",
                         "ktOuterBond", "krOuterBond", "fn0OuterBond", "ft0OuterBond", "mom0OuterBond",
                         "powOuterBond", "en2OuterBond", "gcInnerBond", "gcOuterBond"};
  for (const char* nm : names) {
    size_t id = S.table.id[nm];
    for (size_t g1 = 0; g1 < S.table.ngroup; ++g1)
      for (size_t g2 = g1; g2 < S.table.ngroup; ++g2)
        if (S.table.defined(id, (int)g1, (int)g2)) head << nm << ' ' << g1 << ' ' << g2 << ' ' << S.table.get(id, (int)g1, (int)g2) << '\n';
  }
  head << "ContactPartnership None\n";
  head << "cellMinSizes " << S.cellMinSizes.x << " " << S.cellMinSizes.y << " " << S.cellMinSizes.z << '\n';
  head << "boxForLinkCellsOpt " << S.boxForLinkCellsOpt << '\n';
  head << "iconf " << S.iconf << '\n';
  head << "nDriven " << S.nDriven << '\n';
  std::string shp = S.shape_file;
  size_t sl = shp.find_last_of('/');
  if (sl != std::string::npos) shp = shp.substr(sl + 1);
  head << "shapeFile " << shp << '\n';
  head << "precision " << S.precision << '\n';
  std::string o = head.str();
  g_prec = S.precision;
  o += "Particles " + std::to_string(S.bodies.size()) + "\n";
  o += "#name group cluster homothety pos.x pos.y pos.z vel.x vel.y vel.z acc.x acc.y acc.z Q.w Q.x Q.y Q.z vrot.x vrot.y vrot.z arot.x arot.y arot.z\n";
  for (auto& P : S.bodies) {
    o += P.shape->name + ' ' + std::to_string(P.group) + ' ' + std::to_string(P.cluster) + ' ';
    put_d(o, P.homothety); o += ' ';
    put_v3(o, P.pos); o += ' '; put_v3(o, P.vel); o += ' '; put_v3(o, P.acc); o += ' ';
    put_d(o, P.Q.s); o += ' '; put_v3(o, P.Q.v); o += ' ';
    put_v3(o, P.vrot); o += ' '; put_v3(o, P.arot); o += '\n';
  }
  std::vector<Contact*> act = S.active;
  std::sort(act.begin(), act.end(), [](const Contact* a, const Contact* b) { return a->k < b->k; });
  o += "Interactions " + std::to_string(act.size()) + "\n";
  const int prev_round = fegetround();
  for (Contact* I : act) {
    o += std::to_string(I->k.i) + ' ' + std::to_string(I->k.j) + ' ' + std::to_string(I->k.type) + ' ' +
         std::to_string(I->k.isub) + ' ' + std::to_string(I->k.jsub) + ' ';
    fesetround(FE_TOWARDZERO);
    put_v3(o, I->n);
    fesetround(prev_round);
    o += ' '; put_d(o, I->dn); o += ' '; put_v3(o, I->pos); o += ' '; put_v3(o, I->vel); o += ' ';
    put_d(o, I->fn); o += ' '; put_v3(o, I->ft); o += ' '; put_v3(o, I->mom); o += ' ';
    put_d(o, I->damp); o += '\n';
  }
  size_t nbi = 0;
  for (auto& m : S.ifaces) nbi += m.size();
  o += "Interfaces " + std::to_string(nbi) + "\n";
  char b[64];
  for (auto& m : S.ifaces)
    for (auto& kv : m) {
      const Iface& BI = kv.second;
      o += std::to_string(BI.i) + ' ' + std::to_string(BI.j) + "  " + std::to_string(BI.bonds.size()) + ' ';
      snprintf(b, sizeof b, "%.6f", BI.dn0); o += b;
      if (S.paramsInInterfaces == 1) {
        const double ps[8] = {BI.kn, BI.kt, BI.kr, BI.fn0, BI.ft0, BI.mom0, BI.power, BI.Gc};
        for (double p : ps) { snprintf(b, sizeof b, " %.6f", p); o += b; }
        o += ' ';
      }
      for (Contact* c : BI.bonds)
        o += "  " + std::to_string(c->k.type) + ' ' + std::to_string(c->k.isub) + ' ' + std::to_string(c->k.jsub);
      o += '\n';
    }
  std::ofstream f(fname);
  if (!f) { g_err = "cannot write " + fname; return false; }
  f << o;
  return true;
}

static void run_steps(Sim& S, long nsteps, const std::string* outdir, long* nl_updates) {
  // Rockable.cpp:2584-2739 (loop body, without the console frames)
  for (long s = 0; s < nsteps; ++s) {
    S.t += S.dt;
    S.interConfC += S.dt;
    S.interVerletC += S.dt;
    verlet_step(S);
    if (outdir && S.interConfC >= S.interConf - S.dt_2) {
      S.iconf++;
      save_conf(S, *outdir + "/conf" + std::to_string(S.iconf));
      servo(S);
      S.interConfC = 0.0;
    }
    if (S.needUpdate || S.interVerletC >= S.interVerlet - S.dt_2) {
      update_nl(S);
      if (nl_updates) (*nl_updates)++;
      if (!S.needUpdate) S.interVerletC = 0.0;
      else S.needUpdate = false;
    }
    if (S.dynamicUpdateNL != 0) dynamic_check(S);
  }
}

static void prepare_integrate(Sim& S) {  // Rockable.cpp:2546-2565
  if (S.dynamicUpdateNL != 0) {
    S.deltaPos.assign(S.bodies.size(), V3());
    S.deltaQ.assign(S.bodies.size(), Quat());
    S.maxDeltaPos = 0.0;
    S.maxDeltaRot = 0.0;
  }
  S.set_dt(S.dt);
}

}  // namespace orc

// ================================================================ C API ====
using namespace orc;
struct orc_sim {
  Sim S;
  bool prepared{false};
};

extern "C" {

void orc_set_variant(const orc_variant* v) { g_var = *v; }
const char* orc_last_error(void) { return g_err.c_str(); }

orc_sim* orc_load(const char* conf_path) {
  orc_sim* s = new orc_sim();
  if (!load_conf(s->S, conf_path)) { delete s; return nullptr; }
  return s;
}
void orc_free(orc_sim* s) { delete s; }
int orc_read_driving(orc_sim* s, const char* path) { return read_driving(s->S, path) ? 0 : -1; }
void orc_update_nl(orc_sim* s) { update_nl(s->S); }

int orc_run(orc_sim* s, int nsteps) {
  if (!s->prepared) { prepare_integrate(s->S); s->prepared = true; }
  long n = 0;
  run_steps(s->S, nsteps, nullptr, &n);
  return (int)n;
}

long orc_integrate(orc_sim* s, const char* outdir, long max_steps) {
  Sim& S = s->S;
  update_nl(S);  // Rockable.cpp:1265
  prepare_integrate(S);
  s->prepared = true;
  std::string od(outdir);
  save_conf(S, od + "/conf" + std::to_string(S.iconf));
  long steps = 0;
  while (S.t <= S.tmax) {
    if (max_steps > 0 && steps >= max_steps) break;
    run_steps(S, 1, &od, nullptr);
    steps++;
  }
  return steps;
}

int orc_save_conf(orc_sim* s, const char* path) { return save_conf(s->S, path) ? 0 : -1; }
int orc_nbodies(const orc_sim* s) { return (int)s->S.bodies.size(); }
int orc_ndriven(const orc_sim* s) { return (int)s->S.nDriven; }

void orc_get_bodies(const orc_sim* s, double* out) {
  for (const Body& P : s->S.bodies) {
    const V3* vs[] = {&P.pos, &P.vel, &P.acc};
    for (auto v : vs) { *out++ = v->x; *out++ = v->y; *out++ = v->z; }
    *out++ = P.Q.s; *out++ = P.Q.v.x; *out++ = P.Q.v.y; *out++ = P.Q.v.z;
    const V3* ws[] = {&P.vrot, &P.arot, &P.force, &P.moment};
    for (auto v : ws) { *out++ = v->x; *out++ = v->y; *out++ = v->z; }
    *out++ = P.homothety; *out++ = P.mass; *out++ = P.group; *out++ = P.cluster;
  }
}
void orc_set_bodies(orc_sim* s, const double* in) {
  for (Body& P : s->S.bodies) {
    V3* vs[] = {&P.pos, &P.vel, &P.acc};
    for (auto v : vs) { v->x = *in++; v->y = *in++; v->z = *in++; }
    P.Q.s = *in++; P.Q.v.x = *in++; P.Q.v.y = *in++; P.Q.v.z = *in++;
    V3* ws[] = {&P.vrot, &P.arot};
    for (auto v : ws) { v->x = *in++; v->y = *in++; v->z = *in++; }
  }
}

long orc_nentries(const orc_sim* s) {
  long n = 0;
  for (auto& m : s->S.inter) n += (long)m.size();
  return n;
}
void orc_get_entries(const orc_sim* s, int64_t* keys, double* st) {
  for (auto& m : s->S.inter)
    for (auto& kv : m) {
      const Contact& c = kv.second;
      *keys++ = (int64_t)c.k.i; *keys++ = (int64_t)c.k.j; *keys++ = c.k.type;
      *keys++ = (int64_t)c.k.isub; *keys++ = (int64_t)c.k.jsub;
      *st++ = c.n.x; *st++ = c.n.y; *st++ = c.n.z; *st++ = c.dn; *st++ = c.prev_dn;
      *st++ = c.pos.x; *st++ = c.pos.y; *st++ = c.pos.z;
      *st++ = c.vel.x; *st++ = c.vel.y; *st++ = c.vel.z;
      *st++ = c.fn; *st++ = c.ft.x; *st++ = c.ft.y; *st++ = c.ft.z;
      *st++ = c.mom.x; *st++ = c.mom.y; *st++ = c.mom.z; *st++ = c.damp;
      double bond = -1.0;
      if (c.stick) {
        long idx = 0;
        for (auto& mm : s->S.ifaces) {
          for (auto& kk : mm) { if (&kk.second == c.stick) bond = (double)idx; idx++; }
        }
      }
      *st++ = bond;
      *st++ = (c.dn < 0.0 || c.stick != nullptr) ? 1.0 : 0.0;
    }
}
long orc_nactive(const orc_sim* s) { return (long)s->S.active.size(); }
long orc_ninterfaces(const orc_sim* s) {
  long n = 0;
  for (auto& m : s->S.ifaces) n += (long)m.size();
  return n;
}
void orc_get_interfaces(const orc_sim* s, double* out) {
  for (auto& m : s->S.ifaces)
    for (auto& kv : m) {
      const Iface& B = kv.second;
      *out++ = (double)B.i; *out++ = (double)B.j; *out++ = (double)B.bonds.size(); *out++ = B.dn0;
      *out++ = B.kn; *out++ = B.kt; *out++ = B.kr; *out++ = B.fn0; *out++ = B.ft0; *out++ = B.mom0;
      *out++ = B.power; *out++ = B.isInner;
    }
}
void orc_get_scalars(const orc_sim* s, double* o) {
  const Sim& S = s->S;
  o[0] = S.t; o[1] = S.dt; o[2] = S.tmax; o[3] = S.interVerlet; o[4] = S.interConf; o[5] = S.DVerlet;
  o[6] = S.dVerlet; o[7] = S.iconf; o[8] = (double)S.nDriven; o[9] = S.numDamp; o[10] = S.totalBrokenArea;
  o[11] = (double)S.nbroken; o[12] = S.gravity.x; o[13] = S.gravity.y; o[14] = S.gravity.z;
}
int orc_get_body_force(const orc_sim* s, double* params, double* body_volume) {
  const Sim& S = s->S;
  for (size_t k = 0; k < S.bf_raw.size() && k < 8; ++k) params[k] = S.bf_raw[k];
  if (body_volume)
    for (size_t b = 0; b < S.bodies.size(); ++b) {
      const Body& P = S.bodies[b];
      double hh = P.homothety;
      body_volume[b] = P.shape->volume * hh * hh * hh;
    }
  return S.bf_kind;
}

void orc_get_stats(const orc_sim* s, double* o) {  // Rockable.cpp:3958-3970
  const Sim& S = s->S;
  double Et = 0.0, Er = 0.0;
  for (size_t i = 0; i < S.bodies.size(); i++) {
    const Body& P = S.bodies[i];
    Et += P.mass * (P.vel * P.vel);
    V3 w = qrot(qconj(P.Q), P.vrot);
    Er += P.inertia[0] * w.x * w.x + P.inertia[1] * w.y * w.y + P.inertia[2] * w.z * w.z;
  }
  o[0] = 0.5 * Et;
  o[1] = 0.5 * Er;
  o[2] = (double)S.active.size();
  size_t nfree = S.bodies.size() > S.nDriven ? S.bodies.size() - S.nDriven : 0;
  o[3] = nfree ? 2.0 * (double)S.active.size() / (double)nfree : 0.0;
  o[4] = (double)S.nbroken;
}
int orc_law_id(const orc_sim* s) { return s->S.law; }
const char* orc_option(const orc_sim* s, const char* key) {
  auto it = s->S.options.find(key);
  return it == s->S.options.end() ? "" : it->second.c_str();
}
int orc_nshapes(const orc_sim* s) { return (int)s->S.shapes.size(); }

void orc_get_shape_sizes(const orc_sim* s, int64_t* z) {
  z[0] = (int64_t)s->S.shapes.size();
  z[1] = z[2] = z[3] = z[4] = 0;
  for (const Shape& sh : s->S.shapes) {
    z[1] += (int64_t)sh.vertex.size();
    z[2] += (int64_t)sh.edge.size();
    z[3] += (int64_t)sh.face.size();
    for (auto& f : sh.face) z[4] += (int64_t)f.size();
  }
}
void orc_get_shapes(const orc_sim* s, int32_t* vo, double* vx, int32_t* eo, int32_t* ed, int32_t* fo, int32_t* fvo,
                    int32_t* fv, double* rad, double* obb) {
  int32_t nv = 0, ne = 0, nf = 0, nfv = 0;
  size_t k = 0;
  for (const Shape& sh : s->S.shapes) {
    vo[k] = nv; eo[k] = ne; fo[k] = nf;
    for (auto& v : sh.vertex) { vx[3 * nv] = v.x; vx[3 * nv + 1] = v.y; vx[3 * nv + 2] = v.z; nv++; }
    for (auto& e : sh.edge) { ed[2 * ne] = (int32_t)e.first; ed[2 * ne + 1] = (int32_t)e.second; ne++; }
    for (auto& f : sh.face) {
      fvo[nf++] = nfv;
      for (size_t id : f) fv[nfv++] = (int32_t)id;
    }
    rad[k] = sh.radius;
    const Obb& o = sh.obb;
    const V3* parts[5] = {&o.center, &o.e[0], &o.e[1], &o.e[2], &o.extent};
    for (int q = 0; q < 5; q++) { obb[15 * k + 3 * q] = parts[q]->x; obb[15 * k + 3 * q + 1] = parts[q]->y; obb[15 * k + 3 * q + 2] = parts[q]->z; }
    k++;
  }
  vo[k] = nv; eo[k] = ne; fo[k] = nf; fvo[nf] = nfv;
}
void orc_get_body_static(const orc_sim* s, int32_t* shape, int32_t* group, int32_t* cluster, double* hom, double* mass,
                         double* inertia) {
  size_t i = 0;
  for (const Body& P : s->S.bodies) {
    shape[i] = (int32_t)P.shape_id; group[i] = P.group; cluster[i] = P.cluster; hom[i] = P.homothety;
    mass[i] = P.mass; inertia[3 * i] = P.inertia.x; inertia[3 * i + 1] = P.inertia.y; inertia[3 * i + 2] = P.inertia.z;
    i++;
  }
}
int orc_ngroup(const orc_sim* s) {
  int g = (int)s->S.table.ngroup;
  for (auto& B : s->S.bodies) g = std::max(g, B.group + 1);
  return g < 1 ? 1 : g;
}
void orc_get_table(const orc_sim* s, double* t) {
  const Sim& S = s->S;
  const size_t ids[22] = {S.idKn, S.idEn2, S.idKt, S.idMu, S.idKr, S.idMur,
                          S.idKnI, S.idKtI, S.idKrI, S.idEn2I, S.idFn0I, S.idFt0I, S.idMom0I, S.idPowI,
                          S.idKnO, S.idKtO, S.idKrO, S.idEn2O, S.idFn0O, S.idFt0O, S.idMom0O, S.idPowO};
  int G = orc_ngroup(s);
  for (int p = 0; p < 22; p++)
    for (int a = 0; a < G; a++)
      for (int b = 0; b < G; b++) t[((size_t)p * G + a) * G + b] = S.table.get(ids[p], a, b);
}
int orc_ncontrols(const orc_sim* s) { return (int)s->S.controls.size(); }
void orc_get_controls(const orc_sim* s, int32_t* type, int32_t* body, double* value, double* vec, int32_t* servo,
                      double* pressure) {
  const Sim& S = s->S;
  for (size_t k = 0; k < S.controls.size(); k++) {
    type[k] = S.controls[k].type; body[k] = (int32_t)S.controls[k].i; value[k] = S.controls[k].value;
    vec[3 * k] = S.controls[k].vec.x; vec[3 * k + 1] = S.controls[k].vec.y; vec[3 * k + 2] = S.controls[k].vec.z;
  }
  servo[0] = S.servo ? 1 : 0;
  servo[1] = (int32_t)S.servo_icontr;
  servo[2] = (int32_t)S.sXmin; servo[3] = (int32_t)S.sXmax; servo[4] = (int32_t)S.sYmin;
  servo[5] = (int32_t)S.sYmax; servo[6] = (int32_t)S.sZmin; servo[7] = (int32_t)S.sZmax;
  *pressure = S.servo_p;
}
int orc_set_param(orc_sim* s, const char* name, int g1, int g2, double value) {
  auto it = s->S.table.id.find(name);
  if (it == s->S.table.id.end()) return -1;
  s->S.table.set(it->second, g1, g2, value);
  return 0;
}
void orc_get_flow(const orc_sim* s, double* o) {
  const Sim& S = s->S;
  o[0] = S.interVerletC; o[1] = S.dynamicUpdateNL; o[2] = S.dispUpdateNL; o[3] = S.angleUpdateNL;
  o[4] = S.paramsInInterfaces; o[5] = S.needUpdate ? 1.0 : 0.0;
}

}  // extern "C"
