// rk_pack.cpp -- seeded packer of sphero-polyhedral grains (host tool).
//
// Builds the loose random packings that the benchmark and test scenes start
// from -- a column of grains on a floor, grains filling a box -- on the CPU,
// so that a process without a GPU builds exactly the same initial state as
// one with a GPU.  Rockable itself gets such states from a preparation run of
// its own step loop (gravity deposition, Rockable.cpp:2538-2746); this tool
// reaches one by geometry alone.
//
// Method: sequential deposition with frictionless sliding, exact grain
// geometry.  One at a time, in their order, grains keep the orientation
// they are given, start at a uniform random point of the footprint just
// above the grains already there, and move down until they rest: straight
// down while nothing is touched, then along the steepest direction their
// contacts allow -- gravity's direction projected onto the cone of
// directions that do not move into a touching support (a tangent plane for
// one contact, the groove of two) -- until three or more supports block
// every descent.  They translate only.  Every move is safe by conservative
// advancement: the distance between the cores (convex hulls of the shape
// vertices) of two grains is computed exactly by GJK (Gilbert, Johnson &
// Keerthi, IEEE J. Robotics Autom. 4(2), 1988), and because the distance
// from a point to a convex set is a convex function of the point, its
// decrease along a straight move is bounded by its present rate: a grain at
// gap g from a support whose normal n closes at rate -u.n along the move u
// can travel g / (-u.n) before they can touch.  No grain ever overlaps
// another, the floor or a side wall.  The deposition is sequential and every
// random draw comes from one seeded generator, so the same input gives the
// same packing on every run and host (the shapes and orientations themselves
// come from numpy and scipy, whose last bits can differ between hosts).
//
// Usage: rk_pack IN OUT.  IN is a little-endian binary file written by
// rockable_gb300/scenes.py (layout in read_input); OUT receives the grains'
// positions (3 doubles each) followed by 8 doubles of statistics.
// Compiled with -ffp-contract=off and only + - * / sqrt in the arithmetic.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct V {
  double x, y, z;
};
inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V operator*(double s, V a) { return {s * a.x, s * a.y, s * a.z}; }
inline V operator-(V a) { return {-a.x, -a.y, -a.z}; }
inline double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double comp(V a, int d) { return d == 0 ? a.x : (d == 1 ? a.y : a.z); }
inline void add_comp(V& a, int d, double s) {
  if (d == 0) a.x += s;
  else if (d == 1) a.y += s;
  else a.z += s;
}

// splitmix64: a portable, seedable generator (Steele, Lea & Flood, OOPSLA 2014)
struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ------------------------------------------------------------------- GJK --
// Support point index of a vertex set in direction d.
inline int support(const V* v, int n, V d) {
  int best = 0;
  double bd = dot(v[0], d);
  for (int k = 1; k < n; ++k) {
    double s = dot(v[k], d);
    if (s > bd) {
      bd = s;
      best = k;
    }
  }
  return best;
}

// Simplex of Minkowski-difference points w = c + a - b (c: centre offset
// x_A - x_B; a, b: vertex offsets of A and B), with the vertex indices that
// made each point.
struct Simplex {
  V w[4];
  int ia[4], ib[4];
  int n;
  void keep(std::initializer_list<int> idx) {
    V w2[4];
    int a2[4], b2[4];
    int m = 0;
    for (int k : idx) {
      w2[m] = w[k];
      a2[m] = ia[k];
      b2[m] = ib[k];
      ++m;
    }
    for (int k = 0; k < m; ++k) {
      w[k] = w2[k];
      ia[k] = a2[k];
      ib[k] = b2[k];
    }
    n = m;
  }
};

// Closest point to the origin of segment (p, q) among the simplex points
// with indices i, j; reduces the simplex to the supporting subset.
inline V closest_segment(Simplex& S, int i, int j) {
  V a = S.w[i], b = S.w[j];
  V ab = b - a;
  double den = dot(ab, ab);
  double t = den > 0.0 ? -dot(a, ab) / den : 0.0;
  if (t <= 0.0) {
    S.keep({i});
    return a;
  }
  if (t >= 1.0) {
    S.keep({j});
    return b;
  }
  S.keep({i, j});
  return a + t * ab;
}

// Closest point to the origin of triangle (i, j, k) by its Voronoi regions
// (vertex, edge and face regions tested in turn).
V closest_triangle(Simplex& S, int i, int j, int k) {
  V a = S.w[i], b = S.w[j], c = S.w[k];
  V ab = b - a, ac = c - a;
  double d1 = -dot(ab, a), d2 = -dot(ac, a);
  if (d1 <= 0.0 && d2 <= 0.0) {
    S.keep({i});
    return a;
  }
  double d3 = -dot(ab, b), d4 = -dot(ac, b);
  if (d3 >= 0.0 && d4 <= d3) {
    S.keep({j});
    return b;
  }
  double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    double t = d1 / (d1 - d3);
    S.keep({i, j});
    return a + t * ab;
  }
  double d5 = -dot(ab, c), d6 = -dot(ac, c);
  if (d6 >= 0.0 && d5 <= d6) {
    S.keep({k});
    return c;
  }
  double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    double t = d2 / (d2 - d6);
    S.keep({i, k});
    return a + t * ac;
  }
  double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
    double t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    S.keep({j, k});
    return b + t * (c - b);
  }
  double den = va + vb + vc;
  if (!(den > 0.0)) {  // degenerate triangle: best of its edges
    Simplex s1 = S, s2 = S, s3 = S;
    V p1 = closest_segment(s1, i, j), p2 = closest_segment(s2, i, k), p3 = closest_segment(s3, j, k);
    double e1 = dot(p1, p1), e2 = dot(p2, p2), e3 = dot(p3, p3);
    if (e1 <= e2 && e1 <= e3) {
      S = s1;
      return p1;
    }
    if (e2 <= e3) {
      S = s2;
      return p2;
    }
    S = s3;
    return p3;
  }
  double v = vb / den, w = vc / den;
  S.keep({i, j, k});
  return a + v * ab + w * ac;
}

// Closest point of the current simplex to the origin; false when the origin
// lies inside the tetrahedron (the cores intersect).
bool closest_simplex(Simplex& S, V& out) {
  if (S.n == 1) {
    out = S.w[0];
    return true;
  }
  if (S.n == 2) {
    out = closest_segment(S, 0, 1);
    return true;
  }
  if (S.n == 3) {
    out = closest_triangle(S, 0, 1, 2);
    return true;
  }
  // tetrahedron: the faces whose plane separates the origin from the
  // opposite vertex
  static const int F[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
  bool any = false;
  double best = 0.0;
  Simplex bestS = S;
  V bestP{0, 0, 0};
  for (int f = 0; f < 4; ++f) {
    V a = S.w[F[f][0]], b = S.w[F[f][1]], c = S.w[F[f][2]], d = S.w[F[f][3]];
    V nrm = cross(b - a, c - a);
    double so = -dot(nrm, a), sd = dot(nrm, d - a);
    if (so * sd < 0.0 || (sd == 0.0 && so != 0.0)) {
      Simplex T = S;
      V p = closest_triangle(T, F[f][0], F[f][1], F[f][2]);
      double e = dot(p, p);
      if (!any || e < best) {
        any = true;
        best = e;
        bestS = T;
        bestP = p;
      }
    }
  }
  if (!any) return false;
  S = bestS;
  out = bestP;
  return true;
}

// Distance between the convex hulls of va (placed at c relative to B) and
// vb; *nrm receives the unit direction from B's closest point to A's.
// Returns a negative value when the hulls intersect.
double gjk(const V* va, int na, const V* vb, int nb, V c, V* nrm) {
  Simplex S;
  S.n = 1;
  S.ia[0] = support(va, na, -c);
  S.ib[0] = support(vb, nb, c);
  S.w[0] = c + va[S.ia[0]] - vb[S.ib[0]];
  V v = S.w[0];
  double scale = dot(c, c) + 1e-30;
  for (int it = 0; it < 64; ++it) {
    double vv = dot(v, v);
    if (vv <= 1e-24 * scale) return -1.0;
    int ia = support(va, na, -v), ib = support(vb, nb, v);
    V w = c + va[ia] - vb[ib];
    bool dup = false;
    for (int k = 0; k < S.n; ++k) dup = dup || (S.ia[k] == ia && S.ib[k] == ib);
    if (dup || vv - dot(v, w) <= 1e-12 * vv) break;
    if (S.n == 3) {
      // a new point in the plane of the current triangle makes a flat
      // tetrahedron whose inside test rounding can decide either way: the
      // triangle's closest point is then final (a face-to-face contact)
      V e1 = S.w[1] - S.w[0], e2 = S.w[2] - S.w[0], e3 = w - S.w[0];
      double vol = dot(e1, cross(e2, e3));
      double ref = std::sqrt(dot(e1, e1) * dot(e2, e2) * dot(e3, e3));
      if (std::fabs(vol) <= 1e-10 * ref) break;
    }
    S.w[S.n] = w;
    S.ia[S.n] = ia;
    S.ib[S.n] = ib;
    S.n++;
    V nv;
    if (!closest_simplex(S, nv)) return -1.0;
    if (dot(nv, nv) >= vv) break;  // no progress (rounding)
    v = nv;
  }
  double d = std::sqrt(dot(v, v));
  *nrm = (1.0 / d) * v;
  return d;
}

// ---------------------------------------------------------------- packer --
struct Body {
  int v0, nv;
  double r, bound, vol;
  double lo[3], hi[3];  // axis-aligned extents of the rounded grain about its centre
};

struct Params {
  double lo[3], hi[3];  // footprint lo/hi x, y (side walls); floor at lo z
  double tol;           // contact tolerance: a grain stops within this gap (m)
  uint64_t seed;
  int max_iters;        // largest number of moves of one grain
  int tries;            // drop sites tried per grain (the lowest rest is kept)
};

// A contact of the grain being placed: the unit normal pushing it away from
// the support (a grain, the floor or a side wall) and the gap.
struct Contact {
  V n;
  double gap;
};

struct Packer {
  Params P;
  std::vector<Body> B;
  std::vector<V> rv;  // rotated vertex offsets of every body
  std::vector<V> pos;
  double bmax = 0.0;
  // the grains at rest, in a 3-D grid of cells one grain diameter wide that
  // grows upwards as the pile does
  std::vector<std::vector<int>> cells;
  int gx = 0, gy = 0, gz = 0;
  double cs = 0.0;

  int clampi(int a, int lo, int hi) const { return a < lo ? lo : (a > hi ? hi : a); }
  int cx(double x) const { return clampi((int)std::floor((x - P.lo[0]) / cs), 0, gx - 1); }
  int cy(double y) const { return clampi((int)std::floor((y - P.lo[1]) / cs), 0, gy - 1); }
  int cz(double z) const { return std::max(0, (int)std::floor((z - P.lo[2]) / cs)); }
  void insert(int i) {
    int z = cz(pos[i].z);
    if (z >= gz) {
      gz = z + 8;
      cells.resize((size_t)gx * gy * gz);
    }
    cells[((size_t)z * gy + cy(pos[i].y)) * gx + cx(pos[i].x)].push_back(i);
  }

  // The grains at rest whose bounding spheres come within `reach` of grain
  // i's (a cell is one grain diameter, so one ring of cells is enough for a
  // reach below a grain radius).
  void neighbours(int i, const V& p, double reach, std::vector<int>& out) const {
    out.clear();
    int x0 = cx(p.x), y0 = cy(p.y), z0 = cz(p.z);
    for (int z = std::max(z0 - 1, 0); z <= std::min(z0 + 1, gz - 1); ++z)
      for (int y = std::max(y0 - 1, 0); y <= std::min(y0 + 1, gy - 1); ++y)
        for (int x = std::max(x0 - 1, 0); x <= std::min(x0 + 1, gx - 1); ++x)
          for (int j : cells[((size_t)z * gy + y) * gx + x]) {
            V c = p - pos[j];
            double rr = B[i].bound + B[j].bound + reach;
            if (dot(c, c) < rr * rr) out.push_back(j);
          }
  }

  // Gap between the rounded surfaces of grains i and j (negative when they
  // overlap) and the unit normal pushing i away from j.
  double gap(int i, const V& p, int j, V* n) const {
    V c = p - pos[j];
    double d = gjk(&rv[B[i].v0], B[i].nv, &rv[B[j].v0], B[j].nv, c, n);
    if (d < 0.0) {
      double l = std::sqrt(dot(c, c));
      *n = (1.0 / l) * c;
      return -1.0;
    }
    return d - B[i].r - B[j].r;
  }

  // Contacts and near supports of grain i: grains, floor and side walls.
  void supports(int i, const V& p, const std::vector<int>& nb, std::vector<Contact>& out) const {
    out.clear();
    for (int j : nb) {
      V n;
      double g = gap(i, p, j, &n);
      out.push_back({n, g});
    }
    const Body& b = B[i];
    out.push_back({{0, 0, 1}, p.z + b.lo[2] - P.lo[2]});
    out.push_back({{1, 0, 0}, p.x + b.lo[0] - P.lo[0]});
    out.push_back({{-1, 0, 0}, P.hi[0] - p.x - b.hi[0]});
    out.push_back({{0, 1, 0}, p.y + b.lo[1] - P.lo[1]});
    out.push_back({{0, -1, 0}, P.hi[1] - p.y - b.hi[1]});
  }

  // The steepest descent direction of a grain that cannot move into its
  // touching supports: gravity's direction projected onto the cone
  // {u : u . n >= 0 for every touching normal n} (the unprojected direction,
  // its projections on one tangent plane and on the groove of two, the best
  // feasible one); zero when none descends.
  V descent(const std::vector<Contact>& cs_, double touch) const {
    std::vector<V> tn;
    for (const Contact& c : cs_)
      if (c.gap <= touch) tn.push_back(c.n);
    const V g{0, 0, -1};
    auto feasible = [&](V u) {
      for (const V& n : tn)
        if (dot(u, n) < -1e-12) return false;
      return true;
    };
    V best{0, 0, 0};
    double rate = 1e-9;  // slowest descent worth moving along
    auto consider = [&](V u) {
      double l = std::sqrt(dot(u, u));
      if (l < 1e-12) return;
      u = (1.0 / l) * u;
      if (-u.z > rate && feasible(u)) {
        rate = -u.z;
        best = u;
      }
    };
    consider(g);
    for (const V& n : tn) consider(g - dot(g, n) * n);
    for (size_t a = 0; a < tn.size(); ++a)
      for (size_t b = a + 1; b < tn.size(); ++b) {
        V e = cross(tn[a], tn[b]);
        double l = std::sqrt(dot(e, e));
        if (l < 1e-9) continue;
        e = (1.0 / l) * e;
        consider(dot(g, e) * e);
      }
    return best;
  }

  // Place grain i at p: fall and slide from there until no descent is left.
  bool settle(int i, V& p, long* moves) const {
    std::vector<int> nb;
    std::vector<Contact> cs_;
    const double touch = 2.0 * P.tol;
    for (int it = 0; it < P.max_iters; ++it) {
      ++*moves;
      neighbours(i, p, bmax, nb);
      supports(i, p, nb, cs_);
      V u = descent(cs_, touch);
      if (dot(u, u) == 0.0) return true;
      // how far along u before any support can be touched: gap over the
      // closing rate (the gap is a convex function along the move), at most
      // half a grain radius, within which the neighbour list holds
      double step = 0.5 * bmax;
      for (const Contact& c : cs_) {
        double rate = -dot(u, c.n);
        if (rate > 1e-12 && c.gap > touch) step = std::min(step, (c.gap - 0.5 * P.tol) / rate);
        else if (rate > 1e-12) step = 0.0;
      }
      if (step <= 0.25 * P.tol) return true;
      p = p + step * u;
    }
    return false;
  }

  void run(double* stats) {
    const int n = (int)B.size();
    Rng rng{P.seed};
    cs = 2.0 * bmax * 1.001;
    gx = std::max(1, (int)std::ceil((P.hi[0] - P.lo[0]) / cs));
    gy = std::max(1, (int)std::ceil((P.hi[1] - P.lo[1]) / cs));
    gz = 8;
    cells.assign((size_t)gx * gy * gz, {});
    std::vector<double> col_top((size_t)gx * gy, P.lo[2]);
    long moves = 0, at_rest = 0;
    const int K = std::max(1, P.tries);
    std::vector<V> cand(K);
    std::vector<long> cmoves(K);
    std::vector<char> crest(K);
    for (int i = 0; i < n; ++i) {
      // K uniform random points of the footprint where the grain fits, each
      // just above the grains already under it; the grain is dropped from
      // each and kept where it comes to rest lowest (the first such on ties)
      for (int k = 0; k < K; ++k) {
        double x = P.lo[0] - B[i].lo[0] + rng.uniform() * ((P.hi[0] - B[i].hi[0]) - (P.lo[0] - B[i].lo[0]));
        double y = P.lo[1] - B[i].lo[1] + rng.uniform() * ((P.hi[1] - B[i].hi[1]) - (P.lo[1] - B[i].lo[1]));
        int x0 = cx(x), y0 = cy(y);
        double top = P.lo[2];
        for (int yy = std::max(y0 - 1, 0); yy <= std::min(y0 + 1, gy - 1); ++yy)
          for (int xx = std::max(x0 - 1, 0); xx <= std::min(x0 + 1, gx - 1); ++xx)
            top = std::max(top, col_top[yy * gx + xx]);
        cand[k] = {x, y, top - B[i].lo[2] + P.tol};
        cmoves[k] = 0;
      }
#pragma omp parallel for schedule(dynamic, 1) if (K > 1)
      for (int k = 0; k < K; ++k) crest[k] = settle(i, cand[k], &cmoves[k]);
      int best = 0;
      for (int k = 0; k < K; ++k) {
        moves += cmoves[k];
        if (k > 0 && cand[k].z < cand[best].z) best = k;
      }
      pos[i] = cand[best];
      at_rest += crest[best];
      insert(i);
      int c = cy(pos[i].y) * gx + cx(pos[i].x);
      col_top[c] = std::max(col_top[c], pos[i].z + B[i].hi[2]);
    }
    // statistics: touching pairs (gap below 1e-6 m), grains on the floor,
    // height, solid fraction below it, largest overlap
    double vol = 0.0, zmax = P.lo[2];
    for (int i = 0; i < n; ++i) {
      vol += B[i].vol;
      zmax = std::max(zmax, pos[i].z + B[i].hi[2]);
    }
    long touching = 0, floor_touch = 0;
    double worst = 0.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : touching, floor_touch) reduction(max : worst)
    for (int i = 0; i < n; ++i) {
      if (pos[i].z + B[i].lo[2] - P.lo[2] < 1e-6) floor_touch++;
      std::vector<int> nb;
      neighbours(i, pos[i], 1e-6, nb);
      for (int j : nb) {
        if (j <= i) continue;
        V nn;
        double g = gap(i, pos[i], j, &nn);
        if (g < 1e-6) touching++;
        worst = std::max(worst, -g);
      }
    }
    stats[0] = (double)touching;
    stats[1] = (double)floor_touch;
    stats[2] = zmax;
    stats[3] = vol / ((P.hi[0] - P.lo[0]) * (P.hi[1] - P.lo[1]) * (zmax - P.lo[2]));
    stats[4] = (double)moves;
    stats[5] = (double)at_rest;
    stats[6] = worst;
    stats[7] = 0.0;
  }
};

bool read_all(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

// Input layout: int64 magic 0x524b5041434b3033 ("RKPACK03"), int64 nshapes,
// int32 nv[nshapes], double radius[nshapes], double vertices[3*sum(nv)],
// int64 nbodies, int32 shape[n], double scale[n], double Q[4n] (w, x, y, z),
// double volume[n], double params[8]: lo xyz, hi xyz, tol, seed;
// int64 max_iters, int64 tries.
int read_input(const char* path, Packer& pk) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  int64_t magic = 0, ns = 0, n = 0;
  bool ok = read_all(f, &magic, 8) && magic == 0x524b5041434b3033LL && read_all(f, &ns, 8) && ns > 0;
  std::vector<int32_t> nv(ok ? ns : 0);
  std::vector<double> rad(ok ? ns : 0);
  ok = ok && read_all(f, nv.data(), 4 * ns) && read_all(f, rad.data(), 8 * ns);
  std::vector<int64_t> vofs(ns + 1, 0);
  for (int64_t s = 0; ok && s < ns; ++s) vofs[s + 1] = vofs[s] + nv[s];
  std::vector<double> verts(ok ? 3 * vofs[ns] : 0);
  ok = ok && read_all(f, verts.data(), 8 * verts.size()) && read_all(f, &n, 8) && n > 0;
  std::vector<int32_t> shape(ok ? n : 0);
  std::vector<double> scale(ok ? n : 0), Q(ok ? 4 * n : 0), vol(ok ? n : 0);
  double prm[8];
  int64_t iters = 0, tries = 0;
  ok = ok && read_all(f, shape.data(), 4 * n) && read_all(f, scale.data(), 8 * n) && read_all(f, Q.data(), 32 * n) &&
       read_all(f, vol.data(), 8 * n) && read_all(f, prm, sizeof prm) && read_all(f, &iters, 8) &&
       read_all(f, &tries, 8);
  fclose(f);
  if (!ok) return -2;
  Params& P = pk.P;
  for (int d = 0; d < 3; ++d) {
    P.lo[d] = prm[d];
    P.hi[d] = prm[3 + d];
  }
  P.tol = prm[6];
  P.seed = (uint64_t)prm[7];
  P.max_iters = (int)iters;
  P.tries = (int)tries;
  pk.B.resize(n);
  pk.pos.assign(n, V{0, 0, 0});
  int64_t tot = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (shape[i] < 0 || shape[i] >= ns) return -3;
    tot += nv[shape[i]];
  }
  pk.rv.resize(tot);
  int64_t at = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double* q = &Q[4 * i];
    double w = q[0], x = q[1], y = q[2], z = q[3];
    double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                   2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                   2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
    Body& b = pk.B[i];
    int s = shape[i];
    double h = scale[i];
    b.v0 = (int)at;
    b.nv = nv[s];
    b.r = rad[s] * h;
    b.vol = vol[i];
    double bound = 0.0;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = 1e300;
      b.hi[d] = -1e300;
    }
    for (int k = 0; k < nv[s]; ++k) {
      const double* v = &verts[3 * (vofs[s] + k)];
      V u{h * (R[0] * v[0] + R[1] * v[1] + R[2] * v[2]), h * (R[3] * v[0] + R[4] * v[1] + R[5] * v[2]),
          h * (R[6] * v[0] + R[7] * v[1] + R[8] * v[2])};
      pk.rv[at++] = u;
      bound = std::max(bound, std::sqrt(dot(u, u)));
      for (int d = 0; d < 3; ++d) {
        b.lo[d] = std::min(b.lo[d], comp(u, d) - b.r);
        b.hi[d] = std::max(b.hi[d], comp(u, d) + b.r);
      }
    }
    b.bound = bound + b.r;
    pk.bmax = std::max(pk.bmax, b.bound);
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: rk_pack IN OUT\n");
    return 2;
  }
  Packer pk;
  int rc = read_input(argv[1], pk);
  if (rc != 0) {
    fprintf(stderr, "rk_pack: cannot read %s (%d)\n", argv[1], rc);
    return 1;
  }
  double stats[8] = {0};
  pk.run(stats);
  FILE* f = fopen(argv[2], "wb");
  if (!f) return 1;
  bool ok = fwrite(pk.pos.data(), sizeof(V), pk.pos.size(), f) == pk.pos.size() &&
            fwrite(stats, sizeof stats, 1, f) == 1;
  fclose(f);
  return ok ? 0 : 1;
}
