// rk_mixed.cu -- narrow phase and force laws of the mixed-precision form.
//
// Same inputs, outputs and semantics as k_narrow_force (rk_step.cu: update of
// Interaction.cpp:143-326, ForceLaw_*.cpp laws, contributions of
// Rockable.cpp:2752-2789), with the arithmetic split by what it needs:
//   FP64  vertex positions (placed with the step's FP64 rotation matrix of each
//         body, rotm: only the vertices of the entries on the FP64 path), the
//         separation vector of the two sub-elements and
//         its length (hence dn), the face normal of a vertex-face contact
//         (FP32 reciprocal-sqrt seed refined by two FP64 Newton steps), the
//         history dn and the Avalanche normal-force increment;
//   FP32  everything measured relative to a body centre or a face vertex:
//         edge / segment parameters, the point-in-polygon test, the contact
//         point, the relative velocity, the tangential force and rolling
//         moment, and the force / moment contributions; and a first test
//         that proves most entries of a dense list apart (apart_f32), which
//         then skip the FP64 path altogether: pass 1 (k_narrow_mixed_quick)
//         settles those and lists the others by type, pass 2
//         (k_narrow_mixed_full) runs the FP64 path on the lists.
// An overlap dn is a small difference of lengths of the order of the
// particle size, which FP32 cannot resolve; all the other quantities are well
// conditioned.  Compiled with fused multiply-adds allowed.
#include "../../include/rk_gpu.h"
#include "rk_bits.cuh"
#include "rk_engine.cuh"

namespace rk {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) {
  F3 r;
  r.x = x; r.y = y; r.z = z;
  return r;
}
__device__ __forceinline__ F3 tof(V3 a) { return f3(d2f(a.x), d2f(a.y), d2f(a.z)); }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator-(F3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 crossf(F3 a, F3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

__device__ __forceinline__ V3 ld3m(const double* a, int64_t k) { return v3(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }
__device__ __forceinline__ void st3m(double* a, int64_t k, F3 v) {
  a[3 * k] = f2d(v.x);
  a[3 * k + 1] = f2d(v.y);
  a[3 * k + 2] = f2d(v.z);
}
// FP64 world position of global vertex k of body b: pos + R (h v), R the
// step's rotation matrix of the body (rotm, written by the body-frame
// kernel), h v from the per-vertex table uv64
__device__ __forceinline__ V3 vtx64g(const Scene& s, int b, int64_t k) {
  const double ux = s.uv64[3 * k], uy = s.uv64[3 * k + 1], uz = s.uv64[3 * k + 2];
  const double* R = s.rotm + 9 * (int64_t)b;
  return v3(s.pos[3 * (int64_t)b] + (R[0] * ux + R[1] * uy + R[2] * uz),
            s.pos[3 * (int64_t)b + 1] + (R[3] * ux + R[4] * uy + R[5] * uz),
            s.pos[3 * (int64_t)b + 2] + (R[6] * ux + R[7] * uy + R[8] * uz));
}
// the same for vertex `local` of body b
__device__ __forceinline__ V3 vtx64(const Scene& s, int b, int local) { return vtx64g(s, b, s.gv_ofs[b] + local); }

// |d| in FP64 from an FP32 reciprocal-sqrt seed and two Newton steps
__device__ __forceinline__ double len64(V3 d, double& inv) {
  double s = d.x * d.x + d.y * d.y + d.z * d.z;
  double y = f2d(rsqrtf(d2f(s)));
  y = y * (1.5 - 0.5 * s * y * y);
  y = y * (1.5 - 0.5 * s * y * y);
  inv = y;
  return s * y;
}

__device__ __forceinline__ F3 ldgvr(const float* g, int64_t k) { return f3(g[3 * k], g[3 * k + 1], g[3 * k + 2]); }
__device__ __forceinline__ float amax(F3 a) { return fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z))); }

// What FP32 geometry alone proves about an entry: its sub-elements'
// vertices relative to body j's centre (the FP32 offsets gvr, plus the
// difference of the two centres rounded to FP32, posf), the same projection
// parameters as the FP64 path, and the separation's length.
//   kApart    the overlap estimate dnf errs by a few ulps of the coordinates
//             (relative ones, and the centres' absolute ones: `cmag`), so an
//             estimate above a margin of 2e-6 m plus 2e-6 of the relative
//             coordinates' magnitude plus 4e-7 of the centres' proves dn > 0:
//             the FP64 length, the contact point and everything after are
//             skipped, and dnf is kept as the entry's dn (a separated entry's
//             dn only matters through its sign);
//   kOutside  the vertex-edge projection parameter or the edge-edge closest-
//             point parameters lie outside their segment by more than their
//             rounding error (bounded the same way, over the segments'
//             lengths): the FP64 path would find the same (it takes these
//             parameters in FP32 too) and drop the sub-contact;
//   0         the FP64 path decides (near the thresholds, other polygons than
//             triangles, nearly parallel edges).
constexpr int kApart = 1, kOutside = 2;

// dn stored as -0.0: a lost sub-contact whose history is zero already
__device__ __forceinline__ bool lost_before(double dn) {
  return __double_as_longlong(dn) == (long long)0x8000000000000000ull;
}
__device__ __forceinline__ int apart_f32(const Scene& s, int type, int i, int j, int isub, int jsub, bool pre,
                                         int4 G, F3 dxij, float rsum, float cmag, float* dnf) {
  const float* g = s.gvr;
  auto gi = [&](int local) { return (int64_t)s.gv_ofs[i] + local; };
  auto gj = [&](int local) { return (int64_t)s.gv_ofs[j] + local; };
  F3 d;
  float mag;
  if (type == 0) {
    const F3 a = ldgvr(g, pre ? G.x : gi(isub)) + dxij, b = ldgvr(g, pre ? G.y : gj(jsub));
    d = a - b;
    mag = fmaxf(amax(a), amax(b));
  } else if (type == 1) {
    int64_t k1, k2;
    if (pre) { k1 = G.y; k2 = G.z; }
    else {
      const int eo = s.edge_ofs[s.shape[j]] + jsub;
      k1 = gj(s.edges[2 * eo]);
      k2 = gj(s.edges[2 * eo + 1]);
    }
    const F3 a = ldgvr(g, pre ? G.x : gi(isub)) + dxij, p1 = ldgvr(g, k1), p2 = ldgvr(g, k2);
    const F3 E = p2 - p1, w = a - p1;
    const float E2 = dotf(E, E);
    const float r = dotf(w, E) / E2;
    mag = fmaxf(amax(a), fmaxf(amax(p1), amax(p2)));
    if (r <= 0.f || r >= 1.f) {
      // r's error: that of w and E (a few ulps of the coordinates) over |E|
      const float tol = 1e-5f + 4e-7f * (mag + cmag) * rsqrtf(E2) * (1.f + fabsf(r));
      return (r < -tol || r > 1.f + tol) ? kOutside : 0;
    }
    d = w - r * E;
  } else if (type == 2) {
    if (!(pre && G.w >= 0)) return 0;  // polygons other than triangles: the FP64 path
    const F3 a = ldgvr(g, G.x) + dxij, A = ldgvr(g, G.y), B = ldgvr(g, G.z), C = ldgvr(g, G.w);
    const F3 bA = B - A, cA = C - A, w = a - A;
    F3 nn = crossf(bA, cA);
    nn = rsqrtf(dotf(nn, nn)) * nn;
    float dist = dotf(w, nn);
    if (dist < 0.f) { nn = -nn; dist = -dist; }
    // the crossing-number test (the FP64 path's, in the same FP32 frame)
    const F3 v1 = rsqrtf(dotf(bA, bA)) * bA, v2 = crossf(nn, v1);
    const F3 P = w - dist * nn;
    const float ori1 = dotf(P, v1), ori2 = dotf(P, v2);
    int odd = 0;
    auto edge = [&](F3 pa, F3 pb) {
      float pa1 = dotf(pa, v1), pb1 = dotf(pb, v1), pa2 = dotf(pa, v2), pb2 = dotf(pb, v2);
      if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
        if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
      }
    };
    const F3 z = f3(0, 0, 0);
    edge(z, bA);
    edge(bA, cA);
    edge(cA, z);
    mag = fmaxf(amax(a), fmaxf(amax(A), fmaxf(amax(B), amax(C))));
    if (!odd) {
      // the projection clearly outside the triangle: farther than the
      // rounding of the coordinates beyond one of its edges (in the plane,
      // on the side away from the third vertex)
      const float tol = 1e-9f + 1e-6f * (mag + cmag);
      const F3 Pv = P, cA2 = cA;
      const float o = dotf(crossf(bA, cA2), nn);  // the triangle's winding about nn
      if (!(fabsf(o) > 0.f)) return 0;
      const F3 ed[3] = {bA, cA2 - bA, -cA2};
      const F3 st[3] = {f3(0, 0, 0), bA, cA2};
      for (int q = 0; q < 3; q++) {
        const F3 e = ed[q];
        const float side = dotf(crossf(e, Pv - st[q]), nn) * rsqrtf(dotf(e, e));
        if ((o > 0.f ? -side : side) > tol) return kOutside;
      }
      return 0;
    }
    *dnf = dist - rsum;
    return *dnf > 2e-6f + 2e-6f * mag + 4e-7f * cmag ? kApart : 0;
  } else {
    int64_t a1, a2, b1, b2;
    if (pre) { a1 = G.x; a2 = G.y; b1 = G.z; b2 = G.w; }
    else {
      const int eoi = s.edge_ofs[s.shape[i]] + isub, eoj = s.edge_ofs[s.shape[j]] + jsub;
      a1 = gi(s.edges[2 * eoi]); a2 = gi(s.edges[2 * eoi + 1]);
      b1 = gj(s.edges[2 * eoj]); b2 = gj(s.edges[2 * eoj + 1]);
    }
    const F3 pi1 = ldgvr(g, a1) + dxij, pi2 = ldgvr(g, a2) + dxij, pj1 = ldgvr(g, b1), pj2 = ldgvr(g, b2);
    const F3 Ei = pi2 - pi1, Ej = pj2 - pj1, w = pi1 - pj1;
    const float c = dotf(Ei, Ei), dd = dotf(Ej, Ej), ee = dotf(Ei, Ej);
    float f = (c * dd) - (ee * ee);
    if (fabsf(f) <= 1.0e-12f) return 0;
    f = 1.0f / f;
    const float a = dotf(Ei, w), b = dotf(Ej, w);
    const float ss = (ee * b - a * dd) * f, tt = (c * b - ee * a) * f;
    mag = fmaxf(fmaxf(amax(pi1), amax(pi2)), fmaxf(amax(pj1), amax(pj2)));
    if (ss <= 0.f || ss >= 1.f || tt <= 0.f || tt >= 1.f) {
      // well-conditioned pairs only (the sine of the edges' angle above
      // 0.1): the parameters' error is then a few ulps of the coordinates
      // over the shorter edge, amplified by at most 100 by the solve
      if (!(f * c * dd < 100.f)) return 0;
      const float tol = 1e-5f + 4e-5f * (mag + cmag) * rsqrtf(fminf(c, dd)) * (1.f + fabsf(ss) + fabsf(tt));
      return (ss < -tol || ss > 1.f + tol || tt < -tol || tt > 1.f + tol) ? kOutside : 0;
    }
    d = (w + ss * Ei) - tt * Ej;
  }
  *dnf = sqrtf(dotf(d, d)) - rsum;
  return *dnf > 2e-6f + 2e-6f * mag + 4e-7f * cmag ? kApart : 0;
}

// The full path of entry e (everything the FP32 proof did not settle);
// returns whether the entry is active.
__device__ __forceinline__ bool narrow_mixed_full(const Scene& s, int64_t e) {
  bool active = false;
  {
    const int i = s.ei[e], j = s.ej[e];
    const uint32_t ts = s.etsub[e];
    const int type = tsub_type(ts), isub = tsub_isub(ts), jsub = tsub_jsub(ts);
    const double dn_old = s.dn[e];
    const int bond = s.bond[e];
    // the sub-elements' global vertices: from the per-entry index table when
    // it holds the list (one load), else through the shape tables
    const bool pre = s.egv_ok != 0;
    const int4 G = pre ? s.egv[e] : make_int4(-1, -1, -1, -1);
    const double Ri = s.rad[i], Rj = s.rad[j];
    const V3 xi = ld3m(s.pos, i), xj = ld3m(s.pos, j);
    double dn = 0.0;
    F3 n = f3(0, 0, 0), ci = f3(0, 0, 0);  // normal, contact point relative to x_i
    bool ok = true;
    if (type == 0) {
      V3 a, b;
      if (pre) {
        a = vtx64g(s, i, G.x);
        b = vtx64g(s, j, G.y);
      } else {
        a = vtx64(s, i, isub);
        b = vtx64(s, j, jsub);
      }
      V3 d = a - b;
      double inv;
      double L = len64(d, inv);
      dn = L - (Ri + Rj);
      n = tof(d * inv);
      ci = tof(a - xi) - d2f(Ri + 0.5 * dn) * n;
    } else if (type == 1) {
      V3 a, p1, p2;
      if (pre) {
        a = vtx64g(s, i, G.x);
        p1 = vtx64g(s, j, G.y);
        p2 = vtx64g(s, j, G.z);
      } else {
        const int eo = s.edge_ofs[s.shape[j]] + jsub;
        p1 = vtx64(s, j, s.edges[2 * eo]);
        p2 = vtx64(s, j, s.edges[2 * eo + 1]);
        a = vtx64(s, i, isub);
      }
      V3 E = p2 - p1, w = a - p1;
      F3 Ef = tof(E), wf = tof(w);
      float r = dotf(wf, Ef) / dotf(Ef, Ef);
      if (r <= 0.f || r >= 1.f) {
        ok = false;
      } else {
        V3 d = w - f2d(r) * E;
        double inv;
        double L = len64(d, inv);
        dn = L - (Ri + Rj);
        n = tof(d * inv);
        ci = tof(a - xi) - d2f(Ri + 0.5 * dn) * n;
      }
    } else if (type == 2) {
      // a triangle's three vertices come from the table; other polygons
      // walk the shape's face list
      const bool tri = pre && G.w >= 0;
      const int* fv = nullptr;
      int nbv = 3;
      V3 A, B, C, a;
      if (tri) {
        A = vtx64g(s, j, G.y);
        B = vtx64g(s, j, G.z);
        C = vtx64g(s, j, G.w);
        a = vtx64g(s, i, G.x);
      } else {
        const int fo = s.face_ofs[s.shape[j]] + jsub;
        const int v0 = s.face_vofs[fo];
        nbv = s.face_vofs[fo + 1] - v0;
        fv = s.face_verts + v0;
        A = vtx64(s, j, fv[0]);
        B = vtx64(s, j, fv[1]);
        C = vtx64(s, j, fv[nbv - 1]);
        a = pre ? vtx64g(s, i, G.x) : vtx64(s, i, isub);
      }
      V3 w = a - A;
      V3 nn = cross(B - A, C - A);
      double inv;
      len64(nn, inv);
      nn = nn * inv;
      double dist = dot(w, nn);
      if (dist < 0.0) { nn = -nn; dist = -dist; }
      // crossing-number test in FP32, relative to the face vertex A
      F3 nf = tof(nn);
      const F3 bA = tof(B - A);
      F3 v1 = rsqrtf(dotf(bA, bA)) * bA;
      F3 v2 = crossf(nf, v1);
      F3 P = tof(w - dist * nn);
      float ori1 = dotf(P, v1), ori2 = dotf(P, v2);
      int odd = 0;
      auto edge = [&](F3 pa, F3 pb) {
        float pa1 = dotf(pa, v1), pb1 = dotf(pb, v1), pa2 = dotf(pa, v2), pb2 = dotf(pb, v2);
        if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
          if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
        }
      };
      if (tri) {
        const F3 z = f3(0, 0, 0), cA = tof(C - A);
        edge(z, bA);
        edge(bA, cA);
        edge(cA, z);
      } else {
        for (int iva = 0; iva < nbv; ++iva) {
          int ivb = iva + 1;
          if (ivb == nbv) ivb = 0;
          edge(tof(vtx64(s, j, fv[iva]) - A), tof(vtx64(s, j, fv[ivb]) - A));
        }
      }
      if (odd) {
        dn = dist - (Ri + Rj);
        n = nf;
        ci = tof(a - xi) - d2f(Ri + 0.5 * dn) * n;
      } else {
        ok = false;
      }
    } else {
      V3 pi1, pi2, pj1, pj2;
      if (pre) {
        pi1 = vtx64g(s, i, G.x);
        pi2 = vtx64g(s, i, G.y);
        pj1 = vtx64g(s, j, G.z);
        pj2 = vtx64g(s, j, G.w);
      } else {
        const int eoi = s.edge_ofs[s.shape[i]] + isub, eoj = s.edge_ofs[s.shape[j]] + jsub;
        pi1 = vtx64(s, i, s.edges[2 * eoi]);
        pi2 = vtx64(s, i, s.edges[2 * eoi + 1]);
        pj1 = vtx64(s, j, s.edges[2 * eoj]);
        pj2 = vtx64(s, j, s.edges[2 * eoj + 1]);
      }
      V3 Ei = pi2 - pi1, Ej = pj2 - pj1, w = pi1 - pj1;
      F3 Eif = tof(Ei), Ejf = tof(Ej), wf = tof(w);
      float c = dotf(Eif, Eif), d = dotf(Ejf, Ejf), ee = dotf(Eif, Ejf);
      float f = (c * d) - (ee * ee);
      if (fabsf(f) > 1.0e-12f) {
        f = 1.0f / f;
        float a = dotf(Eif, wf), b = dotf(Ejf, wf);
        float ss = (ee * b - a * d) * f;
        float tt = (c * b - ee * a) * f;
        if (ss <= 0.f || ss >= 1.f || tt <= 0.f || tt >= 1.f) {
          ok = false;
        } else {
          V3 dd = (w + f2d(ss) * Ei) - f2d(tt) * Ej;
          double inv;
          double L = len64(dd, inv);
          dn = L - (Ri + Rj);
          n = tof(dd * inv);
          ci = tof((pi1 - xi) + f2d(ss) * Ei) - d2f(Ri + 0.5 * dn) * n;
        }
      } else {
        ok = false;
      }
    }
    // a separated entry (no bond) keeps only its dn: the relative velocity,
    // the history and the law are skipped unless its geometry is recorded;
    // a lost sub-contact restarts its history from zero (its dn stored as
    // -0.0: "lost, history zeroed", which the next step need not rewrite)
    if (!ok) dn = -0.0;
    active = (dn < 0.0 || bond >= 0);
    double fn = 0.0;
    F3 ft = f3(0, 0, 0), mom = f3(0, 0, 0);
    if (active || (ok && s.record_geom)) {
      const F3 dx = tof(xj - xi);
      const F3 wi = tof(ld3m(s.vrot, i)), wj = tof(ld3m(s.vrot, j));
      F3 cj = ci - dx;
      F3 cvel;
      if (ok) {
        const F3 dv = tof(ld3m(s.vel, j) - ld3m(s.vel, i));
        cvel = (dv - crossf(cj, wj)) + crossf(ci, wi);
        fn = s.fn[e];
        ft = tof(ld3m(s.ft, e));
        mom = tof(ld3m(s.mom, e));
        if (s.record_geom || bond >= 0) {
          st3m(s.gn, e, n);
          st3m(s.gpos, e, tof(xi) + ci);
          st3m(s.gvel, e, cvel);
        }
      } else {  // a bond whose sub-contact is lost: its last recorded geometry
        n = tof(ld3m(s.gn, e));
        ci = tof(ld3m(s.gpos, e) - xi);
        cj = ci - dx;
        cvel = tof(ld3m(s.gvel, e));
      }
      if (active) {
        const double* P = s.table[s.group[i] * s.ngroup + s.group[j]].p;
        const float dt = d2f(s.dt);
        const float damp = d2f(s.damp[e]);
        const F3 dw = wj - wi;
        if (s.law == RK_LAW_STICKEDLINKS && bond >= 0) {
          float kn, kt, kr, fn0, ft0, mom0, power;
          double dn0 = s.if_dn0[bond];
          if (s.params_in_interfaces == 1) {
            const double* q = s.if_par + 8 * (int64_t)bond;
            kn = d2f(q[0]); kt = d2f(q[1]); kr = d2f(q[2]); fn0 = d2f(q[3]); ft0 = d2f(q[4]);
            mom0 = d2f(q[5]); power = d2f(q[6]);
          } else if (s.cluster[i] == s.cluster[j]) {
            kn = d2f(P[RK_P_KN_IN]); kt = d2f(P[RK_P_KT_IN]); kr = d2f(P[RK_P_KR_IN]); fn0 = d2f(P[RK_P_FN0_IN]);
            ft0 = d2f(P[RK_P_FT0_IN]); mom0 = d2f(P[RK_P_MOM0_IN]); power = d2f(P[RK_P_POW_IN]);
            dn0 = 0.0;
          } else {
            kn = d2f(P[RK_P_KN_OUT]); kt = d2f(P[RK_P_KT_OUT]); kr = d2f(P[RK_P_KR_OUT]);
            fn0 = d2f(P[RK_P_FN0_OUT]); ft0 = d2f(P[RK_P_FT0_OUT]); mom0 = d2f(P[RK_P_MOM0_OUT]);
            power = d2f(P[RK_P_POW_OUT]);
          }
          float vn = dotf(cvel, n);
          fn = -f2d(kn) * (dn - dn0) + f2d(damp * vn);
          F3 vt = cvel - vn * n;
          ft = ft + (kt * dt) * vt;
          ft = ft + damp * vt;
          mom = mom + (kr * dt) * dw;
          float yield = powf(sqrtf(dotf(ft, ft)) / ft0, power) + powf(sqrtf(dotf(mom, mom)) / mom0, power) -
                        d2f(fn) / fn0 - 1.0f;
          if (yield > 0.f) s.if_break[bond] = 1;
        } else if (dn > 0.0) {
          fn = 0.0;
          ft = f3(0, 0, 0);
          mom = f3(0, 0, 0);
        } else if (s.law == RK_LAW_AVALANCHE) {
          const float kn = d2f(P[RK_P_KN]), en2 = d2f(P[RK_P_EN2]), kt = d2f(P[RK_P_KT]);
          const float mu = d2f(P[RK_P_MU]), kr = d2f(P[RK_P_KR]), mur = d2f(P[RK_P_MUR]);
          double prev_dn = ok ? dn_old : 0.0;
          if (prev_dn > 0.0) prev_dn = 0.0;
          double ddn = dn - prev_dn;
          if (ddn > 0.0) fn = -f2d(kn * en2) * dn;
          else if (ddn < 0.0) fn = fn - f2d(kn) * ddn;
          if (fn < 0.0) fn = 0.0;
          F3 vt = cvel - dotf(cvel, n) * n;
          ft = ft + (kt * dt) * vt;
          float thr = fabsf(mu * d2f(fn));
          float ft2 = dotf(ft, ft);
          if (ft2 > 0.f && ft2 > thr * thr) ft = (thr * rsqrtf(ft2)) * ft;
          mom = mom + (kr * dt) * dw;
          F3 br;
          F3 w0;
          if (i < s.n_driven) { br = cj; w0 = wj; }
          else { br = ci; w0 = wi; }
          float r = dotf(br, w0) / dotf(w0, w0);
          br = br - r * w0;
          float thm = fabsf(mur * sqrtf(dotf(br, br)) * d2f(fn));
          float m2 = dotf(mom, mom);
          if (m2 > 0.f && m2 > thm * thm) mom = (thm * rsqrtf(m2)) * mom;
        } else {  // Default law, and the contact branch of StickedLinks
          const float kn = d2f(P[RK_P_KN]), kt = d2f(P[RK_P_KT]), mu = d2f(P[RK_P_MU]);
          const float kr = d2f(P[RK_P_KR]), mur = d2f(P[RK_P_MUR]);
          const bool sticked = s.law == RK_LAW_STICKEDLINKS;
          float vn = dotf(cvel, n);
          double fne = -f2d(kn) * dn;
          fn = fne + f2d(damp * vn);
          if (fn < 0.0) fn = 0.0;
          F3 vt = cvel - vn * n;
          ft = ft + (kt * dt) * vt;
          float thr = fabsf(mu * d2f(sticked ? fn : fne));
          float ft2 = dotf(ft, ft);
          if (ft2 > 0.f && ft2 >= thr * thr) ft = (thr * rsqrtf(ft2)) * ft;
          if (sticked || kr > 0.f) {
            mom = mom + (kr * dt) * dw;
            float thm = fabsf(mur * d2f(fn));
            float m2 = dotf(mom, mom);
            if (m2 > 0.f && m2 >= thm * thm) mom = (thm * rsqrtf(m2)) * mom;
          }
        }
        F3 f = d2f(fn) * n + ft;
        st3m(s.cf, e, f);
        st3m(s.cmi, e, crossf(ci, f) + mom);
        st3m(s.cmj, e, crossf(cj, -f) - mom);
      }
    }
    // stores that change nothing are skipped: a lost sub-contact that was
    // lost already (dn -0.0, history zero); bonded entries always store
    const bool same = bond < 0 && !ok && lost_before(dn_old);
    if (!same) {
      s.dn[e] = dn;
      if (active || !ok) {
        s.fn[e] = fn;
        st3m(s.ft, e, ft);
        st3m(s.mom, e, mom);
      }
    }
    s.act[e] = active ? 1 : 0;
  }
  return active;
}

// Pass 1, every entry (threads follow the entries grouped by sub-contact
// type: fewer divergent branches per warp; measured 30 % faster than the
// storage order, whose loads coalesce but whose warps mix the types, and as
// fast as two entries per thread): an entry of no bond that FP32
// proves clearly apart or with its projection clearly outside (apart_f32)
// is finished here with FP32 alone -- a separated entry keeps its history
// and takes the FP32 estimate as its dn (only its sign is used), a lost
// sub-contact restarts its history from zero (dn -0.0) -- and stores only
// what changes.  The others go to the list of their type (one atomic per
// warp and type) for pass 2.  Warps of pass 1 thus issue almost no FP64
// instruction, and the FP64 path runs on dense warps of the entries that
// need it (on GB300, where each warp-wide FP64 instruction is expensive,
// a warp whose lanes mostly skip the FP64 path still pays for all of it).
__global__ void k_narrow_mixed_quick(Scene s) {
  if (step_halted(s)) return;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool slow = false;
  int type = 0, e = 0;
  if (k < s.ne) {
    e = s.nperm[k];
    const int bond = s.bond[e];
    const uint32_t ts = s.etsub[e];
    type = tsub_type(ts);
    int quick = 0;
    float dnf = 0.f;
    if (bond < 0 && !s.record_geom && s.gvr) {
      const int i = s.ei[e], j = s.ej[e];
      const int4 G = s.egv_ok ? s.egv[e] : make_int4(-1, -1, -1, -1);
      const float4 pi = s.posf[i], pj = s.posf[j];
      const F3 dxij = f3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
      const float cmag = fmaxf(fmaxf(fabsf(pi.x), fabsf(pi.y)), fmaxf(fabsf(pi.z), fmaxf(fabsf(pj.x),
                         fmaxf(fabsf(pj.y), fabsf(pj.z)))));
      quick = apart_f32(s, type, i, j, tsub_isub(ts), tsub_jsub(ts), s.egv_ok != 0, G, dxij, pi.w + pj.w, cmag,
                        &dnf);
    }
    if (quick == kApart) {  // dn > 0 proven: separated, history untouched
      const double dn_old = s.dn[e];
      if (!(dn_old > 0.0)) s.dn[e] = f2d(dnf);
      s.act[e] = 0;
    } else if (quick == kOutside) {  // the sub-contact lost
      if (!lost_before(s.dn[e])) {
        s.dn[e] = -0.0;
        s.fn[e] = 0.0;
        const F3 z = f3(0, 0, 0);
        st3m(s.ft, e, z);
        st3m(s.mom, e, z);
      }
      s.act[e] = 0;
    } else {
      slow = true;
    }
  }
  const int lane = threadIdx.x & 31;
  for (int t = 0; t < 4; t++) {
    const unsigned bal = __ballot_sync(0xffffffffu, slow && type == t);
    if (!bal) continue;
    unsigned long long base = 0;
    if (lane == __ffs(bal) - 1) base = atomicAdd(&s.flags[FLAG_NSLOW + t], (unsigned long long)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, __ffs(bal) - 1);
    if (slow && type == t) {
      const unsigned long long at = s.flags[FLAG_TOFS + t] + base + __popc(bal & ((1u << lane) - 1u));
      if (at < s.flags[FLAG_TOFS + t + 1]) s.slow[at] = e;
      else atomicOr(&s.flags[FLAG_ERROR], 1ull);  // cannot happen while nperm and its type runs agree
    }
  }
}

// Pass 2: the full path over the four lists, one after the other, by whole
// warps (grid-stride); the last block to finish empties the lists for the
// next step.  At least 5 blocks per SM: 96 registers, no spills, 20 warps
// per SM instead of 16 (latency-bound otherwise).
constexpr int kSlowThreads = 128;
__global__ void __launch_bounds__(kSlowThreads, 5) k_narrow_mixed_full(Scene s) {
  if (step_halted(s)) return;
  int64_t cnt[4], total = 0;
#pragma unroll
  for (int t = 0; t < 4; t++) {  // (a list never exceeds its type run)
    cnt[t] = min((int64_t)s.flags[FLAG_NSLOW + t], (int64_t)(s.flags[FLAG_TOFS + t + 1] - s.flags[FLAG_TOFS + t]));
    total += cnt[t];
  }
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * kSlowThreads) >> 5;
  for (int64_t base = ((blockIdx.x * (int64_t)kSlowThreads + threadIdx.x) >> 5) * 32; base < total;
       base += nwarps * 32) {
    const int64_t q = base + lane;
    bool active = false;
    if (q < total) {
      int t = 0;
      int64_t r = q;
#pragma unroll
      for (int u = 0; u < 3; u++)  // the list of q (constant indices: cnt stays in registers)
        if (t == u && r >= cnt[u]) {
          r -= cnt[u];
          t = u + 1;
        }
      active = narrow_mixed_full(s, s.slow[(int64_t)s.flags[FLAG_TOFS + t] + r]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, active);
    if (lane == 0 && m) atomicAdd(&s.flags[FLAG_NACTIVE], (unsigned long long)__popc(m));
  }
  __syncthreads();  // every thread of the block has read the counts
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long arrived = atomicAdd(&s.flags[FLAG_SLOW_TICKET], 1ull);
    if (arrived == gridDim.x - 1ull) {
      for (int t = 0; t < 4; t++) s.flags[FLAG_NSLOW + t] = 0ull;
      s.flags[FLAG_SLOW_TICKET] = 0ull;
    }
  }
}

int launch_narrow_force_mixed(const Scene& s, cudaStream_t st) {
  if (s.ne <= 0) return 0;
  const int t = s.tpb[0] > 0 ? s.tpb[0] : 128;
  k_narrow_mixed_quick<<<(unsigned)((s.ne + t - 1) / t), t, 0, st>>>(s);
  // enough warps for every entry to have a lane, up to 16 blocks per SM
  const int64_t blocks = std::min<int64_t>((s.ne + kSlowThreads - 1) / kSlowThreads, 152 * 16);
  k_narrow_mixed_full<<<(unsigned)blocks, kSlowThreads, 0, st>>>(s);
  return 2;
}
cudaError_t narrow_mixed_attributes(cudaFuncAttributes* a) { return cudaFuncGetAttributes(a, k_narrow_mixed_quick); }

}  // namespace rk
