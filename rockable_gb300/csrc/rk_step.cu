// rk_step.cu -- per-step kernels of the FP64 engine (velocity-Verlet step of
// Rockable::velocityVerletStep with the accelerations() pipeline).
//
// Kernel sequence of one step:
//   controls_pre  (1 thread)        servo + driven bodies        Rockable.cpp:1979-2033, DrivingSystem.cpp:251-268
//   drift         (thread / body)   first half-kick + drift      Rockable.cpp:2036-2055
//   glob_vertices (thread / vertex) global vertex positions      Particle.cpp:55-65
//   narrow_force  (thread / entry)  update + force law + f, M    Interaction.cpp:143-326, ForceLaw_*.cpp,
//                                                                Rockable.cpp:2934-3046, 2752-2789
//   gather_accel  (thread / body)   ordered resultants, Newton-  Rockable.cpp:3220-3275, 3419-3552,
//                                   Euler, second half-kick      3806-3868, 2131-2155
//   bond_break / iface_break        postponed bond rupture       Rockable.cpp:3350-3413
//
// Bit parity: compiled with --fmad=false; the resultant of every body is
// summed in the reference's serial order (entries in key order), so the FP64
// form reproduces the CPU path bit for bit.
#include <cstdio>

#include "../../include/rk_gpu.h"
#include "rk_engine.cuh"
#include "rk_guard.cuh"
#define RK_BODY_NS exact
#include "rk_body.cuh"

namespace rk {

// ----------------------------------------------------------------- K0 ----
__global__ void k_controls_pre(Scene s) {
  if (step_halted(s)) return;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (s.servo_kind == 1) {  // tritriIsostaticCompression
    const int* w = s.servo_walls;
    const double Xmin = s.pos[3 * w[0] + 0] + s.rad[w[0]];
    const double Xmax = s.pos[3 * w[1] + 0] - s.rad[w[1]];
    const double Ymin = s.pos[3 * w[2] + 1] + s.rad[w[2]];
    const double Ymax = s.pos[3 * w[3] + 1] - s.rad[w[3]];
    const double Zmin = s.pos[3 * w[4] + 2] + s.rad[w[4]];
    const double Zmax = s.pos[3 * w[5] + 2] - s.rad[w[5]];
    const double dX = fabs(Xmax - Xmin), dY = fabs(Ymax - Ymin), dZ = fabs(Zmax - Zmin);
    const double surfX = dY * dZ, surfY = dX * dZ, surfZ = dY * dX;
    s.controls[s.servo_icontr + 1].value = -s.servo_p * surfX;
    s.controls[s.servo_icontr + 3].value = -s.servo_p * surfY;
    s.controls[s.servo_icontr + 5].value = -s.servo_p * surfZ;
  }
  // velocityControlledDrive (Rockable.cpp:1856-1900)
  for (int k = 0; k < s.ncontrols; k++) {
    const Control c = s.controls[k];
    int b = c.body;
    switch (c.type) {
      case RK_X_VEL: s.vel[3 * b] = c.value; s.pos[3 * b] += s.dt * c.value; break;
      case RK_Y_VEL: s.vel[3 * b + 1] = c.value; s.pos[3 * b + 1] += s.dt * c.value; break;
      case RK_Z_VEL: s.vel[3 * b + 2] = c.value; s.pos[3 * b + 2] += s.dt * c.value; break;
      case RK_XROT_VEL: case RK_YROT_VEL: case RK_ZROT_VEL: case RK_XYZROT_VEL: {
        V3 w;
        if (c.type == RK_XROT_VEL) w = v3(c.value, 0.0, 0.0);
        else if (c.type == RK_YROT_VEL) w = v3(0.0, c.value, 0.0);
        else if (c.type == RK_ZROT_VEL) w = v3(0.0, 0.0, c.value);
        else w = v3(c.vec[0], c.vec[1], c.vec[2]);
        Q4 q = ldq(s.Q, b);
        qaddscaled(q, qdot(q, w), s.dt);
        qnormalize(q);
        stq(s.Q, b, q);
      } break;
      default: break;
    }
  }
  // force-driven components (Rockable.cpp:1988-2033)
  for (int k = 0; k < s.ncontrols; k++) {
    const Control c = s.controls[k];
    int b = c.body;
    switch (c.type) {
      case RK_X_FOR: case RK_Y_FOR: case RK_Z_FOR: {
        int d = c.type - RK_X_FOR;
        s.pos[3 * b + d] += s.dt * s.vel[3 * b + d] + s.dt2_2 * s.acc[3 * b + d];
        s.vel[3 * b + d] += s.dt_2 * s.acc[3 * b + d];
      } break;
      case RK_XROT_MOM: case RK_YROT_MOM: case RK_ZROT_MOM: case RK_XYZROT_MOM: {
        V3 wr = ld3(s.vrot, b), ar = ld3(s.arot, b);
        V3 w;
        if (c.type == RK_XROT_MOM) w = wr.x * v3(1.0, 0.0, 0.0);
        else if (c.type == RK_YROT_MOM) w = wr.y * v3(0.0, 1.0, 0.0);
        else if (c.type == RK_ZROT_MOM) w = wr.z * v3(0.0, 0.0, 1.0);
        else w = wr;
        Q4 q = ldq(s.Q, b);
        qaddscaled(q, qdot(q, w), s.dt);
        qnormalize(q);
        stq(s.Q, b, q);
        if (c.type == RK_XROT_MOM) wr.x += s.dt_2 * ar.x;
        else if (c.type == RK_YROT_MOM) wr.y += s.dt_2 * ar.y;
        else if (c.type == RK_ZROT_MOM) wr.z += s.dt_2 * ar.z;
        else wr = wr + s.dt_2 * ar;
        st3(s.vrot, b, wr);
      } break;
      default: break;
    }
  }
}

// --------------------------------------------------------- force laws ----
struct LawIn {
  double dn, dn_old, damp;
  V3 n, vel, cpos;
  V3 wi, wj, xi, xj;
  bool i_driven;
  int gi, gj;     // groups
  int ci, cj;     // clusters
  int bond;
};

__device__ __forceinline__ void law_default(const Scene& s, const LawIn& L, double& fn, V3& ft, V3& mom) {
  if (L.dn > 0.0) { fn = 0.0; ft = v3(0, 0, 0); mom = v3(0, 0, 0); return; }
  const double* P = s.table[L.gi * s.ngroup + L.gj].p;
  double kn = P[RK_P_KN], kt = P[RK_P_KT], mu = P[RK_P_MU], kr = P[RK_P_KR], mur = P[RK_P_MUR];
  double vn = dot(L.vel, L.n);
  double fne = -kn * L.dn;
  double fnv = L.damp * vn;
  fn = fne + fnv;
  if (fn < 0.0) fn = 0.0;
  V3 vt = L.vel - vn * L.n;
  ft = ft + kt * (vt * s.dt);
  double threshold = fabs(mu * fne);
  double ft2 = dot(ft, ft);
  if (ft2 > 0.0 && ft2 >= threshold * threshold) ft = ft * (threshold / sqrt(ft2));
  if (kr > 0.0) {
    mom = mom + (kr * (L.wj - L.wi)) * s.dt;
    double thr = fabs(mur * fn);
    double m2 = dot(mom, mom);
    if (m2 > 0.0 && m2 >= thr * thr) mom = mom * (thr / sqrt(m2));
  }
}

__device__ __forceinline__ void law_avalanche(const Scene& s, const LawIn& L, double& fn, V3& ft, V3& mom) {
  if (L.dn > 0.0) { fn = 0.0; ft = v3(0, 0, 0); mom = v3(0, 0, 0); return; }
  const double* P = s.table[L.gi * s.ngroup + L.gj].p;
  double kn = P[RK_P_KN], en2 = P[RK_P_EN2], kt = P[RK_P_KT], mu = P[RK_P_MU], kr = P[RK_P_KR], mur = P[RK_P_MUR];
  double prev_dn = L.dn_old;
  if (prev_dn > 0.0) prev_dn = 0.0;
  double ddn = L.dn - prev_dn;
  if (ddn > 0.0) fn = -kn * en2 * L.dn;
  else if (ddn < 0.0) fn = fn + -kn * ddn;
  if (fn < 0.0) fn = 0.0;
  V3 vt = L.vel - dot(L.vel, L.n) * L.n;
  ft = ft + kt * (s.dt * vt);
  double thr = fabs(mu * fn);
  double ft2 = dot(ft, ft);
  if (ft2 > 0.0 && ft2 > thr * thr) ft = ft * (thr / sqrt(ft2));
  mom = mom + (kr * (L.wj - L.wi)) * s.dt;
  V3 branch;
  if (L.i_driven) {
    branch = L.cpos - L.xj;
    double r = dot(branch, L.wj) / dot(L.wj, L.wj);
    branch = branch - r * L.wj;
  } else {
    branch = L.cpos - L.xi;
    double r = dot(branch, L.wi) / dot(L.wi, L.wi);
    branch = branch - r * L.wi;
  }
  double thm = fabs(mur * sqrt(norm2(branch)) * fn);
  double m2 = dot(mom, mom);
  if (m2 > 0.0 && m2 > thm * thm) mom = mom * (thm / sqrt(m2));
}

__device__ __forceinline__ void law_sticked(const Scene& s, const LawIn& L, double& fn, V3& ft, V3& mom) {
  if (L.bond >= 0) {
    double kn, kt, kr, fn0, ft0, mom0, power;
    double dn0 = s.if_dn0[L.bond];
    bool inner = (L.ci == L.cj);
    if (s.params_in_interfaces == 1) {
      const double* q = s.if_par + 8 * (int64_t)L.bond;
      kn = q[0]; kt = q[1]; kr = q[2]; fn0 = q[3]; ft0 = q[4]; mom0 = q[5]; power = q[6];
    } else {
      const double* P = s.table[L.gi * s.ngroup + L.gj].p;
      if (inner) {
        kn = P[RK_P_KN_IN]; kt = P[RK_P_KT_IN]; kr = P[RK_P_KR_IN]; fn0 = P[RK_P_FN0_IN]; ft0 = P[RK_P_FT0_IN];
        mom0 = P[RK_P_MOM0_IN]; power = P[RK_P_POW_IN];
        dn0 = 0.0;
      } else {
        kn = P[RK_P_KN_OUT]; kt = P[RK_P_KT_OUT]; kr = P[RK_P_KR_OUT]; fn0 = P[RK_P_FN0_OUT]; ft0 = P[RK_P_FT0_OUT];
        mom0 = P[RK_P_MOM0_OUT]; power = P[RK_P_POW_OUT];
      }
    }
    double vn = dot(L.vel, L.n);
    double fne = -kn * (L.dn - dn0);
    double fnv = L.damp * vn;
    fn = fne + fnv;
    V3 vt = (L.vel - (vn * L.n));
    ft = ft + kt * (vt * s.dt);
    V3 ftv = L.damp * vt;
    ft = ft + ftv;
    mom = mom + (kr * (L.wj - L.wi)) * s.dt;
    double yield = pow(sqrt(norm2(ft)) / ft0, power) + pow(sqrt(norm2(mom)) / mom0, power) - fn / fn0 - 1.0;
    if (yield > 0.0) s.if_break[L.bond] = 1;
  } else {
    if (L.dn > 0.0) { fn = 0.0; ft = v3(0, 0, 0); mom = v3(0, 0, 0); return; }
    const double* P = s.table[L.gi * s.ngroup + L.gj].p;
    double kn = P[RK_P_KN], kt = P[RK_P_KT], mu = P[RK_P_MU], kr = P[RK_P_KR], mur = P[RK_P_MUR];
    double vn = dot(L.vel, L.n);
    double fne = -kn * L.dn;
    double fnv = L.damp * vn;
    fn = fne + fnv;
    if (fn < 0.0) fn = 0.0;
    V3 vt = L.vel - vn * L.n;
    ft = ft + kt * (vt * s.dt);
    double thr = fabs(mu * fn);
    double ft2 = dot(ft, ft);
    if (ft2 > 0.0 && ft2 >= thr * thr) ft = ft * (thr / sqrt(ft2));
    mom = mom + (kr * (L.wj - L.wi)) * s.dt;
    double thm = fabs(mur * fn);
    double m2 = dot(mom, mom);
    if (m2 > 0.0 && m2 >= thm * thm) mom = mom * (thm / sqrt(m2));
  }
}

// ----------------------------------------------------------------- K2 ----
__device__ __forceinline__ V3 gvx(const double* g, int k) { return v3(g[3 * k], g[3 * k + 1], g[3 * k + 2]); }

__global__ void k_narrow_force(Scene s) {
  if (step_halted(s)) return;
  // threads follow the entries grouped by sub-contact type (fewer divergent
  // branches per warp); every entry is computed on its own
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool active = false;
  if (k < s.ne) {
    const int64_t e = s.nperm[k];
    const int i = s.ei[e], j = s.ej[e];
    const uint32_t ts = s.etsub[e];
    const int type = tsub_type(ts), isub = tsub_isub(ts), jsub = tsub_jsub(ts);
    const double dn_old = s.dn[e];
    const int bond = s.bond[e];
    const double* gi = s.gv + 3 * s.gv_ofs[i];
    const double* gj = s.gv + 3 * s.gv_ofs[j];
    const double Ri = s.rad[i], Rj = s.rad[j];
    V3 n = v3(0, 0, 0), cpos = v3(0, 0, 0);
    double dn = 0.0;
    bool ok = true;
    if (type == 0) {  // vertex-vertex
      V3 a = gvx(gi, isub), b = gvx(gj, jsub);
      n = a - b;
      dn = normalize(n) - (Ri + Rj);
      cpos = a - n * (Ri + 0.5 * dn);
    } else if (type == 1) {  // vertex-edge
      const int sj = s.shape[j];
      const int eo = s.edge_ofs[sj] + jsub;
      V3 p1 = gvx(gj, s.edges[2 * eo]), p2 = gvx(gj, s.edges[2 * eo + 1]);
      V3 a = gvx(gi, isub);
      V3 E = p2 - p1, v = a - p1;
      double r = dot(v, E) / dot(E, E);
      if (r <= 0.0 || r >= 1.0) {
        ok = false;
      } else {
        n = a - (p1 + r * E);
        dn = normalize(n) - (Ri + Rj);
        cpos = a - n * (Ri + 0.5 * dn);
      }
    } else if (type == 2) {  // vertex-face
      const int sj = s.shape[j];
      const int fo = s.face_ofs[sj] + jsub;
      const int v0 = s.face_vofs[fo], nbv = s.face_vofs[fo + 1] - v0;
      const int* fv = s.face_verts + v0;
      V3 A = gvx(gj, fv[0]), B = gvx(gj, fv[1]), C = gvx(gj, fv[nbv - 1]);
      V3 a = gvx(gi, isub);
      V3 v = a - A;
      V3 v1 = B - A;
      normalize(v1);
      V3 v2 = C - A;
      n = cross(v1, v2);
      normalize(n);
      double dist = dot(v, n);
      if (dist < 0.0) { n = -n; dist = -dist; }
      V3 P = a - dist * n;
      int odd = 0;
      v2 = cross(n, v1);
      double ori1 = dot(P, v1), ori2 = dot(P, v2);
      for (int iva = 0; iva < nbv; ++iva) {
        int ivb = iva + 1;
        if (ivb == nbv) ivb = 0;
        V3 pa = gvx(gj, fv[iva]), pb = gvx(gj, fv[ivb]);
        double pa1 = dot(pa, v1), pb1 = dot(pb, v1), pa2 = dot(pa, v2), pb2 = dot(pb, v2);
        if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
          if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
        }
      }
      if (odd) {
        dn = dist - (Ri + Rj);
        cpos = a - n * (Ri + 0.5 * dn);
      } else {
        ok = false;
      }
    } else {  // edge-edge
      const int si = s.shape[i], sj = s.shape[j];
      const int eoi = s.edge_ofs[si] + isub, eoj = s.edge_ofs[sj] + jsub;
      V3 pi1 = gvx(gi, s.edges[2 * eoi]), pi2 = gvx(gi, s.edges[2 * eoi + 1]);
      V3 pj1 = gvx(gj, s.edges[2 * eoj]), pj2 = gvx(gj, s.edges[2 * eoj + 1]);
      V3 Ei = pi2 - pi1, Ej = pj2 - pj1, v = pi1 - pj1;
      double c = dot(Ei, Ei), d = dot(Ej, Ej), ee = dot(Ei, Ej);
      double f = (c * d) - (ee * ee);
      if (fabs(f) > 1.0e-12) {
        f = 1.0 / f;
        double a = dot(Ei, v), b = dot(Ej, v);
        double ss = (ee * b - a * d) * f;
        double tt = (c * b - ee * a) * f;
        if (ss <= 0.0 || ss >= 1.0 || tt <= 0.0 || tt >= 1.0) {
          ok = false;
        } else {
          n = (pi1 + ss * Ei) - (pj1 + tt * Ej);
          dn = normalize(n) - (Ri + Rj);
          cpos = pi1 + ss * Ei - n * (Ri + 0.5 * dn);
        }
      } else {
        ok = false;
      }
    }
    const V3 xi = ld3(s.pos, i), xj = ld3(s.pos, j);
    const V3 wi = ld3(s.vrot, i), wj = ld3(s.vrot, j);
    V3 cvel;
    double fn;
    V3 ft, mom;
    if (ok) {
      const V3 vi = ld3(s.vel, i), vj = ld3(s.vel, j);
      cvel = (vj - cross(cpos - xj, wj)) - (vi - cross(cpos - xi, wi));
      fn = s.fn[e];
      ft = ld3(s.ft, e);
      mom = ld3(s.mom, e);
      if (s.record_geom || bond >= 0) {
        st3(s.gn, e, n);
        st3(s.gpos, e, cpos);
        st3(s.gvel, e, cvel);
      }
    } else {  // Interaction::deactivate (Interaction.cpp:123-128)
      dn = 0.0;
      fn = 0.0;
      ft = v3(0, 0, 0);
      mom = v3(0, 0, 0);
      if (bond >= 0) {  // a bonded entry stays active with its previous geometry
        n = ld3(s.gn, e);
        cpos = ld3(s.gpos, e);
        cvel = ld3(s.gvel, e);
      } else {
        cvel = v3(0, 0, 0);
      }
    }
    active = (dn < 0.0 || bond >= 0);
    if (active) {
      LawIn L;
      L.dn = dn; L.dn_old = ok ? dn_old : 0.0; L.damp = s.damp[e];
      L.n = n; L.vel = cvel; L.cpos = cpos;
      L.wi = wi; L.wj = wj; L.xi = xi; L.xj = xj;
      L.i_driven = i < s.n_driven;
      L.gi = s.group[i]; L.gj = s.group[j];
      L.ci = s.cluster[i]; L.cj = s.cluster[j];
      L.bond = bond;
      if (s.law == RK_LAW_AVALANCHE) law_avalanche(s, L, fn, ft, mom);
      else if (s.law == RK_LAW_STICKEDLINKS) law_sticked(s, L, fn, ft, mom);
      else law_default(s, L, fn, ft, mom);
      // Rockable::incrementResultants (Rockable.cpp:2752-2789)
      V3 f = fn * n + ft;
      V3 Ci = (cpos - xi), Cj = (cpos - xj);
      st3(s.cf, e, f);
      st3(s.cmi, e, cross(Ci, f) + mom);
      st3(s.cmj, e, cross(Cj, -f) - mom);
    }
    s.dn[e] = dn;
    if (active || !ok) {
      s.fn[e] = fn;
      st3(s.ft, e, ft);
      st3(s.mom, e, mom);
    }
    s.act[e] = active ? 1 : 0;
  }
  unsigned m = __ballot_sync(0xffffffffu, active);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(&s.flags[FLAG_NACTIVE], (unsigned long long)__popc(m));
}

// ----------------------------------------------------------------- K3 ----
// Bodies with many entries: one warp per body.  The lanes load 32 positions
// of the serial order at a time (the j-side entries before the body's own
// block, its block, the rest of the j-side: jsplit), and lanes 0-5 each add
// one of the six components (F.x, F.y, F.z, M.x, M.y, M.z) of those 32
// contributions, broadcast by shuffles, in that order: the same sums as the
// one-thread loop (F - f added as F + (-f), which IEEE arithmetic makes the
// same number), six short chains instead of one long one.
constexpr int kHeavyWarps = 4;  // warps per block
__global__ void __launch_bounds__(32 * kHeavyWarps) k_gather_heavy(Scene s, const int* list, int count) {
  if (step_halted(s)) return;
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const int b = list[w];
  const int64_t i0 = s.iofs[b], i1 = s.iofs[b + 1];
  const int64_t j0 = s.jofs[b], j1 = s.jofs[b + 1], js = s.jsplit[b];
  const int64_t nA = js - j0, nB = i1 - i0, L = nA + nB + (j1 - js);
  V3 F, M;
  init_resultant(s, b, F, M);
  const double start[6] = {F.x, F.y, F.z, M.x, M.y, M.z};
  double acc = lane < 6 ? start[lane] : 0.0;
  for (int64_t c0 = 0; c0 < L; c0 += 32) {
    const int64_t p = c0 + lane;
    int valid = 0;
    double c[6] = {0, 0, 0, 0, 0, 0};
    if (p < L) {
      int64_t e;
      bool jside;
      if (p < nA) { e = s.jlist[j0 + p]; jside = true; }
      else if (p < nA + nB) { e = i0 + (p - nA); jside = false; }
      else { e = s.jlist[js + (p - nA - nB)]; jside = true; }
      if (s.act[e]) {
        valid = 1;
        const V3 f = ld3(s.cf, e), m = jside ? ld3(s.cmj, e) : ld3(s.cmi, e);
        c[0] = jside ? -f.x : f.x;
        c[1] = jside ? -f.y : f.y;
        c[2] = jside ? -f.z : f.z;
        c[3] = m.x; c[4] = m.y; c[5] = m.z;
      }
    }
    const unsigned any = __ballot_sync(0xffffffffu, valid);
    const int nk = (int)min((int64_t)32, L - c0);
    for (int k = 0; k < nk; k++) {
      if (!((any >> k) & 1u)) continue;
      const double v0 = __shfl_sync(0xffffffffu, c[0], k), v1 = __shfl_sync(0xffffffffu, c[1], k);
      const double v2 = __shfl_sync(0xffffffffu, c[2], k), v3_ = __shfl_sync(0xffffffffu, c[3], k);
      const double v4 = __shfl_sync(0xffffffffu, c[4], k), v5 = __shfl_sync(0xffffffffu, c[5], k);
      const double v = lane == 0 ? v0 : lane == 1 ? v1 : lane == 2 ? v2 : lane == 3 ? v3_ : lane == 4 ? v4 : v5;
      if (lane < 6) acc = acc + v;
    }
  }
  if (lane < 3) s.force[3 * (int64_t)b + lane] = acc;
  else if (lane < 6) s.moment[3 * (int64_t)b + lane - 3] = acc;
}

// ----------------------------------------------------------------- K4 ----
__global__ void k_bond_break(Scene s) {
  if (step_halted(s)) return;
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.ne) return;
  int bond = s.bond[e];
  if (bond < 0 || !s.if_break[bond]) return;
  s.bond[e] = -1;
  if (s.dn[e] >= 0.0) {
    s.fn[e] = 0.0;
    st3(s.ft, e, v3(0, 0, 0));
  } else {
    V3 T = ld3(s.ft, e);
    double FT = normalize(T);
    int gi = s.group[s.if_i[bond]], gj = s.group[s.if_j[bond]];
    double mu = s.table[gi * s.ngroup + gj].p[RK_P_MU];
    double thr = fabs(mu * s.fn[e]);
    if (FT > thr) st3(s.ft, e, thr * T);
  }
}

__global__ void k_iface_break(Scene s) {
  if (step_halted(s)) return;
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= s.nif) return;
  if (!s.if_break[k]) return;
  s.if_break[k] = 0;
  if (!s.if_broken[k]) {
    s.if_broken[k] = 1;
    atomicAdd(&s.flags[FLAG_NBROKEN], 1ull);
    s.flags[FLAG_NEED_UPDATE] = 1ull;
  }
}

// ---------------------------------------------------- dynamic NL guard ----
// Rockable.cpp:1571-1596: accumulated displacement and rotation since the
// last guard-triggered update; running maxima are kept in the flag block.
__global__ void k_guard(Scene s) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double t1 = 0.0, t2 = 0.0;
  if (i < s.n) {
    V3 dp = ld3(s.dpos, i);
    Q4 dq = ldq(s.dq, i);
    if (s.flags[FLAG_GRESET]) {
      dp = v3(0, 0, 0);
      dq = q4(1.0, 0.0, 0.0, 0.0);
    }
    dp = dp + ld3(s.vel, i) * s.dt;
    t1 = norm2(dp);
    qaddscaled(dq, qdot(ldq(s.Q, i), ld3(s.vrot, i)), s.dt);
    t2 = qangle(dq);
    st3(s.dpos, i, dp);
    stq(s.dq, i, dq);
  }
  // both are >= 0: the IEEE bit patterns order like the values
  for (int o = 16; o > 0; o >>= 1) {
    t1 = fmax(t1, __shfl_xor_sync(0xffffffffu, t1, o));
    t2 = fmax(t2, __shfl_xor_sync(0xffffffffu, t2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&s.flags[FLAG_GPOS], (unsigned long long)__double_as_longlong(t1));
    atomicMax(&s.flags[FLAG_GROT], (unsigned long long)__double_as_longlong(t2));
  }
}

__global__ void k_guard_finalize(Scene s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  s.flags[FLAG_GRESET] = 0ull;
  double mp = sqrt(__longlong_as_double((long long)s.flags[FLAG_GPOS]));
  double mr = __longlong_as_double((long long)s.flags[FLAG_GROT]);
  if (mp >= s.disp_update || mr >= s.angle_update) {
    s.flags[FLAG_NEED_UPDATE] = 1ull;
    s.flags[FLAG_GRESET] = 1ull;
    s.flags[FLAG_GPOS] = 0ull;
    s.flags[FLAG_GROT] = 0ull;
  }
}

// kinetic energies (Rockable.cpp:3958-3970), two partial sums per block
__global__ void k_kinetic(Scene s, double* out) {
  __shared__ double sh[2][256];
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double et = 0.0, er = 0.0;
  if (i < s.n) {
    V3 v = ld3(s.vel, i);
    et = s.mass[i] * dot(v, v);
    V3 w = qrot(qconj(ldq(s.Q, i)), ld3(s.vrot, i));
    V3 I = ld3(s.inertia, i);
    er = I.x * w.x * w.x + I.y * w.y * w.y + I.z * w.z * w.z;
  }
  sh[0][threadIdx.x] = et;
  sh[1][threadIdx.x] = er;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = sh[0][0];
    out[2 * blockIdx.x + 1] = sh[1][0];
  }
}

// ------------------------------------------------------------ launchers ----
static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int launch_controls_pre(const Scene& s, cudaStream_t st) {
  if (s.ncontrols == 0 && s.servo_kind == 0) return 0;
  k_controls_pre<<<1, 32, 0, st>>>(s);
  return 1;
}
static inline int tpb_or(const Scene& s, int k, int d) { return s.tpb[k] > 0 ? s.tpb[k] : d; }

// The per-body kernels come in two builds (rk_body.cuh): exact (this file,
// no contraction) and fused (rk_fast.cu), the latter for the mixed form.
// h v of every body vertex (shape frame), FP64 and FP32: a vertex's
// placement then reads one record instead of the chain body -> shape ->
// shape vertex offset -> shape vertex.
__global__ void k_body_verts(Scene s) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= s.nvert) return;
  const int b = s.gv_body[k];
  const double* sv = s.svert + 3 * ((int64_t)s.vert_ofs[s.shape[b]] + (k - s.gv_ofs[b]));
  const double h = s.hom[b];
  const double u[3] = {h * sv[0], h * sv[1], h * sv[2]};
  for (int d = 0; d < 3; d++) s.uv64[3 * k + d] = u[d];
  s.uvf[k] = make_float4((float)u[0], (float)u[1], (float)u[2], 0.f);
}
int launch_body_verts(const Scene& s, cudaStream_t st) {
  if (s.nvert <= 0) return 0;
  k_body_verts<<<nblk(s.nvert, 256), 256, 0, st>>>(s);
  return 1;
}

int launch_drift(const Scene& s, cudaStream_t st) {
  int64_t nf = s.n - s.n_driven;
  if (nf <= 0) return 0;
  const int t = tpb_or(s, 3, 128);
  if (s.fast_body) return 0;  // made by the step's body-frame launch (launch_glob_vertices)
  exact::k_drift<<<nblk(nf, t), t, 0, st>>>(s);
  return 1;
}
int launch_glob_vertices(const Scene& s, cudaStream_t st, bool all, const uint8_t* mark) {
  const int64_t nv = all || s.fast_body ? s.nvert : s.nlv;
  if (nv <= 0) return 0;
  const int t = tpb_or(s, 2, 256);
  if (s.fast_body) {
    // the mixed form's step needs only the FP32 offsets and the FP64 frames;
    // a list update needs the FP64 world vertices as well
    int k = launch_body_frames(s, nblk(s.n, t), t, all ? 0 : 1, st);
    if (all) k += launch_fused_glob(s, nblk(nv, t), t, 0, mark, st);
    return k;
  }
  exact::k_glob_vertices<<<nblk(nv, t), t, 0, st>>>(s, all ? 0 : 1, all ? mark : nullptr);
  return 1;
}
int launch_narrow_force(const Scene& s, cudaStream_t st) {
  if (s.ne <= 0) return 0;
  const int t = tpb_or(s, 0, 128);
  k_narrow_force<<<nblk(s.ne, t), t, 0, st>>>(s);
  return 1;
}
int launch_gather_accel(const Scene& s, int apply_kick, cudaStream_t st) {
  if (s.n <= 0) return 0;
  // (a batched skin step zeroes it in k_skin_begin)
  if (s.sk_out && apply_kick && !s.sk_ctl) cudaMemsetAsync(s.sk_out, 0, 8 * sizeof(unsigned int), st);
  const int t = tpb_or(s, 1, 128);
  if (s.fast_body) return launch_fused_gather(s, nblk(s.n, t), t, apply_kick, st);  // one body per thread
  exact::k_gather_accel<<<nblk(s.n, t), t, 0, st>>>(s, apply_kick);
  return 1;
}

// Largest block each tuned kernel can be launched with (register limit).
int max_tpb(int which, int form_mixed) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaSuccess;
  if (which == 0) e = form_mixed ? narrow_mixed_attributes(&a) : cudaFuncGetAttributes(&a, k_narrow_force);
  else if (form_mixed) e = fused_attributes(which, &a);
  else if (which == 1) e = cudaFuncGetAttributes(&a, exact::k_gather_accel);
  else if (which == 2) e = cudaFuncGetAttributes(&a, exact::k_glob_vertices);
  else e = cudaFuncGetAttributes(&a, exact::k_drift);
  return e == cudaSuccess ? a.maxThreadsPerBlock : 128;
}
int launch_gather_heavy(const Scene& s, cudaStream_t st) {
  if (s.nheavy <= 0) return 0;
  if (s.fast_body) return launch_fused_heavy(s, s.heavy, (int)s.nheavy, st);
  k_gather_heavy<<<(unsigned)((s.nheavy + kHeavyWarps - 1) / kHeavyWarps), 32 * kHeavyWarps, 0, st>>>(
      s, s.heavy, (int)s.nheavy);
  return 1;
}
int launch_gather_heavy_lazy(const Scene& s, cudaStream_t st) {
  if (s.nheavy_lazy <= 0) return 0;
  if (s.fast_body) return launch_fused_heavy(s, s.heavy_lazy, (int)s.nheavy_lazy, st);
  k_gather_heavy<<<(unsigned)((s.nheavy_lazy + kHeavyWarps - 1) / kHeavyWarps), 32 * kHeavyWarps, 0, st>>>(
      s, s.heavy_lazy, (int)s.nheavy_lazy);
  return 1;
}
int launch_breakage(const Scene& s, cudaStream_t st) {
  if (s.nif <= 0) return 0;
  int k = 0;
  if (s.ne > 0) { k_bond_break<<<nblk(s.ne, 256), 256, 0, st>>>(s); k++; }
  k_iface_break<<<nblk(s.nif, 256), 256, 0, st>>>(s);
  return k + 1;
}
int launch_guard(const Scene& s, cudaStream_t st) {
  if (s.n <= 0) return 0;
  k_guard<<<nblk(s.n, 128), 128, 0, st>>>(s);
  k_guard_finalize<<<1, 32, 0, st>>>(s);
  return 2;
}
// Packed kinematics: stage = pos (3n) | vel (3n) | acc (3n) | Q (4n) |
// vrot (3n) | arot (3n); dir 0 scatters it into the body arrays, 1 gathers.
__global__ void k_kin_pack(Scene s, double* stage, int dir) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n = s.n;
  if (k >= 19 * n) return;
  double* dst;
  int64_t off;
  if (k < 9 * n) {
    const int64_t a = k / (3 * n);
    off = k - a * 3 * n;
    dst = a == 0 ? s.pos : (a == 1 ? s.vel : s.acc);
  } else if (k < 13 * n) {
    off = k - 9 * n;
    dst = s.Q;
  } else {
    const int64_t a = (k - 13 * n) / (3 * n);
    off = k - 13 * n - a * 3 * n;
    dst = a == 0 ? s.vrot : s.arot;
  }
  if (dir == 0) dst[off] = stage[k];
  else stage[k] = dst[off];
}
int launch_kin_pack(const Scene& s, double* stage, int dir, cudaStream_t st) {
  if (s.n <= 0) return 0;
  k_kin_pack<<<nblk(19 * s.n, 256), 256, 0, st>>>(s, stage, dir);
  return 1;
}

int launch_kinetic_energy(const Scene& s, double* d_out2, cudaStream_t st) {
  if (s.n <= 0) return 0;
  k_kinetic<<<nblk(s.n, 256), 256, 0, st>>>(s, d_out2);
  return (int)nblk(s.n, 256);
}

}  // namespace rk
