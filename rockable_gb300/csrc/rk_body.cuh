// rk_body.cuh -- per-body kernels of the step (drift, world vertices of the
// listed bodies, resultants + Newton-Euler + second half-kick with the fused
// learned-skin guard), included twice: by rk_step.cu, compiled without
// contraction into fused multiply-adds (kernels in rk::exact, the FP64 form
// that reproduces the reference arithmetic bit for bit), and by rk_fast.cu,
// compiled with it (rk::fused: only the world-vertex kernel, with
// RK_BODY_GLOB_ONLY defined; the mixed form has its own drift and resultant
// kernels there).  Define RK_BODY_NS before including.
#ifndef RK_BODY_HELPERS
#define RK_BODY_HELPERS
#include "rk_engine.cuh"
#include "rk_guard.cuh"

namespace rk {

__device__ __forceinline__ V3 ld3(const double* a, int64_t k) { return v3(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }
__device__ __forceinline__ void st3(double* a, int64_t k, V3 v) {
  a[3 * k] = v.x;
  a[3 * k + 1] = v.y;
  a[3 * k + 2] = v.z;
}
__device__ __forceinline__ Q4 ldq(const double* a, int64_t k) {
  return q4(a[4 * k], a[4 * k + 1], a[4 * k + 2], a[4 * k + 3]);
}
__device__ __forceinline__ void stq(double* a, int64_t k, Q4 q) {
  a[4 * k] = q.s;
  a[4 * k + 1] = q.v.x;
  a[4 * k + 2] = q.v.y;
  a[4 * k + 3] = q.v.z;
}

__device__ __forceinline__ V3 euler_domega(V3 I, V3 w, V3 M) {
  return v3((M.x - (I.z - I.y) * w.y * w.z) / I.x, (M.y - (I.x - I.z) * w.z * w.x) / I.y,
            (M.z - (I.y - I.x) * w.x * w.y) / I.z);
}

// The body force plugin's force and moment on free body b, each starting at
// zero (the plugins' getForceAndMoment).
__device__ __forceinline__ void body_force(const Scene& s, int64_t b, V3& f, V3& m) {
  f = v3(0, 0, 0);
  m = v3(0, 0, 0);
  const double* p = s.bf;
  if (s.bf_kind == RK_BF_ATTRACTING_POINT) {  // BodyForce_AttractingPoint.cpp:51-59
    V3 d = v3(p[0], p[1], p[2]) - ld3(s.pos, b);
    const double l2 = norm2(d);
    if (l2 > 0.0) {
      d = d * (1.0 / sqrt(l2));
      f = (s.mass[b] * p[3]) * d;
    }
  } else if (s.bf_kind == RK_BF_PREFERRED_DIRECTION) {  // BodyForce_PreferredDirection.cpp:58-80
    V3 axisB = qrot(ldq(s.Q, b), v3(p[0], p[1], p[2]));
    normalize(axisB);
    const V3 axis = v3(p[3], p[4], p[5]);
    V3 u = cross(axis, axisB);
    normalize(u);
    const double cosa = dot(axisB, axis);
    double angle = acos(cosa);
    double sgn = -1.0;
    if (cosa < 0.0) {
      sgn = 1.0;
      angle = p[7] - angle;
    }
    m = ((p[6] * sgn) * u) * angle;
  } else if (s.bf_kind == RK_BF_VISCOUS_FLUID) {  // BodyForce_ViscousFluid.cpp:47-58
    const V3 v = ld3(s.vel, b);
    f = ((p[0] * p[1]) * s.bf_surf[b]) * v3(v.x * v.x, v.y * v.y, v.z * v.z);
  }
}

// Imposed force / moment components of a driven body (Rockable.cpp:2904-2928);
// a free body starts from the body force (Rockable.cpp:2887-2901: zero plus
// the plugin's force and moment).
__device__ __forceinline__ void init_resultant(const Scene& s, int64_t b, V3& F, V3& M) {
  F = v3(0, 0, 0);
  M = v3(0, 0, 0);
  if (b >= s.n_driven) {
    if (s.bf_kind != RK_BF_NONE) {
      V3 f, m;
      body_force(s, b, f, m);
      F = F + f;
      M = M + m;
    }
    return;
  }
  for (int k = 0; k < s.ncontrols; k++) {
    const Control c = s.controls[k];
    if (c.body != b) continue;
    switch (c.type) {
      case RK_X_FOR: F.x = c.value; break;
      case RK_Y_FOR: F.y = c.value; break;
      case RK_Z_FOR: F.z = c.value; break;
      case RK_XROT_MOM: M.x = c.value; break;
      case RK_YROT_MOM: M.y = c.value; break;
      case RK_ZROT_MOM: M.z = c.value; break;
      case RK_XYZROT_MOM: M = v3(c.vec[0], c.vec[1], c.vec[2]); break;
      default: break;
    }
  }
}

// Resultant force and moment of body b (is_heavy 0 or 1) in the serial order.
__device__ __forceinline__ void body_resultant(const Scene& s, int64_t b, V3& F, V3& M) {
  if (s.is_heavy[b]) {  // summed by k_gather_heavy, in the same order
    F = ld3(s.force, b);
    M = ld3(s.moment, b);
  } else {
    init_resultant(s, b, F, M);
    // Resultants in the serial order of the active entries (key order): the
    // j-side entries before b's own block, b's block, the remaining j-side.
    // Four positions of that sequence are loaded together, then added in
    // order (same sums, a quarter of the dependent load chains).
    const int64_t i0 = s.iofs[b], i1 = s.iofs[b + 1];
    const int64_t j0 = s.jofs[b], j1 = s.jofs[b + 1], js = s.jsplit[b];
    const int64_t nA = js - j0, nAB = nA + (i1 - i0), L = nAB + (j1 - js);
    for (int64_t p0 = 0; p0 < L; p0 += 4) {
      int64_t e[4];
      bool jside[4], on[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int64_t p = p0 + u;
        on[u] = p < L;
        jside[u] = p < nA || p >= nAB;
        e[u] = !on[u] ? 0 : (p < nA ? (int64_t)s.jlist[j0 + p] : (p < nAB ? i0 + (p - nA) : (int64_t)s.jlist[js + (p - nAB)]));
      }
      bool a[4];
#pragma unroll
      for (int u = 0; u < 4; u++) a[u] = on[u] && s.act[e[u]];
      V3 f[4], m[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (a[u]) {
          f[u] = ld3(s.cf, e[u]);
          m[u] = jside[u] ? ld3(s.cmj, e[u]) : ld3(s.cmi, e[u]);
        } else {
          f[u] = v3(0, 0, 0);
          m[u] = v3(0, 0, 0);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (!a[u]) continue;
        F = jside[u] ? F - f[u] : F + f[u];
        M = M + m[u];
      }
    }
  }
}

__device__ __forceinline__ void gather_body(const Scene& s, int64_t b, int apply_kick) {
  const bool driven = b < s.n_driven;
  if (s.is_heavy[b] == 2) {
    // a driven body whose resultant feeds no state (no force / moment
    // control): summed on demand by k_gather_heavy when downloaded
    st3(s.acc, b, v3(0, 0, 0));
    st3(s.arot, b, v3(0, 0, 0));
    return;
  }
  V3 F, M;
  body_resultant(s, b, F, M);
  const double fm = 1.0 - s.num_damp, fp = 1.0 + s.num_damp;
  const V3 vel = ld3(s.vel, b), vrot = ld3(s.vrot, b);
  const double mass = s.mass[b];
  const V3 inertia = ld3(s.inertia, b);
  const Q4 q = ldq(s.Q, b);
  if (driven) {
    V3 acc = v3(0, 0, 0), arot = v3(0, 0, 0);
    if (s.num_damp > 0.0) {  // Rockable.cpp:3814-3835
      for (int k = 0; k < s.ncontrols; k++) {
        const Control c = s.controls[k];
        if (c.body != b) continue;
        if (c.type == RK_X_FOR) F.x *= (F.x * vel.x > 0.0) ? fm : fp;
        else if (c.type == RK_Y_FOR) F.y *= (F.y * vel.y > 0.0) ? fm : fp;
        else if (c.type == RK_Z_FOR) F.z *= (F.z * vel.z > 0.0) ? fm : fp;
      }
    }
    for (int k = 0; k < s.ncontrols; k++) {  // Rockable.cpp:3448-3507
      const Control c = s.controls[k];
      if (c.body != b) continue;
      switch (c.type) {
        case RK_X_FOR: acc.x = F.x / mass; break;
        case RK_Y_FOR: acc.y = F.y / mass; break;
        case RK_Z_FOR: acc.z = F.z / mass; break;
        case RK_XROT_MOM: case RK_YROT_MOM: case RK_ZROT_MOM: case RK_XYZROT_MOM: {
          Q4 qi = qconj(q);
          V3 w;
          if (c.type == RK_XROT_MOM) w = v3(vrot.x, 0.0, 0.0);
          else if (c.type == RK_YROT_MOM) w = v3(0.0, vrot.y, 0.0);
          else if (c.type == RK_ZROT_MOM) w = v3(0.0, 0.0, vrot.z);
          else w = vrot;
          V3 om = qrot(qi, w);
          V3 Mb = qrot(qi, M);
          V3 dw = qrot(q, euler_domega(inertia, om, Mb));
          if (c.type == RK_XROT_MOM) arot.x = dw.x;
          else if (c.type == RK_YROT_MOM) arot.y = dw.y;
          else if (c.type == RK_ZROT_MOM) arot.z = dw.z;
          else arot = dw;
        } break;
        default: break;
      }
    }
    V3 v = vel, wr = vrot;
    if (apply_kick) {  // Rockable.cpp:2084-2117
      for (int k = 0; k < s.ncontrols; k++) {
        const Control c = s.controls[k];
        if (c.body != b) continue;
        switch (c.type) {
          case RK_X_FOR: v.x += s.dt_2 * acc.x; break;
          case RK_Y_FOR: v.y += s.dt_2 * acc.y; break;
          case RK_Z_FOR: v.z += s.dt_2 * acc.z; break;
          case RK_XROT_MOM: wr.x += s.dt_2 * arot.x; break;
          case RK_YROT_MOM: wr.y += s.dt_2 * arot.y; break;
          case RK_ZROT_MOM: wr.z += s.dt_2 * arot.z; break;
          case RK_XYZROT_MOM: wr = wr + s.dt_2 * arot; break;
          default: break;
        }
      }
    }
    st3(s.acc, b, acc);
    st3(s.arot, b, arot);
    st3(s.vel, b, v);
    st3(s.vrot, b, wr);
  } else {
    if (s.num_damp > 0.0) {  // Rockable.cpp:3837-3866
      double factor = (dot(F, vel) > 0.0) ? fm : fp;
      F = F * factor;
      factor = (dot(M, vrot) > 0.0) ? fm : fp;
      M = M * factor;
    }
    V3 acc = vdiv(F, mass) + v3(s.gravity[0], s.gravity[1], s.gravity[2]);
    Q4 qi = qconj(q);
    V3 om = qrot(qi, vrot);
    V3 Mb = qrot(qi, M);
    V3 arot = qrot(q, euler_domega(inertia, om, Mb));
    st3(s.acc, b, acc);
    st3(s.arot, b, arot);
    if (apply_kick) {
      st3(s.vel, b, vel + s.dt_2 * acc);
      st3(s.vrot, b, vrot + s.dt_2 * arot);
    }
  }
  st3(s.force, b, F);
  st3(s.moment, b, M);
}

}  // namespace rk
#endif  // RK_BODY_HELPERS

namespace rk {
namespace RK_BODY_NS {

#ifndef RK_BODY_GLOB_ONLY
// ----------------------------------------------------------------- K1 ----
__global__ void k_drift(Scene s) {
  if (step_halted(s)) return;
  int64_t i = s.n_driven + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.n) return;
  V3 p = ld3(s.pos, i), v = ld3(s.vel, i), a = ld3(s.acc, i);
  V3 w = ld3(s.vrot, i), al = ld3(s.arot, i);
  Q4 q = ldq(s.Q, i);
  const Q4 q0 = q;
  const V3 dx = s.dt * v + s.dt2_2 * a;
  p = p + dx;
  v = v + s.dt_2 * a;
  qaddscaled(q, qdot(q, w), s.dt);
  qaddscaled(q, qddot(q, w, al), s.dt2_2);
  qnormalize(q);
  w = w + s.dt_2 * al;
  if (s.sk_path) {
    // learned-skin path bound: |dx| plus the rotation angle of the step
    // (at most 2c(1 + c) for the chord c = |q - q0| of unit quaternions)
    // times the swing radius, rounded up
    const float cx = (float)(q.s - q0.s), cy = (float)(q.v.x - q0.v.x), cz = (float)(q.v.y - q0.v.y),
                cw = (float)(q.v.z - q0.v.z);
    const float c = sqrtf(cx * cx + cy * cy + cz * cz + cw * cw);
    const float ex = (float)dx.x, ey = (float)dx.y, ez = (float)dx.z;
    const float inc = sqrtf(ex * ex + ey * ey + ez * ez) + 2.f * c * (1.f + c) * s.sk_rsw[i];
    s.sk_path[i] += inc * (1.f + 1e-5f) + 1e-12f;
  }
  st3(s.pos, i, p);
  st3(s.vel, i, v);
  stq(s.Q, i, q);
  st3(s.vrot, i, w);
}

#endif  // RK_BODY_GLOB_ONLY

// global vertex k of body b: pos + Q (h v)
// With only_listed, the vertices of s.lv (the bodies with neighbour-list
// entries): within a step only the narrow phase reads these positions, and
// only for bodies in the list; a list update recomputes every body first
// (a partial refresh, the bodies of its pairs: `mark`).
__global__ void k_glob_vertices(Scene s, int only_listed, const uint8_t* mark) {
  if (step_halted(s)) return;
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= (only_listed ? s.nlv : s.nvert)) return;
  if (only_listed) k = s.lv[k];
  int b = s.gv_body[k];
  if (mark && !mark[b]) return;
  const int local = (int)(k - s.gv_ofs[b]);
  const V3 u = v3(s.uv64[3 * k], s.uv64[3 * k + 1], s.uv64[3 * k + 2]);  // h v, computed at upload
  V3 r = qrot(ldq(s.Q, b), u);
  V3 g = ld3(s.pos, b) + r;
  st3(s.gv, k, g);
  if (s.gvr) {
    s.gvr[3 * k] = (float)r.x;
    s.gvr[3 * k + 1] = (float)r.y;
    s.gvr[3 * k + 2] = (float)r.z;
    if (local == 0) {
      const V3 p = ld3(s.pos, b);
      s.posf[b] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)s.rad[b]);
    }
  }
}

#ifndef RK_BODY_GLOB_ONLY
__global__ void k_gather_accel(Scene s, int apply_kick) {
  if (step_halted(s)) return;
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < s.n) gather_body(s, b, apply_kick);
  // the learned skin's guard on the state this step leaves (all lanes)
  if (s.sk_out && apply_kick) skin_guard_body(s, b);
  if (s.sk_ctl) skin_batch_step_end(s);
}

#endif  // RK_BODY_GLOB_ONLY

}  // namespace RK_BODY_NS
}  // namespace rk
