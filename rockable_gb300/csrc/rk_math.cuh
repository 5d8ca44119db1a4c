// rk_math.cuh -- FP64 vector / quaternion kernels of the step engine.
//
// The operation order of every function is fixed: the FP64 form is compiled
// with --fmad=false so that each result is bit-identical to Rockable's CPU
// arithmetic (the toofus vec3 / quat kernels used by src/Core/Particle.cpp,
// Interaction.cpp and Rockable.cpp).  Do not "simplify" an expression here
// without re-running the bit-parity tests.
#pragma once
#include <cuda_runtime.h>

namespace rk {

struct V3 {
  double x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(double x, double y, double z) {
  V3 r;
  r.x = x; r.y = y; r.z = z;
  return r;
}
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ double norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// vector / scalar is a multiplication by the inverse (toofus vec3::operator/)
__host__ __device__ __forceinline__ V3 vdiv(V3 a, double s) {
  double inv = 1.0 / s;
  return v3(a.x * inv, a.y * inv, a.z * inv);
}
// normalise in place, return the norm before normalisation
__host__ __device__ __forceinline__ double normalize(V3& a) {
  double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  if (n > 0.0) {
    double inv = 1.0 / n;
    a.x *= inv; a.y *= inv; a.z *= inv;
  }
  return n;
}

struct Q4 {
  double s;
  V3 v;
};
__host__ __device__ __forceinline__ Q4 q4(double s, double x, double y, double z) {
  Q4 q;
  q.s = s; q.v = v3(x, y, z);
  return q;
}
__host__ __device__ __forceinline__ Q4 qconj(Q4 q) {
  Q4 r;
  r.s = q.s; r.v = -q.v;
  return r;
}
// rotate u from the body frame to the global frame: t = 2 v x u; u + s t + v x t
__host__ __device__ __forceinline__ V3 qrot(Q4 q, V3 u) {
  V3 t = 2.0 * cross(q.v, u);
  return u + q.s * t + cross(q.v, t);
}
// dQ/dt = 1/2 (0, w) (x) Q for a global-frame angular velocity w
__host__ __device__ __forceinline__ Q4 qdot(Q4 q, V3 w) {
  Q4 r;
  r.s = -0.5 * dot(w, q.v);
  r.v = 0.5 * (q.s * w + cross(w, q.v));
  return r;
}
// d2Q/dt2 = 1/2 (0, a) (x) Q - 1/4 |w|^2 Q
__host__ __device__ __forceinline__ Q4 qddot(Q4 q, V3 w, V3 a) {
  double w2 = dot(w, w);
  Q4 r;
  r.s = -0.5 * dot(a, q.v) - 0.25 * w2 * q.s;
  r.v = 0.5 * (q.s * a + cross(a, q.v)) - 0.25 * w2 * q.v;
  return r;
}
__host__ __device__ __forceinline__ void qaddscaled(Q4& a, Q4 b, double f) {  // a += (b *= f)
  b.s *= f;
  b.v = v3(b.v.x * f, b.v.y * f, b.v.z * f);
  a.s += b.s;
  a.v = a.v + b.v;
}
__host__ __device__ __forceinline__ void qnormalize(Q4& q) {
  double n = sqrt(dot(q.v, q.v) + q.s * q.s);
  if (n > 0.0) {
    double f = 1.0 / n;
    q.s *= f;
    q.v = v3(q.v.x * f, q.v.y * f, q.v.z * f);
  }
}
__host__ __device__ __forceinline__ double qangle(Q4 q) {
  double s = q.s;
  if (s > 1.0) s = 1.0;
  if (s < -1.0) s = -1.0;
  return 2.0 * acos(s);
}

// Oriented box: center, three unit axes, half extents.
struct Obb {
  V3 c, e0, e1, e2, ext;
};

__host__ __device__ __forceinline__ double comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// Separating-axis test of two oriented boxes (15 axes), same operation order
// as the oracle's restatement of toofus OBB::intersect.
__host__ __device__ inline bool obb_intersect(const Obb& a, const Obb& b) {
  const double eps = 1e-12;
  V3 ae[3] = {a.e0, a.e1, a.e2};
  V3 be[3] = {b.e0, b.e1, b.e2};
  double R[3][3], AR[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[i][j] = dot(ae[i], be[j]);
      AR[i][j] = fabs(R[i][j]) + eps;
    }
  V3 d = b.c - a.c;
  double t[3] = {dot(d, ae[0]), dot(d, ae[1]), dot(d, ae[2])};
  double aext[3] = {a.ext.x, a.ext.y, a.ext.z};
  double bext[3] = {b.ext.x, b.ext.y, b.ext.z};
  double ra, rb;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    ra = aext[i];
    rb = bext[0] * AR[i][0] + bext[1] * AR[i][1] + bext[2] * AR[i][2];
    if (fabs(t[i]) > ra + rb) return false;
  }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    ra = aext[0] * AR[0][j] + aext[1] * AR[1][j] + aext[2] * AR[2][j];
    rb = bext[j];
    if (fabs(t[0] * R[0][j] + t[1] * R[1][j] + t[2] * R[2][j]) > ra + rb) return false;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      ra = aext[i1] * AR[i2][j] + aext[i2] * AR[i1][j];
      rb = bext[j1] * AR[i][j2] + bext[j2] * AR[i][j1];
      double tt = t[i2] * R[i1][j] - t[i1] * R[i2][j];
      if (fabs(tt) > ra + rb) return false;
    }
  }
  return true;
}

}  // namespace rk
