// rk_fast.cu -- per-body kernels of the mixed form.
//
// The world-vertex kernel of rk_body.cuh is compiled here a second time with
// fused multiply-adds allowed (rk::fused::k_glob_vertices), and driven bodies
// go through its FP64 helpers (gather_body).  Free bodies take the kernels of
// namespace rk::mx, written for GB300's FP64 rate (about 1/77 of
// its FP32 rate, and a hardware FP64 <-> FP32 conversion costs as much as an
// FP64 add): the state (positions, velocities, quaternions, angular
// velocities) stays FP64 and is advanced by FP64 additions of increments
// computed in FP32 -- dt v + dt^2/2 a, dt/2 a, the quaternion derivative terms
// (normalised in FP64) -- and the Newton-Euler update runs in FP32 from the
// FP64 resultants (the force plus m g summed in FP64 first, so that a body at
// rest keeps a small acceleration to float precision).  Conversions use the
// integer-pipe routines of rk_bits.cuh.  An increment's relative error is
// 2^-24 (6e-8): a position moves by dt v ~ 1e-6 m per step, so its error is
// ~1e-13 m against contact overlaps of 1e-8 m and more.
#include "../../include/rk_gpu.h"
#include "rk_bits.cuh"
#include "rk_engine.cuh"
#include "rk_guard.cuh"
#define RK_BODY_NS fused
#define RK_BODY_GLOB_ONLY
#include "rk_body.cuh"

namespace rk {
namespace mx {

struct f3v {
  float x, y, z;
};
struct q4f {
  float s, x, y, z;
};
__device__ __forceinline__ f3v mk3(float x, float y, float z) {
  f3v r;
  r.x = x; r.y = y; r.z = z;
  return r;
}
__device__ __forceinline__ q4f mk4(float s, float x, float y, float z) {
  q4f r;
  r.s = s; r.x = x; r.y = y; r.z = z;
  return r;
}
__device__ __forceinline__ f3v operator+(f3v a, f3v b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3v operator*(float k, f3v a) { return mk3(k * a.x, k * a.y, k * a.z); }
__device__ __forceinline__ f3v crossf(f3v a, f3v b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dotf(f3v a, f3v b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3v cvt3(V3 a) { return mk3(d2f(a.x), d2f(a.y), d2f(a.z)); }
__device__ __forceinline__ q4f cvt4(Q4 q) { return mk4(d2f(q.s), d2f(q.v.x), d2f(q.v.y), d2f(q.v.z)); }
__device__ __forceinline__ f3v ld3f(const double* a, int64_t k) { return mk3(d2f(a[3 * k]), d2f(a[3 * k + 1]), d2f(a[3 * k + 2])); }
// FP64 a + FP32 increment d (one FP64 add per component)
__device__ __forceinline__ V3 addinc(V3 a, f3v d) { return v3(a.x + f2d(d.x), a.y + f2d(d.y), a.z + f2d(d.z)); }
__device__ __forceinline__ void st3f(double* a, int64_t k, f3v v) {
  a[3 * k] = f2d(v.x);
  a[3 * k + 1] = f2d(v.y);
  a[3 * k + 2] = f2d(v.z);
}

// u rotated by the unit quaternion q: t = 2 v x u; u + s t + v x t
__device__ __forceinline__ f3v qrotf(q4f q, f3v u) {
  const f3v v = mk3(q.x, q.y, q.z);
  const f3v t = 2.f * crossf(v, u);
  return u + q.s * t + crossf(v, t);
}
// dQ/dt = 1/2 (0, w) (x) Q and d2Q/dt2 = 1/2 (0, a) (x) Q - 1/4 |w|^2 Q
__device__ __forceinline__ q4f qdotf(q4f q, f3v w) {
  const f3v v = mk3(q.x, q.y, q.z);
  const f3v r = 0.5f * (q.s * w + crossf(w, v));
  return mk4(-0.5f * dotf(w, v), r.x, r.y, r.z);
}
__device__ __forceinline__ q4f qddotf(q4f q, f3v w, f3v a) {
  const f3v v = mk3(q.x, q.y, q.z);
  const float w2 = 0.25f * dotf(w, w);
  const f3v r = 0.5f * (q.s * a + crossf(a, v));
  return mk4(-0.5f * dotf(a, v) - w2 * q.s, r.x - w2 * v.x, r.y - w2 * v.y, r.z - w2 * v.z);
}
// Euler's equations in the principal frame (iI: the inverse moments)
__device__ __forceinline__ f3v euler_f(f3v I, f3v iI, f3v w, f3v M) {
  return mk3((M.x - (I.z - I.y) * w.y * w.z) * iI.x, (M.y - (I.x - I.z) * w.z * w.x) * iI.y,
             (M.z - (I.y - I.x) * w.x * w.y) * iI.z);
}

// First half of the velocity-Verlet step for the free bodies (the FP64 form:
// Rockable.cpp:2056-2083 through rk_body.cuh's k_drift).
__device__ __forceinline__ void drift_body(const Scene& s, int64_t i) {
  const float dt = d2f(s.dt), dt_2 = d2f(s.dt_2), dt2_2 = d2f(s.dt2_2);
  const V3 p = ld3(s.pos, i), v = ld3(s.vel, i), w = ld3(s.vrot, i);
  const Q4 q = ldq(s.Q, i);
  const f3v vf = cvt3(v), af = ld3f(s.acc, i), wf = cvt3(w), lf = ld3f(s.arot, i);
  const q4f qf = cvt4(q);
  const f3v dx = dt * vf + dt2_2 * af;
  // quaternion: the same two terms as the FP64 form (the second from the
  // quaternion after the first) as an FP32 increment dq; qd = q + dq in FP64,
  // then the normalisation as an FP64 scale: with eps = |qd|^2 - 1 (FP64),
  // qd / sqrt(1 + eps) = qd + c qd, c = -eps/2 + 3 eps^2/8 (|eps| ~ |dq|^2)
  const q4f d1 = qdotf(qf, wf);
  const q4f q1 = mk4(qf.s + dt * d1.s, qf.x + dt * d1.x, qf.y + dt * d1.y, qf.z + dt * d1.z);
  const q4f d2 = qddotf(q1, wf, lf);
  const q4f dq = mk4(dt * d1.s + dt2_2 * d2.s, dt * d1.x + dt2_2 * d2.x, dt * d1.y + dt2_2 * d2.y,
                     dt * d1.z + dt2_2 * d2.z);
  const Q4 qd = q4(q.s + f2d(dq.s), q.v.x + f2d(dq.x), q.v.y + f2d(dq.y), q.v.z + f2d(dq.z));
  double e = fma(qd.s, qd.s, -1.0);
  e = fma(qd.v.x, qd.v.x, e);
  e = fma(qd.v.y, qd.v.y, e);
  e = fma(qd.v.z, qd.v.z, e);
  const float ef = d2f(e);
  float cf = ef * (-0.5f + 0.375f * ef);
  double c = f2d(cf);
  if (!(fabsf(ef) < 1e-3f)) {
    // a rotation too large for the two-term series (a violent kick): the
    // exact normalisation, which keeps |Q| = 1 however fast the body spins
    c = 1.0 / sqrt(1.0 + e) - 1.0;
    cf = d2f(c);
  }
  if (s.sk_path) {
    // learned-skin path bound (as in rk_body.cuh's k_drift): |dx| plus the
    // rotation bound 2ch(1 + ch) of the chord ch = |q_new - q| <= |dq| + |c| |qd|
    // times the swing radius, rounded up
    const float ch = sqrtf(dq.s * dq.s + dq.x * dq.x + dq.y * dq.y + dq.z * dq.z) + fabsf(cf) * 1.001f;
    const float d = sqrtf(dotf(dx, dx)) + 2.f * ch * (1.f + ch) * s.sk_rsw[i];
    s.sk_path[i] += d * (1.f + 1e-5f) + 1e-12f;
  }
  st3(s.pos, i, addinc(p, dx));
  st3(s.vel, i, addinc(v, dt_2 * af));
  st3(s.vrot, i, addinc(w, dt_2 * lf));
  stq(s.Q, i, q4(fma(c, qd.s, qd.s), fma(c, qd.v.x, qd.v.x), fma(c, qd.v.y, qd.v.y), fma(c, qd.v.z, qd.v.z)));
}
__global__ void k_drift(Scene s) {
  if (step_halted(s)) return;
  const int64_t i = s.n_driven + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < s.n) drift_body(s, i);
}

// Resultants, Newton-Euler and the second half-kick (Rockable.cpp:3837-3866,
// 2084-2117 in the FP64 form); driven bodies take the generic FP64 path.
// Two kernels:
//   k_gather_sums    kGatherLanes lanes per body: each lane sums every
//                    kGatherLanes-th of the body's active entries (its own
//                    block, then its j-side list), the lanes' sums are
//                    reduced by shuffles in a fixed order, and the first lane
//                    stores them (6 floats per body).  A body's serial sum
//                    would be a chain of ~50 dependent loads on a dense list;
//                    the mixed form promises no serial order, and this order
//                    is the same on every run.
//   k_gather_accel   one thread per body: the resultant, Newton-Euler and
//                    the kick, whose FP64 instructions (the state is FP64)
//                    then run on full warps instead of on one lane in
//                    kGatherLanes (a warp issues an instruction once for all
//                    its lanes); every thread of both kernels has work.
// Bodies summed by k_gather_heavy (one block each) read that kernel's
// resultant.
__global__ void k_gather_sums(Scene s) {
  if (step_halted(s)) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = t / kGatherLanes;
  const int l = (int)(t % kGatherLanes);
  const bool group_sum = b < s.n && b >= s.n_driven && (s.is_heavy[b] == 0 || s.is_heavy[b] == 3);
  // FP32 sums: the contributions were computed in FP32 (the narrow phase
  // stores them widened, so the narrowing back is exact), and a sum of a
  // body's few dozen terms in FP32 errs by less than their own rounding
  // adds up to; the FP64 pipe, GB300's scarcest, stays free
  float a[6] = {0, 0, 0, 0, 0, 0};
  if (group_sum) {
    const int64_t i0 = s.iofs[b], i1 = s.iofs[b + 1], j0 = s.jofs[b], j1 = s.jofs[b + 1];
    for (int64_t e = i0 + l; e < i1; e += kGatherLanes) {
      if (!s.act[e]) continue;
      const V3 f = ld3(s.cf, e), m = ld3(s.cmi, e);
      a[0] += d2f(f.x); a[1] += d2f(f.y); a[2] += d2f(f.z);
      a[3] += d2f(m.x); a[4] += d2f(m.y); a[5] += d2f(m.z);
    }
    for (int64_t p = j0 + l; p < j1; p += kGatherLanes) {
      const int64_t e = s.jlist[p];
      if (!s.act[e]) continue;
      const V3 f = ld3(s.cf, e), m = ld3(s.cmj, e);
      a[0] -= d2f(f.x); a[1] -= d2f(f.y); a[2] -= d2f(f.z);
      a[3] += d2f(m.x); a[4] += d2f(m.y); a[5] += d2f(m.z);
    }
  }
#pragma unroll
  for (int d = 0; d < 6; d++)
    for (int o = kGatherLanes / 2; o > 0; o >>= 1) a[d] += __shfl_xor_sync(0xffffffffu, a[d], o);
  if (group_sum && l == 0)
#pragma unroll
    for (int d = 0; d < 6; d++) s.gsum[6 * b + d] = a[d];
}

__global__ void k_gather_accel(Scene s, int apply_kick) {
  if (step_halted(s)) return;
  float kin[12] = {};
  bool have = false;
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < s.n) {
    if (b < s.n_driven) {
      gather_body(s, b, apply_kick);
    } else {
      const int hv = (int)s.is_heavy[b];
      V3 F, M;
      if (hv == 0 || hv == 3) {
        const float* a = s.gsum + 6 * b;
        init_resultant(s, b, F, M);
        F = F + v3(f2d(a[0]), f2d(a[1]), f2d(a[2]));
        M = M + v3(f2d(a[3]), f2d(a[4]), f2d(a[5]));
      } else {  // summed by k_gather_heavy
        F = ld3(s.force, b);
        M = ld3(s.moment, b);
      }
      const V3 vel = ld3(s.vel, b), vrot = ld3(s.vrot, b);
      if (s.num_damp > 0.0) {  // the sign tests stay FP64: near zero they decide a factor 1 +- damp
        const double fm = 1.0 - s.num_damp, fp = 1.0 + s.num_damp;
        F = F * ((dot(F, vel) > 0.0) ? fm : fp);
        M = M * ((dot(M, vrot) > 0.0) ? fm : fp);
      }
      const double mass = s.mass[b];
      const f3v Fg = cvt3(v3(fma(mass, s.gravity[0], F.x), fma(mass, s.gravity[1], F.y), fma(mass, s.gravity[2], F.z)));
      const float4 imi = reinterpret_cast<const float4*>(s.inv_mi)[b];
      const f3v acc = imi.x * Fg;
      const q4f qf = cvt4(ldq(s.Q, b));
      const q4f qi = mk4(qf.s, -qf.x, -qf.y, -qf.z);
      const f3v wf = cvt3(vrot);
      const f3v om = qrotf(qi, wf), Mb = qrotf(qi, cvt3(M));
      const f3v arot = qrotf(qf, euler_f(ld3f(s.inertia, b), mk3(imi.y, imi.z, imi.w), om, Mb));
      st3f(s.acc, b, acc);
      st3f(s.arot, b, arot);
      f3v vf = cvt3(vel), wk = wf;
      if (apply_kick) {
        const float h = d2f(s.dt_2);
        st3(s.vel, b, addinc(vel, h * acc));
        st3(s.vrot, b, addinc(vrot, h * arot));
        vf = vf + h * acc;
        wk = wk + h * arot;
      }
      st3(s.force, b, F);
      st3(s.moment, b, M);
      const float k[12] = {vf.x, vf.y, vf.z, acc.x, acc.y, acc.z, wk.x, wk.y, wk.z, arot.x, arot.y, arot.z};
#pragma unroll
      for (int d = 0; d < 12; d++) kin[d] = k[d];
      have = true;
    }
  }
  // the learned skin's guard on the state this step leaves (every thread)
  if (s.sk_out && apply_kick) skin_guard_body_t<CvtBits>(s, b < s.n ? b : s.n, have, kin);
  if (s.sk_ctl) skin_batch_step_end(s);
}

// The mixed form's per-step body frames, in place of the FP64 world vertices:
// one thread per body computes the FP64 rotation matrix of its quaternion
// (the matrix of qrot, Particle.cpp:55-65 places the vertices with it) for
// the narrow phase's FP64 path, which places only the vertices of the
// entries it computes, and its FP32 copy; then the block's threads write the
// FP32 offsets (world vertex - centre, the FP32 test's coordinates) of all
// the block's bodies' vertices, coalesced, from the FP32 matrix.  The FP64
// work per body is one matrix instead of one rotation per vertex.
// With DRIFT (the step's launch), each free body's thread first makes its
// drift (the first half of the velocity-Verlet step, above), so that the
// frames read the state the drift just wrote: one launch and one pass over
// the bodies instead of two.
template <bool DRIFT>
__global__ void k_body_frames(Scene s) {
  if (step_halted(s)) return;
  extern __shared__ float fr[];  // [blockDim.x][10]: the FP32 matrix (and a pad)
  const int64_t b0 = blockIdx.x * (int64_t)blockDim.x;
  const int64_t b = b0 + threadIdx.x;
  if (b < s.n) {
    if (DRIFT && b >= s.n_driven) drift_body(s, b);
    const Q4 q = ldq(s.Q, b);
    const double xx = q.v.x * q.v.x, yy = q.v.y * q.v.y, zz = q.v.z * q.v.z;
    const double xy = q.v.x * q.v.y, xz = q.v.x * q.v.z, yz = q.v.y * q.v.z;
    const double sx = q.s * q.v.x, sy = q.s * q.v.y, sz = q.s * q.v.z;
    const double R[9] = {1.0 - 2.0 * (yy + zz), 2.0 * (xy - sz),       2.0 * (xz + sy),
                         2.0 * (xy + sz),       1.0 - 2.0 * (xx + zz), 2.0 * (yz - sx),
                         2.0 * (xz - sy),       2.0 * (yz + sx),       1.0 - 2.0 * (xx + yy)};
    double* out = s.rotm + 9 * b;
#pragma unroll
    for (int d = 0; d < 9; d++) {
      out[d] = R[d];
      fr[10 * threadIdx.x + d] = d2f(R[d]);
    }
    fr[10 * threadIdx.x + 9] = 0.f;
    const V3 p = ld3(s.pos, b);
    s.posf[b] = make_float4(d2f(p.x), d2f(p.y), d2f(p.z), d2f(s.rad[b]));
  }
  __syncthreads();
  const int64_t bend = min(b0 + (int64_t)blockDim.x, s.n);
  if (b0 >= bend) return;
  const int64_t k1 = s.gv_ofs[bend];
  for (int64_t k = s.gv_ofs[b0] + threadIdx.x; k < k1; k += blockDim.x) {
    const float* f = fr + 10 * (s.gv_body[k] - b0);
    const float4 u = s.uvf[k];  // h v, FP32
    const float ux = u.x, uy = u.y, uz = u.z;
    s.gvr[3 * k] = f[0] * ux + f[1] * uy + f[2] * uz;
    s.gvr[3 * k + 1] = f[3] * ux + f[4] * uy + f[5] * uz;
    s.gvr[3 * k + 2] = f[6] * ux + f[7] * uy + f[8] * uz;
  }
}

// Resultant of a body with many entries (one block per body): threads sum
// strided parts, then a tree reduction.  The order differs from the serial
// order the FP64 form keeps (rk_step.cu's k_gather_heavy); the mixed form
// does not promise bit parity.
constexpr int kHeavyThreads = 256;
__global__ void __launch_bounds__(kHeavyThreads) k_gather_heavy(Scene s, const int* list) {
  if (step_halted(s)) return;
  __shared__ double red[kHeavyThreads / 32][6];
  const int b = list[blockIdx.x];
  const int t = threadIdx.x;
  double a[6] = {0, 0, 0, 0, 0, 0};
  const int64_t i0 = s.iofs[b], i1 = s.iofs[b + 1], j0 = s.jofs[b], j1 = s.jofs[b + 1];
  for (int64_t e = i0 + t; e < i1; e += kHeavyThreads) {
    if (!s.act[e]) continue;
    const V3 f = ld3(s.cf, e), m = ld3(s.cmi, e);
    a[0] += f.x; a[1] += f.y; a[2] += f.z;
    a[3] += m.x; a[4] += m.y; a[5] += m.z;
  }
  for (int64_t p = j0 + t; p < j1; p += kHeavyThreads) {
    const int64_t e = s.jlist[p];
    if (!s.act[e]) continue;
    const V3 f = ld3(s.cf, e), m = ld3(s.cmj, e);
    a[0] -= f.x; a[1] -= f.y; a[2] -= f.z;
    a[3] += m.x; a[4] += m.y; a[5] += m.z;
  }
#pragma unroll
  for (int d = 0; d < 6; d++)
    for (int o = 16; o > 0; o >>= 1) a[d] += __shfl_down_sync(0xffffffffu, a[d], o);
  if ((t & 31) == 0)
    for (int d = 0; d < 6; d++) red[t >> 5][d] = a[d];
  __syncthreads();
  if (t == 0) {
    V3 F, M;
    init_resultant(s, b, F, M);
    for (int w = 0; w < kHeavyThreads / 32; w++) {
      F = F + v3(red[w][0], red[w][1], red[w][2]);
      M = M + v3(red[w][3], red[w][4], red[w][5]);
    }
    st3(s.force, b, F);
    st3(s.moment, b, M);
  }
}

}  // namespace mx

int launch_body_frames(const Scene& s, unsigned blocks, int threads, int with_drift, cudaStream_t st) {
  if (with_drift) mx::k_body_frames<true><<<blocks, threads, 10 * sizeof(float) * threads, st>>>(s);
  else mx::k_body_frames<false><<<blocks, threads, 10 * sizeof(float) * threads, st>>>(s);
  return 1;
}
int launch_fused_glob(const Scene& s, unsigned blocks, int threads, int only_listed, const uint8_t* mark,
                      cudaStream_t st) {
  fused::k_glob_vertices<<<blocks, threads, 0, st>>>(s, only_listed, mark);
  return 1;
}
int launch_fused_gather(const Scene& s, unsigned blocks, int threads, int apply_kick, cudaStream_t st) {
  mx::k_gather_sums<<<(unsigned)((s.n * kGatherLanes + 255) / 256), 256, 0, st>>>(s);
  mx::k_gather_accel<<<blocks, threads, 0, st>>>(s, apply_kick);
  return 2;
}
int launch_fused_heavy(const Scene& s, const int* list, int count, cudaStream_t st) {
  mx::k_gather_heavy<<<count, mx::kHeavyThreads, 0, st>>>(s, list);
  return 1;
}
cudaError_t fused_attributes(int which, cudaFuncAttributes* a) {
  if (which == 1) return cudaFuncGetAttributes(a, mx::k_gather_accel);
  if (which == 2) return cudaFuncGetAttributes(a, mx::k_body_frames<true>);
  return cudaFuncGetAttributes(a, mx::k_drift);
}

}  // namespace rk
