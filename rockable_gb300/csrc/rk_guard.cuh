// rk_guard.cuh -- per-body evaluation of the learned skin's exact guard
// (see rk_skin.cu for the bounds), shared by the resultant kernel, which
// runs it at the end of every step of the skin mode.
#pragma once
#include "rk_bits.cuh"
#include "rk_engine.cuh"

namespace rk {

// Upper bound of the rotation angle between two unit quaternions: with c
// the shorter of the chords |q - q0| and |q + q0|, the angle is
// 4 asin(c / 2) <= 2 c (1 + c).
__device__ __forceinline__ double quat_chord(const double* q, const double* q0) {
  double m2 = 0.0, p2 = 0.0;
  for (int d = 0; d < 4; d++) {
    const double m = q[d] - q0[d], p = q[d] + q0[d];
    m2 += m * m;
    p2 += p * p;
  }
  return sqrt(fmin(m2, p2));
}
__device__ __forceinline__ double rot_bound(const double* q, const double* q0) {
  const double c = quat_chord(q, q0);
  return 2.0 * c * (1.0 + c);
}

// FP64 -> float conversion of the guard: the hardware one (FP64 form) or
// the integer-pipe one (mixed form); the margins below cover either.
struct CvtHw {
  __device__ static float f(double x) { return (float)x; }
};
struct CvtBits {
  __device__ static float f(double x) { return d2f(x); }
};

// Guard of body b after a step, evaluated by the thread that finished the
// body's update (the resultant kernel); every thread of the block must call
// it (block reduction, blocks of at most 512 threads).  sk_out (zeroed before the step): [0] max delta,
// [1] max |v| of the free bodies, [2] max g (float bits, atomicMax),
// [3] number of flagged bodies (g >= flag_at), [4..5] unused,
// [6] max delta and [7] max g bounded for the state after the NEXT step:
// the next drift's motion is bounded from the velocities and accelerations
// this step leaves (free bodies); driven bodies do not move between steps
// when no control drives them, which is the only case the host uses the
// bound for.
// With have_kin, kin holds the body's velocity, acceleration, angular
// velocity and angular acceleration after the step as floats (12 values,
// the caller's registers); otherwise they are read back and converted.
template <class C>
__device__ __forceinline__ void skin_guard_body_t(const Scene& s, int64_t b, bool have_kin, const float* kin) {
  const double* ref_pos = s.sk_ref_pos;
  const double* ref_q = s.sk_ref_q;
  const float* rsw = s.sk_rsw;
  float* maxd = s.sk_maxd;
  const float* path = s.sk_path;
  const float flag_at = s.sk_flag_at;
  uint8_t* flag = s.sk_flag;
  unsigned int* out = s.sk_out;
  float dmax = 0.f, vmax = 0.f, gmax = 0.f, pdmax = 0.f, pgmax = 0.f;
  unsigned nflag = 0;
  if (b < s.n) {
    // differences in FP64, the rest in float rounded up (relative 1e-5 covers
    // the float rounding of the norms, 1e-12 m the conversions)
    const float dx = C::f(s.pos[3 * b] - ref_pos[3 * b]), dy = C::f(s.pos[3 * b + 1] - ref_pos[3 * b + 1]),
                dz = C::f(s.pos[3 * b + 2] - ref_pos[3 * b + 2]);
    float m2 = 0.f, p2 = 0.f;
    for (int d = 0; d < 4; d++) {
      const float m = C::f(s.Q[4 * b + d] - ref_q[4 * b + d]), p = C::f(s.Q[4 * b + d] + ref_q[4 * b + d]);
      m2 += m * m;
      p2 += p * p;
    }
    const float chord = sqrtf(fminf(m2, p2)) * (1.f + 1e-5f);
    dmax = (sqrtf(dx * dx + dy * dy + dz * dz) + 2.f * chord * (1.f + chord) * rsw[b]) * (1.f + 1e-5f) + 1e-12f;
    const float md = fmaxf(maxd[b], dmax);
    maxd[b] = md;
    // driven bodies are moved by their controls, not by the drift: no path
    const float pth = b >= s.n_driven ? path[b] : INFINITY;
    gmax = fminf(pth, 2.f * md);
    const bool f = gmax >= flag_at;
    flag[b] = f ? 1 : 0;
    nflag = f ? 1u : 0u;
    if (b >= s.n_driven) {
      float k[12];
      if (have_kin) {
#pragma unroll
        for (int d = 0; d < 12; d++) k[d] = kin[d];
      } else {
        for (int d = 0; d < 3; d++) {
          k[d] = C::f(s.vel[3 * b + d]);
          k[3 + d] = C::f(s.acc[3 * b + d]);
          k[6 + d] = C::f(s.vrot[3 * b + d]);
          k[9 + d] = C::f(s.arot[3 * b + d]);
        }
      }
      const float vx = k[0], vy = k[1], vz = k[2];
      vmax = sqrtf(vx * vx + vy * vy + vz * vz);
      // bound of the next drift: |dt v + dt^2/2 a| and a rotation of at most
      // |w| dt + |alpha| dt^2/2 (the normalised quaternion update, 1 % margin
      // for its second-order terms); a step of angle t moves the chord c by at
      // most t/2, so 2c(1 + c) grows by at most t (1 + 2c + t/2).  Only decides
      // when the exact values must be read, so a bound is enough.
      const float ax = k[3], ay = k[4], az = k[5];
      const float wx = k[6], wy = k[7], wz = k[8];
      const float lx = k[9], ly = k[10], lz = k[11];
      const float dt = (float)s.dt, dt2 = (float)s.dt2_2;
      const float dxb = dt * vmax + dt2 * sqrtf(ax * ax + ay * ay + az * az);
      const float thb = dt * sqrtf(wx * wx + wy * wy + wz * wz) + dt2 * sqrtf(lx * lx + ly * ly + lz * lz);
      const float inc = 1.01f * (dxb + thb * rsw[b] * (1.f + 2.f * chord + thb)) + 1e-12f;
      pdmax = dmax + inc;
      pgmax = fminf(path[b] + inc, 2.f * fmaxf(md, pdmax));
    } else {
      pdmax = dmax;
      pgmax = gmax;
    }
  }
  // warp, then block reduction through shared memory: one atomic per block
  // and quantity (the block size is at most 512 threads)
  for (int o = 16; o > 0; o >>= 1) {
    dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    gmax = fmaxf(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
    pdmax = fmaxf(pdmax, __shfl_xor_sync(0xffffffffu, pdmax, o));
    pgmax = fmaxf(pgmax, __shfl_xor_sync(0xffffffffu, pgmax, o));
    nflag += __shfl_xor_sync(0xffffffffu, nflag, o);
  }
  __shared__ float red[16][5];
  __shared__ unsigned redn[16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    red[warp][0] = dmax;
    red[warp][1] = vmax;
    red[warp][2] = gmax;
    red[warp][3] = pdmax;
    red[warp][4] = pgmax;
    redn[warp] = nflag;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; w++) {
      dmax = fmaxf(dmax, red[w][0]);
      vmax = fmaxf(vmax, red[w][1]);
      gmax = fmaxf(gmax, red[w][2]);
      pdmax = fmaxf(pdmax, red[w][3]);
      pgmax = fmaxf(pgmax, red[w][4]);
      nflag += redn[w];
    }
    atomicMax(&out[0], __float_as_uint(dmax));
    atomicMax(&out[1], __float_as_uint(vmax));
    atomicMax(&out[2], __float_as_uint(gmax));
    if (nflag) atomicAdd(&out[3], nflag);
    atomicMax(&out[6], __float_as_uint(pdmax));
    atomicMax(&out[7], __float_as_uint(pgmax));
  }
}

// End of a batched skin step (control block sk_ctl, see rk_skin.cu): every
// block of the resultant kernel calls it after its guard atomics (all its
// threads); the last block to arrive reads the step's guard words, counts the
// step and halts the batch when the host has to act -- a refresh is due or
// the batch's step budget is spent -- and otherwise zeroes the counters for
// the next step (the guard words and the active-contact count).
__device__ __forceinline__ void skin_batch_step_end(const Scene& s) {
  __shared__ int last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&s.sk_ctl[7], 1u) == gridDim.x - 1 ? 1 : 0;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile unsigned int* ctl = s.sk_ctl;
  volatile unsigned int* out = s.sk_out;
  const unsigned ex = ctl[1] + 1u, since = ctl[2] + 1u;
  ctl[1] = ex;
  ctl[2] = since;
  ctl[7] = 0u;
  unsigned int g[8];
  for (int d = 0; d < 8; d++) {
    g[d] = out[d];
    ctl[8 + d] = g[d];
  }
  const float crit = __uint_as_float(ctl[6] ? g[2] : g[0]);
  if (crit >= __uint_as_float(ctl[5]) || since >= ctl[4] || ex >= ctl[3]) {
    ctl[0] = 1u;
  } else {
    for (int d = 0; d < 8; d++) out[d] = 0u;
    s.flags[FLAG_NACTIVE] = 0ull;
  }
}

__device__ __forceinline__ void skin_guard_body(const Scene& s, int64_t b) {
  const float none[12] = {};
  skin_guard_body_t<CvtHw>(s, b, false, none);
}

}  // namespace rk
