// rk_extract.cuh -- Rockable's DataExtractors (src/DataExtractors/*.cpp) as
// device reductions over the SoA state, for rk_extract_* in rk_api.cu: the
// host gets a few numbers instead of downloading the bodies and the list at
// every record.  Compiled with rk_api.cu (FP64 without fused multiply-adds),
// so a vertex is placed with the same operations as the host's
// Particle::GlobVertex and the extremes are bit-identical to a serial pass;
// sums are tree sums in a fixed order (the same numbers on every run,
// within the rounding of a different order from the serial sum).
#pragma once
#include <cstring>
#include "rk_engine.cuh"
#include "rk_math.cuh"

namespace rk {

constexpr int kExtBlocks = 256, kExtThreads = 256;

// FP64 <-> unsigned 64-bit with the same order (atomic min / max of doubles)
__device__ __forceinline__ unsigned long long ext_ord(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double ext_unord(unsigned long long o) {
  const unsigned long long u = (o & 0x8000000000000000ull) ? (o & 0x7fffffffffffffffull) : ~o;
  double d;
  memcpy(&d, &u, 8);
  return d;
}

// block sum of v in a fixed order (thread 0 returns it)
__device__ __forceinline__ double ext_block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sh[k];
  __syncthreads();
  return t;
}

// MeanVelocity (DataExtractor_MeanVelocity.cpp:24-32): per block, the sum of
// |v| of its bodies (grid-stride); part[blockIdx.x]
__global__ void __launch_bounds__(kExtThreads) k_ext_speed(Scene s, double* part) {
  __shared__ double sh[kExtThreads / 32];
  double a = 0.0;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < s.n; b += (int64_t)gridDim.x * blockDim.x) {
    const double x = s.vel[3 * b], y = s.vel[3 * b + 1], z = s.vel[3 * b + 2];
    a += sqrt(x * x + y * y + z * z);
  }
  const double t = ext_block_sum(a, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// dnStat (DataExtractor_dnStat.cpp:35-68) over the active entries (dn < 0 or
// bonded, from the stored history: the reference's activeInteractions,
// Rockable.cpp:3005-3029, in the same order): per block,
// [0] sum dn, [1] sum of the negative ones, [2] their count, [3] sum of the
// others, [4] their count, [5] the smallest dn, [6] its entry (the first of
// equal ones, as the serial strict comparison keeps), [7] the largest dn
__device__ __forceinline__ bool ext_before(double a, int64_t ia, double b, int64_t ib) {
  return a < b || (!(b < a) && ia < ib);
}
__global__ void __launch_bounds__(kExtThreads) k_ext_dn(Scene s, double* part) {
  __shared__ double sh[kExtThreads / 32];
  __shared__ double smin[kExtThreads], smax[kExtThreads];
  __shared__ int64_t sidx[kExtThreads];
  double sum = 0.0, sneg = 0.0, nneg = 0.0, spos = 0.0, npos = 0.0, mn = 1e20, mx = -1e20;
  int64_t imn = INT64_MAX;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < s.ne; e += (int64_t)gridDim.x * blockDim.x) {
    const double dn = s.dn[e];
    if (!(dn < 0.0 || s.bond[e] >= 0)) continue;
    sum += dn;
    if (dn < 0.0) {
      sneg += dn;
      nneg += 1.0;
    } else {
      spos += dn;
      npos += 1.0;
    }
    if (ext_before(dn, e, mn, imn) && dn < 1e20) {
      mn = dn;
      imn = e;
    }
    if (dn > mx) mx = dn;
  }
  const double t0 = ext_block_sum(sum, sh), t1 = ext_block_sum(sneg, sh), t2 = ext_block_sum(nneg, sh);
  const double t3 = ext_block_sum(spos, sh), t4 = ext_block_sum(npos, sh);
  smin[threadIdx.x] = mn;
  sidx[threadIdx.x] = imn;
  smax[threadIdx.x] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)blockDim.x; k++) {
      if (ext_before(smin[k], sidx[k], mn, imn) && sidx[k] != INT64_MAX) {
        mn = smin[k];
        imn = sidx[k];
      }
      if (smax[k] > mx) mx = smax[k];
    }
    double* o = part + 8 * blockIdx.x;
    o[0] = t0; o[1] = t1; o[2] = t2; o[3] = t3; o[4] = t4;
    o[5] = mn;
    o[6] = (double)imn;  // exact up to 2^53 entries; INT64_MAX: none
    o[7] = mx;
  }
}

// ClusterAABB (DataExtractor_ClusterAABB.cpp:31-65): the box of the vertices
// of the bodies of one cluster, each enlarged by its body's Minkowski radius;
// ext[0..2] ordered minima, ext[3..5] ordered maxima, ext[6] set when any
__global__ void k_ext_cluster_box(Scene s, int cluster, unsigned long long* ext) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= s.nvert) return;
  const int b = s.gv_body[k];
  if (s.cluster[b] != cluster) return;
  // Particle::GlobVertex: pos + Q (h v), the operations of qrot
  const V3 u = v3(s.uv64[3 * k], s.uv64[3 * k + 1], s.uv64[3 * k + 2]);
  const Q4 q = q4(s.Q[4 * b], s.Q[4 * b + 1], s.Q[4 * b + 2], s.Q[4 * b + 3]);
  const V3 g = v3(s.pos[3 * b], s.pos[3 * b + 1], s.pos[3 * b + 2]) + qrot(q, u);
  const double r = s.rad[b];
  const double lo[3] = {g.x - r, g.y - r, g.z - r}, hi[3] = {g.x + r, g.y + r, g.z + r};
  for (int d = 0; d < 3; d++) {
    atomicMin(ext + d, ext_ord(lo[d]));
    atomicMax(ext + 3 + d, ext_ord(hi[d]));
  }
  atomicMax(ext + 6, 1ull);
}

// DuoBalance (DataExtractor_DuoBalance.cpp:31-85): sub-contacts of the pair
// (i, j), either way round, with dn < 0, by type
__global__ void k_ext_duo(Scene s, int bi, int bj, unsigned long long* cnt) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.ne) return;
  const int i = s.ei[e], j = s.ej[e];
  if (!((i == bi && j == bj) || (i == bj && j == bi))) return;
  if (!(s.dn[e] < 0.0)) return;
  atomicAdd(cnt + tsub_type(s.etsub[e]), 1ull);
}

// TrackBody (DataExtractor_TrackBody.cpp:67-80): one body's pos, vel, acc,
// Q, vrot, arot, force, moment (25 numbers)
__global__ void k_ext_body(Scene s, int64_t b, double* out) {
  const int t = threadIdx.x;
  if (t >= 25) return;
  const double* src[8] = {s.pos, s.vel, s.acc, s.Q, s.vrot, s.arot, s.force, s.moment};
  const int cnt[8] = {3, 3, 3, 4, 3, 3, 3, 3};
  int f = 0, k = t;
  while (k >= cnt[f]) k -= cnt[f++];
  out[t] = src[f][cnt[f] * b + k];
}

}  // namespace rk
