// rk_nl.cu -- neighbour-list rebuild on the GPU.
//
// Semantics follow Rockable's UpdateNL_bruteForce (Rockable.cpp:1614-1662)
// with AddOrRemoveInteractions_bruteForce (Rockable.cpp:1309-1432):
//   * a body pair (i < j, not both driven, no unbroken interface) is
//     "visited" when their OBBs enlarged by DVerlet/2 intersect;
//   * in a visited pair every sub-contact candidate is tested, except the
//     vertex-owned ones whose vertex cube fails the OBB cull; a tested
//     candidate that is NEAR is kept (history carried) or inserted (fresh
//     history), a tested candidate that is not NEAR is removed;
//   * entries of pairs that are not visited, and untested candidates, are
//     kept untouched.
// UpdateNL_linkCells visits exactly the same pairs when its cells contain the
// enlarged boxes, so both options map onto this exact pair predicate.
//
// Pipeline (all on the context stream, a few host reads of counts):
//   body_obb -> pairs (all-pairs AABB filter or uniform grid, then the FP64
//   SAT) -> half-pairs (both directions, radix-sorted) -> candidates (one
//   warp per half-pair: cull mask, NEAR keys appended) -> key sort -> old-entry
//   classification and order-preserving compaction -> merge by key ->
//   history carry -> i-side offsets and j-side list.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "rk_bits.cuh"
#include "rk_ctx.cuh"

namespace rk {

__device__ __forceinline__ V3 g3(const double* a, int64_t k) { return v3(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }

__device__ __forceinline__ Obb load_obb(const double* o) {
  Obb b;
  b.c = v3(o[0], o[1], o[2]);
  b.e0 = v3(o[3], o[4], o[5]);
  b.e1 = v3(o[6], o[7], o[8]);
  b.e2 = v3(o[9], o[10], o[11]);
  b.ext = v3(o[12], o[13], o[14]);
  return b;
}
__device__ __forceinline__ void enlarge(Obb& b, double d) {
  b.ext.x += d;
  b.ext.y += d;
  b.ext.z += d;
}

// Particle::updateObb (Particle.cpp:78-86) and the AABB of the box enlarged
// by DVerlet/2, rounded outward to float for the pair filter.
__global__ void k_body_obb(Scene s) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= s.n) return;
  const double* so = s.sobb + 15 * s.shape[b];
  Obb o = load_obb(so);
  Q4 q = q4(s.Q[4 * b], s.Q[4 * b + 1], s.Q[4 * b + 2], s.Q[4 * b + 3]);
  o.e0 = qrot(q, o.e0);
  o.e1 = qrot(q, o.e1);
  o.e2 = qrot(q, o.e2);
  o.c = qrot(q, o.c);
  double h = s.hom[b];
  o.ext = h * o.ext;
  o.c = h * o.c;
  o.c = o.c + v3(s.pos[3 * b], s.pos[3 * b + 1], s.pos[3 * b + 2]);
  double* out = s.bobb + 15 * b;
  out[0] = o.c.x; out[1] = o.c.y; out[2] = o.c.z;
  out[3] = o.e0.x; out[4] = o.e0.y; out[5] = o.e0.z;
  out[6] = o.e1.x; out[7] = o.e1.y; out[8] = o.e1.z;
  out[9] = o.e2.x; out[10] = o.e2.y; out[11] = o.e2.z;
  out[12] = o.ext.x; out[13] = o.ext.y; out[14] = o.ext.z;
  float* of = s.bobbf + 15 * b;  // float copy for the pair test's pre-classification
  for (int q = 0; q < 15; q++) of[q] = d2f(out[q]);
  {  // the vertex box placed, in float (the pruning tests carry the rounding margin)
    const double* sb = s.sbox + 6 * s.shape[b];
    const V3 bc = v3(s.pos[3 * b], s.pos[3 * b + 1], s.pos[3 * b + 2]) + qrot(q, h * v3(sb[0], sb[1], sb[2]));
    const V3 ax[3] = {qrot(q, v3(1, 0, 0)), qrot(q, v3(0, 1, 0)), qrot(q, v3(0, 0, 1))};
    float* bx = s.bbox + 15 * b;
    bx[0] = d2f(bc.x); bx[1] = d2f(bc.y); bx[2] = d2f(bc.z);
    for (int k = 0; k < 3; k++) {
      bx[3 + 3 * k] = d2f(ax[k].x);
      bx[4 + 3 * k] = d2f(ax[k].y);
      bx[5 + 3 * k] = d2f(ax[k].z);
      bx[12 + k] = d2f(h * sb[3 + k]);
    }
  }
  const double d = 0.5 * s.DVerlet;
  const double ex = o.ext.x + d, ey = o.ext.y + d, ez = o.ext.z + d;
  const double hw[3] = {ex * fabs(o.e0.x) + ey * fabs(o.e1.x) + ez * fabs(o.e2.x),
                        ex * fabs(o.e0.y) + ey * fabs(o.e1.y) + ez * fabs(o.e2.y),
                        ex * fabs(o.e0.z) + ey * fabs(o.e1.z) + ez * fabs(o.e2.z)};
  const double c[3] = {o.c.x, o.c.y, o.c.z};
  if (!isfinite(c[0] + c[1] + c[2] + hw[0] + hw[1] + hw[2]))
    atomicMax(s.flags + FLAG_NONFINITE, (unsigned long long)b + 1ull);
  float* bb = s.baabb + 6 * b;
  for (int k = 0; k < 3; k++) {
    double m = 1e-6 * (hw[k] + fabs(c[k])) + 1e-12;  // slack covering the SAT epsilon
    bb[k] = __double2float_rd(c[k] - hw[k] - m);
    bb[3 + k] = __double2float_ru(c[k] + hw[k] + m);
  }
}

// Bounding spheres of every sub-element (vertices, edges, faces) in world
// coordinates, as floats with the radius rounded up: the conservative filter
// in front of the FP64 NEAR predicates.  A vertex sphere's centre is its FP64
// world vertex rounded to nearest (the float NEAR classification relies on
// that); everything else comes from the FP32 vertex offsets gvr (world vertex
// - body centre, written with the world vertices; relative error below 4e-7),
// so that the kernel issues no FP64 arithmetic: GB300's FP64 pipe made it
// FP64-bound.  Conversions use the integer-pipe routines of rk_bits.cuh.
__global__ void k_spheres(Scene s, int64_t nsph, const uint8_t* mark) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nsph) return;
  const int b = s.sph_body[k];
  if (mark && !mark[b]) return;
  const int local = (int)(k - s.sph_ofs[b]);
  const int sh = s.shape[b];
  const int64_t g0 = s.gv_ofs[b];
  const double* g = s.gv + 3 * g0;
  const float* gr = s.gvr + 3 * g0;
  const int nv = s.vert_ofs[sh + 1] - s.vert_ofs[sh];
  const int e0 = s.edge_ofs[sh], ne = s.edge_ofs[sh + 1] - e0;
  const int f0 = s.face_ofs[sh];
  if (local < nv) {  // vertex: its position; the body bound is the largest vertex distance
    const int v = local;
    s.sph[k] = make_float4(d2f(g[3 * v]), d2f(g[3 * v + 1]), d2f(g[3 * v + 2]), 0.f);
    const float dx = gr[3 * v], dy = gr[3 * v + 1], dz = gr[3 * v + 2];
    // rounded up: the offsets' error and a few float roundings, covered by 2e-6
    const float d = sqrtf(dx * dx + dy * dy + dz * dz) * (1.f + 2e-6f) + 1e-30f;
    atomicMax(reinterpret_cast<unsigned int*>(s.bnd) + b, __float_as_uint(d));  // non-negative floats order as their bits
  } else {
    // Edge (midpoint, half length) or face (centroid, largest vertex
    // distance), from the FP32 offsets relative to the element's first
    // vertex; the float centre is off the exact one by rounding, so the
    // radius is the largest distance from that float centre, scaled up by
    // 1e-5 and padded by 1e-6 of the coordinate magnitude: the sphere still
    // holds the element.
    const bool edge = local < nv + ne;
    const int* vl;
    int cnt;
    if (edge) {
      vl = s.edges + 2 * (e0 + (local - nv));
      cnt = 2;
    } else {
      const int f = local - nv - ne;
      const int v0 = s.face_vofs[f0 + f];
      vl = s.face_verts + v0;
      cnt = s.face_vofs[f0 + f + 1] - v0;
    }
    const float ox = gr[3 * vl[0]], oy = gr[3 * vl[0] + 1], oz = gr[3 * vl[0] + 2];
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int q = 1; q < cnt; q++) {
      cx += gr[3 * vl[q]] - ox;
      cy += gr[3 * vl[q] + 1] - oy;
      cz += gr[3 * vl[q] + 2] - oz;
    }
    const float inv = 1.f / (float)cnt;
    cx *= inv;
    cy *= inv;
    cz *= inv;
    float r2 = cx * cx + cy * cy + cz * cz;  // vertex 0
    for (int q = 1; q < cnt; q++) {
      const float ex = (gr[3 * vl[q]] - ox) - cx, ey = (gr[3 * vl[q] + 1] - oy) - cy, ez = (gr[3 * vl[q] + 2] - oz) - cz;
      r2 = fmaxf(r2, ex * ex + ey * ey + ez * ez);
    }
    const float px = d2f(g[3 * vl[0]]) + cx, py = d2f(g[3 * vl[0] + 1]) + cy, pz = d2f(g[3 * vl[0] + 2]) + cz;
    const float mag = fmaxf(fmaxf(fabsf(px), fabsf(py)), fabsf(pz));
    s.sph[k] = make_float4(px, py, pz, sqrtf(r2) * (1.f + 1e-5f) + 1e-6f * mag + 1e-9f);
  }
}

// bodies whose resultant is summed by a warp (see k_gather_heavy): in the
// step when the resultant is used, on demand otherwise; and the vertices of
// the bodies with entries (the only ones the step's narrow phase reads), in
// per-body runs whose order between bodies does not matter
__global__ void k_heavy(Scene s, unsigned long long* count) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= s.n) return;
  int64_t c = (s.iofs[b + 1] - s.iofs[b]) + (s.jofs[b + 1] - s.jofs[b]);
  if (c > 0 && !s.fast_body) {  // (the mixed form's step places its vertices from the body frames)
    const int64_t v0 = s.gv_ofs[b], nv = s.gv_ofs[b + 1] - v0;
    const int64_t at = (int64_t)atomicAdd(&count[3], (unsigned long long)nv);
    for (int64_t l = 0; l < nv; l++) s.lv[at + l] = (int)(v0 + l);
  }
  {  // split of the j-side list around b's own block (entry indices ascend in it)
    const int64_t i0 = s.iofs[b];
    int64_t lo = s.jofs[b], hi = s.jofs[b + 1];
    while (lo < hi) {
      const int64_t m = (lo + hi) >> 1;
      if (s.jlist[m] < i0) lo = m + 1;
      else hi = m;
    }
    s.jsplit[b] = lo;
  }
  bool h = c > kHeavy;
  uint8_t kind = 0;
  if (h && s.needres[b] && s.fast_body && c <= kHeavyWarp) {
    kind = 3;  // the mixed form's resultant sums kernel sums it with its 8 lanes, like any body
  } else if (h && s.needres[b]) {
    kind = 1;
    s.heavy[atomicAdd(&count[0], 1ull)] = (int)b;
  } else if (h) {
    kind = 2;
    s.heavy_lazy[atomicAdd(&count[1], 1ull)] = (int)b;
  }
  s.is_heavy[b] = kind;
}

__device__ __forceinline__ int64_t lower_bound_u64(const uint64_t* a, int64_t n, uint64_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (a[m] < x) lo = m + 1;
    else hi = m;
  }
  return lo;
}

__device__ __forceinline__ bool has_iface(const Scene& s, int i, int j) {
  // unbroken interface (i, j) stored under its first body (Rockable.cpp:1637-1641)
  int64_t lo = s.if_ofs[i], hi = s.if_ofs[i + 1];
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (s.if_j[m] < j) lo = m + 1;
    else hi = m;
  }
  return lo < s.if_ofs[i + 1] && s.if_j[lo] == j && !s.if_broken[lo];
}

// The FP64 separating-axis test of two placed boxes enlarged by DVerlet/2
// (Rockable.cpp:1627-1654), decided in float where the answer is clear: a
// separation along one of the six face axes by more than the rounding
// margin makes the FP64 test false as well, and one box's centre inside the
// other (shrunk by the margin) makes it true as well; then the nine edge-edge
// axes the same way, and an overlap by more than the margin along all
// fifteen axes makes it true; only the cases in between run the FP64 test,
// so the result is the FP64 test's.
__device__ __forceinline__ bool obb_pair_intersect(const Scene& s, int64_t i, int64_t j) {
  const float* A = s.bobbf + 15 * i;
  const float* B = s.bobbf + 15 * j;
  const float d = 0.5f * (float)s.DVerlet;
  const float ea[3] = {A[12] + d, A[13] + d, A[14] + d}, eb[3] = {B[12] + d, B[13] + d, B[14] + d};
  const float tx = B[0] - A[0], ty = B[1] - A[1], tz = B[2] - A[2];
  float R[3][3];
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      R[a][b] = A[3 + 3 * a] * B[3 + 3 * b] + A[4 + 3 * a] * B[4 + 3 * b] + A[5 + 3 * a] * B[5 + 3 * b];
  const float mag = fmaxf(fmaxf(fabsf(A[0]), fabsf(A[1])), fabsf(A[2])) + fmaxf(fmaxf(fabsf(B[0]), fabsf(B[1])), fabsf(B[2])) +
                    ea[0] + ea[1] + ea[2] + eb[0] + eb[1] + eb[2];
  const float m = 1e-6f * mag + 1e-9f;
  bool in_a = true, in_b = true;
  bool clear = true;  // every axis so far overlaps by more than its margin
  float ta[3];
  for (int a = 0; a < 3; a++) {  // face axes of A
    ta[a] = tx * A[3 + 3 * a] + ty * A[4 + 3 * a] + tz * A[5 + 3 * a];
    const float t = fabsf(ta[a]);
    const float r = ea[a] + eb[0] * fabsf(R[a][0]) + eb[1] * fabsf(R[a][1]) + eb[2] * fabsf(R[a][2]);
    if (t > r + m) return false;
    in_a = in_a && t < ea[a] - m;
    clear = clear && t < r - m;
  }
  for (int b = 0; b < 3; b++) {  // face axes of B
    const float t = fabsf(tx * B[3 + 3 * b] + ty * B[4 + 3 * b] + tz * B[5 + 3 * b]);
    const float r = eb[b] + ea[0] * fabsf(R[0][b]) + ea[1] * fabsf(R[1][b]) + ea[2] * fabsf(R[2][b]);
    if (t > r + m) return false;
    in_b = in_b && t < eb[b] - m;
    clear = clear && t < r - m;
  }
  if (in_a || in_b) return true;
  // the nine edge-edge axes A_a x B_b, in A's frame; one more product level
  // than the face axes, hence the wider margin
  const float mc = 4e-6f * mag + 1e-9f;
  for (int a = 0; a < 3; a++) {
    const int a1 = a == 2 ? 0 : a + 1, a2 = a == 0 ? 2 : a - 1;
    for (int b = 0; b < 3; b++) {
      const int b1 = b == 2 ? 0 : b + 1, b2 = b == 0 ? 2 : b - 1;
      const float r = ea[a1] * fabsf(R[a2][b]) + ea[a2] * fabsf(R[a1][b]) + eb[b1] * fabsf(R[a][b2]) +
                      eb[b2] * fabsf(R[a][b1]);
      const float t = fabsf(ta[a2] * R[a1][b] - ta[a1] * R[a2][b]);
      if (t > r + mc) return false;
      clear = clear && t < r - mc;
    }
  }
  // no axis separates in FP64 either when all fifteen overlap by more than
  // their margins: the FP64 test is true
  if (clear) return true;
  Obb oi = load_obb(s.bobb + 15 * i), oj = load_obb(s.bobb + 15 * j);
  enlarge(oi, 0.5 * s.DVerlet);
  enlarge(oj, 0.5 * s.DVerlet);
  return obb_intersect(oi, oj);
}

// All-pairs broad phase: float AABB filter (tiled through shared memory),
// then eligibility and the FP64 SAT of the enlarged OBBs.
constexpr int kPairTile = 128;
__global__ void k_pairs(Scene s, const uint8_t* only, uint64_t* pairs, int64_t cap, unsigned long long* counter) {
  __shared__ float sb[kPairTile][6];
  const int64_t i = blockIdx.x * (int64_t)kPairTile + threadIdx.x;
  const bool vi = i < s.n;
  float a[6];
  for (int k = 0; k < 6; k++) a[k] = vi ? s.baabb[6 * i + k] : 0.f;
  const int64_t jstart = blockIdx.x * (int64_t)kPairTile;
  for (int64_t j0 = jstart; j0 < s.n; j0 += kPairTile) {
    __syncthreads();
    int64_t jl = j0 + threadIdx.x;
    if (jl < s.n)
      for (int k = 0; k < 6; k++) sb[threadIdx.x][k] = s.baabb[6 * jl + k];
    __syncthreads();
    if (!vi) continue;
    int jn = (int)min((int64_t)kPairTile, s.n - j0);
    for (int t = 0; t < jn; t++) {
      int64_t j = j0 + t;
      if (j <= i) continue;
      if (a[0] > sb[t][3] || sb[t][0] > a[3] || a[1] > sb[t][4] || sb[t][1] > a[4] || a[2] > sb[t][5] ||
          sb[t][2] > a[5])
        continue;
      if (i < s.n_driven && j < s.n_driven) continue;
      if (only && !only[i] && !only[j]) continue;
      if (s.scene_of && s.scene_of[i] != s.scene_of[j]) continue;
      if (has_iface(s, (int)i, (int)j)) continue;
      if (!obb_pair_intersect(s, i, j)) continue;
      unsigned long long k = atomicAdd(counter, 1ull);
      if ((int64_t)k < cap) pairs[k] = ((uint64_t)i << 21) | (uint64_t)j;
    }
  }
}


// ------------------------------------------------------------- grid ----
// Uniform grid broad phase (the role of Rockable's linkCells,
// Rockable.cpp:1667-1809): bodies are binned by the centre of their enlarged
// AABB in cells at least as large as every non-oversized body's AABB, so two
// boxes that overlap are in the same or adjacent cells; bodies larger than a
// cell (walls, floors, slopes) are tested against every body of their scene.
// The pair predicate is the same as the all-pairs one: same pairs found.
__device__ __forceinline__ bool pair_predicate(const Scene& s, int64_t i, int64_t j) {
  // i < j
  if (i < s.n_driven && j < s.n_driven) return false;
  if (s.scene_of && s.scene_of[i] != s.scene_of[j]) return false;
  const float* a = s.baabb + 6 * i;
  const float* b = s.baabb + 6 * j;
  if (a[0] > b[3] || b[0] > a[3] || a[1] > b[4] || b[1] > a[4] || a[2] > b[5] || b[2] > a[5]) return false;
  if (has_iface(s, (int)i, (int)j)) return false;
  return obb_pair_intersect(s, i, j);
}

__device__ __forceinline__ float extent_of(const float* bb) {
  return fmaxf(fmaxf(bb[3] - bb[0], bb[4] - bb[1]), bb[5] - bb[2]);
}

__global__ void k_grid_sum(Scene s, double* sum) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = b < s.n ? (double)extent_of(s.baabb + 6 * b) : 0.0;
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(sum, e);
}

// float <-> unsigned with the same order (for atomic min / max)
__device__ __forceinline__ unsigned int ord_of(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
static inline float float_of_ord(unsigned int o) {
  const unsigned int u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// the largest extent among bodies not larger than lim, and the range of all
// bodies' box centres (ordered bits: lo[3] from all-ones, hi[3] from zero)
__global__ void k_grid_max(Scene s, float lim, unsigned int* maxbits, unsigned int* lo, unsigned int* hi) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float e = 0.f;
  unsigned int cl[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, ch[3] = {0u, 0u, 0u};
  if (b < s.n) {
    const float* bb = s.baabb + 6 * b;
    e = extent_of(bb);
    if (!(e <= lim)) e = 0.f;
    for (int a = 0; a < 3; a++) cl[a] = ch[a] = ord_of(0.5f * (bb[a] + bb[3 + a]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    for (int a = 0; a < 3; a++) {
      cl[a] = min(cl[a], __shfl_xor_sync(0xffffffffu, cl[a], o));
      ch[a] = max(ch[a], __shfl_xor_sync(0xffffffffu, ch[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(maxbits, __float_as_uint(e));
    for (int a = 0; a < 3; a++) {
      atomicMin(lo + a, cl[a]);
      atomicMax(hi + a, ch[a]);
    }
  }
}

// Cell code of the sort key (above the 21 body bits): per axis as many bits
// as the cells the bodies' box centres span (plus one spare cell on each
// side), at most 14 (11 with several scenes); several scenes: the scene
// index (mod 512) above them, so bodies of different scenes that share a
// region of space fall in different cells.  The fewer bits, the fewer
// passes of the key sort.  Coordinates are clamped at the edges of the
// range; clamping keeps neighbouring cells neighbours, so the search stays
// conservative (far bodies only share a cell, filtered later).  The largest
// coordinate stays one below all-ones so that no cell code equals the
// all-ones key that sorts the oversized bodies last.
struct CellFormat {
  int bits[3], off[3], max[3];  // per-axis bits, offset of cell 0, largest coordinate
  int total;                    // bits of the code (with the scene's)
  bool batched;
};
static CellFormat make_cell_format(bool batched, float inv_cell, const float lo[3], const float hi[3]) {
  CellFormat f;
  f.batched = batched;
  f.total = batched ? 9 : 0;
  const int cap = batched ? 11 : 14;
  for (int a = 0; a < 3; a++) {
    double c0 = std::floor((double)lo[a] * inv_cell), c1 = std::floor((double)hi[a] * inv_cell);
    if (!(c0 <= c1) || !std::isfinite(c0) || !std::isfinite(c1)) c0 = c1 = 0.0;
    const double range = c1 - c0 + 1.0;  // cells spanned; coordinates 1..range, spare 0 and range + 1
    int b = 1;
    while (b < cap && (double)((1 << b) - 2) < range + 1.0) b++;
    f.bits[a] = b;
    f.max[a] = (1 << b) - 2;
    f.off[a] = (int)std::max(-1e9, std::min(1e9, 1.0 - c0));
    f.total += b;
  }
  return f;
}

__device__ __forceinline__ int cell_coord(float x, float inv_cell, const CellFormat& f, int a) {
  float v = floorf(x * inv_cell) + (float)f.off[a];
  v = fminf(fmaxf(v, 0.f), (float)f.max[a]);
  return (int)v;
}

__device__ __forceinline__ uint64_t cell_code(uint64_t scene, int x, int y, int z, const CellFormat& f) {
  const uint64_t c = ((uint64_t)x << (f.bits[1] + f.bits[2])) | ((uint64_t)y << f.bits[2]) | (uint64_t)z;
  return f.batched ? ((scene & 511u) << (f.bits[0] + f.bits[1] + f.bits[2])) | c : c;
}

__global__ void k_grid_keys(Scene s, CellFormat f, float cell, float inv_cell, uint64_t* keys, int* over,
                            unsigned long long* nover) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= s.n) return;
  const float* bb = s.baabb + 6 * b;
  if (extent_of(bb) > cell) {
    keys[b] = ~0ull;
    over[atomicAdd(nover, 1ull)] = (int)b;
    return;
  }
  const int cx = cell_coord(0.5f * (bb[0] + bb[3]), inv_cell, f, 0), cy = cell_coord(0.5f * (bb[1] + bb[4]), inv_cell, f, 1),
            cz = cell_coord(0.5f * (bb[2] + bb[5]), inv_cell, f, 2);
  const uint64_t scene = f.batched ? (uint64_t)(uint32_t)s.scene_of[b] : 0u;
  keys[b] = (cell_code(scene, cx, cy, cz, f) << 21) | (uint64_t)b;
}

// With `only` (a partial refresh), body i enumerates its pairs when it is
// flagged, with every neighbour that is not flagged or has a larger index.
// kGridLanes threads per body and neighbour column (the nine (x, y) columns
// around its cell), each testing every kGridLanes-th body of the column:
// short chains of dependent loads (key, boxes, interfaces) per thread.
constexpr int kGridLanes = 4;
__global__ void k_grid_pairs(Scene s, CellFormat f, const uint8_t* only, const uint64_t* keys, int64_t nnorm,
                             uint64_t* pairs, int64_t cap, unsigned long long* counter) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = (int)(t % kGridLanes);
  const int64_t g = t / kGridLanes;
  const int64_t k = g / 9;
  const int col = (int)(g - 9 * k);
  if (k >= nnorm) return;
  const uint64_t key = keys[k];
  const int64_t i = (int64_t)(key & ((1u << 21) - 1));
  if (only && !only[i]) return;
  const uint64_t code = key >> 21;
  const int bxyz = f.bits[0] + f.bits[1] + f.bits[2];
  const uint64_t scene = f.batched ? (code >> bxyz) : 0u;
  const int cx = (int)((code >> (f.bits[1] + f.bits[2])) & ((1u << f.bits[0]) - 1u));
  const int cy = (int)((code >> f.bits[2]) & ((1u << f.bits[1]) - 1u)), cz = (int)(code & ((1u << f.bits[2]) - 1u));
  // z is the lowest field of the cell code: the three cells (x, y, z-1..z+1)
  // of a neighbour column are one contiguous key range
  const int z0 = max(cz - 1, 0), z1 = min(cz + 1, f.max[2]);
  const int x = cx + col / 3 - 1, y = cy + col % 3 - 1;
  if (x < 0 || y < 0 || x > f.max[0] || y > f.max[1]) return;
  const uint64_t first = cell_code(scene, x, y, z0, f) << 21;
  const uint64_t last = cell_code(scene, x, y, z1, f);
  for (int64_t q = lower_bound_u64(keys, nnorm, first) + lane; q < nnorm && (keys[q] >> 21) <= last; q += kGridLanes) {
    const int64_t j = (int64_t)(keys[q] & ((1u << 21) - 1));
    if (only ? (j == i || (only[j] && j < i)) : (j <= i)) continue;
    const int64_t lo = min(i, j), hi = max(i, j);
    if (!pair_predicate(s, lo, hi)) continue;
    unsigned long long at = atomicAdd(counter, 1ull);
    if ((int64_t)at < cap) pairs[at] = ((uint64_t)lo << 21) | (uint64_t)hi;
  }
}

// oversized body o against every body j of its scene (each pair once)
__global__ void k_over_pairs(Scene s, const uint8_t* only, const int* over, const uint8_t* is_over, uint64_t* pairs,
                             int64_t cap, unsigned long long* counter) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int o = over[blockIdx.y];
  if (j >= s.n || j == o) return;
  if (is_over[j] && j < o) return;  // counted from the other oversized body
  if (only && !only[o] && !only[j]) return;
  const int64_t i0 = min((int64_t)o, j), j0 = max((int64_t)o, j);
  if (!pair_predicate(s, i0, j0)) return;
  unsigned long long at = atomicAdd(counter, 1ull);
  if ((int64_t)at < cap) pairs[at] = ((uint64_t)i0 << 21) | (uint64_t)j0;
}

__global__ void k_mark_over(const int* over, int nover, uint8_t* is_over) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nover) is_over[over[k]] = 1;
}

// the two bodies of every pair of a partial refresh (their world vertices
// and spheres are the only ones its candidate tests read)
__global__ void k_mark_pair_bodies(const uint64_t* pairs, int64_t np, uint8_t* mark) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= np) return;
  const uint64_t p = pairs[k];
  mark[p >> 21] = 1;
  mark[p & ((1u << 21) - 1)] = 1;
}

__global__ void k_half_pairs(const uint64_t* pairs, int64_t np, uint64_t* hp) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= np) return;
  uint64_t p = pairs[k];
  uint64_t i = p >> 21, j = p & ((1u << 21) - 1);
  hp[2 * k] = (i << 21) | j;
  hp[2 * k + 1] = (j << 21) | i;
}

// ------------------------------------------------- NEAR predicates ----
// Particle.cpp:88-209, with vertex positions from the per-step table.
struct PairView {
  const double* gb;  // owner global vertices
  const double* gp;  // partner global vertices
  int sb, sp;        // shapes
  double Rb, Rp, dmax;
};

__device__ __forceinline__ bool near_vv(const PairView& P, int v, int w) {
  V3 a = g3(P.gb, v), b = g3(P.gp, w);
  double sum = P.Rb + P.Rp + P.dmax;
  return norm2(b - a) <= sum * sum;
}
__device__ __forceinline__ bool near_ve(const Scene& s, const PairView& P, int v, int e) {
  const int eo = s.edge_ofs[P.sp] + e;
  V3 piv = g3(P.gb, v);
  V3 p0 = g3(P.gp, s.edges[2 * eo]), p1 = g3(P.gp, s.edges[2 * eo + 1]);
  V3 E = p1 - p0, w = piv - p0;
  double r = dot(w, E) / dot(E, E);
  if (r < -P.dmax) return false;
  if (r > 1.0 + P.dmax) return false;
  double sum = P.Rb + P.Rp + P.dmax;
  return norm2(piv - (p0 + r * E)) <= sum * sum;
}
__device__ __forceinline__ bool near_vf(const Scene& s, const PairView& P, int v, int f) {
  const int fo = s.face_ofs[P.sp] + f;
  const int v0 = s.face_vofs[fo], nbv = s.face_vofs[fo + 1] - v0;
  const int* fv = s.face_verts + v0;
  V3 A = g3(P.gp, fv[0]), B = g3(P.gp, fv[1]), C = g3(P.gp, fv[nbv - 1]);
  V3 piv = g3(P.gb, v);
  V3 w = piv - A;
  V3 v1 = B - A;
  normalize(v1);
  V3 v2 = C - A;
  V3 n = cross(v1, v2);
  normalize(n);
  double dist = dot(w, n);
  if (dist < 0.0) { n = -n; dist = -dist; }
  V3 Pp = piv - dist * n;
  int odd = 0;
  v2 = cross(n, v1);
  double ori1 = dot(Pp, v1), ori2 = dot(Pp, v2);
  for (int iva = 0; iva < nbv; ++iva) {
    int ivb = iva + 1;
    if (ivb == nbv) ivb = 0;
    V3 pa = g3(P.gp, fv[iva]), pb = g3(P.gp, fv[ivb]);
    double pa1 = dot(pa, v1), pb1 = dot(pb, v1), pa2 = dot(pa, v2), pb2 = dot(pb, v2);
    if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
      if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) odd = 1 - odd;
    }
  }
  if (odd == 1) {
    dist -= (P.Rb + P.Rp);
    if (dist <= P.dmax) return true;
  }
  return false;
}
__device__ __forceinline__ bool near_ee(const Scene& s, const PairView& P, int eb, int ep) {
  const int ob = s.edge_ofs[P.sb] + eb, op = s.edge_ofs[P.sp] + ep;
  V3 pj0 = g3(P.gp, s.edges[2 * op]), pj1 = g3(P.gp, s.edges[2 * op + 1]);
  V3 pi0 = g3(P.gb, s.edges[2 * ob]), pi1 = g3(P.gb, s.edges[2 * ob + 1]);
  V3 Ei = pi1 - pi0, Ej = pj1 - pj0, w = pi0 - pj0;
  double c = dot(Ei, Ei), d = dot(Ej, Ej), e = dot(Ei, Ej);
  double f = (c * d) - (e * e);
  if (fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    double a = dot(Ei, w), b = dot(Ej, w);
    double ss = (e * b - a * d) * f;
    double tt = (c * b - e * a) * f;
    if (ss >= 0.0 && ss <= 1.0 && tt >= 0.0 && tt <= 1.0) {
      V3 n = (pi0 + ss * Ei) - (pj0 + tt * Ej);
      double sum = P.Rb + P.Rp + P.dmax;
      return norm2(n) <= sum * sum;
    }
  }
  return false;
}

// ------------------------------------------ geometric NEAR (skin mode) ----
// Distance-only tests on float coordinates (the vertex spheres' centres are
// the vertices): vertex-vertex, vertex-segment, vertex-polygon and
// segment-segment distances against R_b + R_p + dVerlet plus a rounding
// margin.  Rockable's NEAR predicates also require the projection of a
// vertex inside the face, or the closest points inside both edges, so a
// sub-contact can start to touch after an arbitrarily small sliding motion;
// with distances only, every sub-contact that touches now was within
// dVerlet of touching at its last test whenever the motion since is below
// dVerlet -- what makes the learned-skin guard exact.  Used only with the
// learned skin; the plain and mixed forms keep the reference predicates.
struct G3 {
  float x, y, z;
};
__device__ __forceinline__ G3 gsub(G3 a, G3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ G3 gmad(G3 a, float t, G3 d) { return {a.x + t * d.x, a.y + t * d.y, a.z + t * d.z}; }
__device__ __forceinline__ float gdot(G3 a, G3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ G3 gcross(G3 a, G3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ G3 gpt(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ float clamp01(float t) { return fminf(fmaxf(t, 0.f), 1.f); }

__device__ __forceinline__ float pt_seg_d2(G3 p, G3 a, G3 b) {
  const G3 ab = gsub(b, a), ap = gsub(p, a);
  const float l2 = gdot(ab, ab);
  const float t = l2 > 0.f ? clamp01(gdot(ap, ab) / l2) : 0.f;
  const G3 d = gmad(ap, -t, ab);
  return gdot(d, d);
}

// squared distance of a point to the line through a and b
__device__ __forceinline__ float pt_line_d2(G3 p, G3 a, G3 b) {
  const G3 ab = gsub(b, a), ap = gsub(p, a);
  const float l2 = gdot(ab, ab);
  const float t = l2 > 0.f ? gdot(ap, ab) / l2 : 0.f;
  const G3 d = gmad(ap, -t, ab);
  return gdot(d, d);
}

// true when the lines through two segments are farther apart than sqrt(lim2)
// (the line distance bounds the segment distance from below); never for
// nearly parallel lines, where that distance is ill-conditioned
__device__ __forceinline__ bool lines_far(G3 p1, G3 q1, G3 p2, G3 q2, float lim2) {
  const G3 d1 = gsub(q1, p1), d2 = gsub(q2, p2), r = gsub(p1, p2);
  const G3 n = gcross(d1, d2);
  const float nn = gdot(n, n);
  if (!(nn > 1e-6f * gdot(d1, d1) * gdot(d2, d2))) return false;
  const float rn = gdot(r, n);
  return rn * rn > lim2 * nn;
}

// Float classification in front of the FP64 NEAR predicates (Rockable's,
// above): from the float world coordinates of the sub-elements (the vertex
// spheres' centres, rounded to nearest from the FP64 world vertices: errors
// of a few 1e-8 of the coordinates' magnitude `mag`), each returns 1 only
// when the FP64 predicate is true for sure -- its distance within `alim` (the
// NEAR distance shrunk by the rejection's rounding margin) and its projection
// parameters or point inside their ranges by more than their rounding error
// -- and -1 only when it is false for sure: a projection parameter or point
// outside its range by more than that error.  On 0 the FP64 predicate
// decides.  (The distance rejections sit at the call sites.)
__device__ __forceinline__ bool accept_vv(G3 a, G3 b, float alim) {
  const G3 d = gsub(a, b);
  return alim > 0.f && gdot(d, d) <= alim * alim;
}
__device__ __forceinline__ int classify_ve(G3 p, G3 a, G3 b, float alim, float dmax, float mag) {
  const G3 E = gsub(b, a), w = gsub(p, a);
  const float E2 = gdot(E, E);
  if (!(E2 > 0.f)) return 0;
  const float r = gdot(w, E) / E2;
  const float tol = 1e-5f + 4e-6f * mag * rsqrtf(E2) * (1.f + fabsf(r));
  if (r < -dmax - tol || r > 1.f + dmax + tol) return -1;  // the FP64 projection test fails too
  if (!(alim > 0.f) || !(r >= -dmax + tol && r <= 1.f + dmax - tol)) return 0;
  const G3 d = gmad(w, -r, E);
  return gdot(d, d) <= alim * alim ? 1 : 0;
}
__device__ __forceinline__ int classify_vf_tri(G3 p, G3 A, G3 B, G3 C, float alim, float mag) {
  const G3 bA = gsub(B, A), cA = gsub(C, A), w = gsub(p, A);
  G3 n = gcross(bA, cA);
  const float nn = gdot(n, n);
  // a well-shaped triangle (the sine of its angle at A above 1e-3), so that
  // the float normal and in-plane distances carry only rounding errors
  if (!(nn > 1e-6f * gdot(bA, bA) * gdot(cA, cA))) return 0;
  const float inv = rsqrtf(nn);
  n = {n.x * inv, n.y * inv, n.z * inv};
  const float dist = gdot(w, n);
  const G3 P = gmad(w, -dist, n);
  const float tol = 1e-9f + 2e-6f * mag;
  const G3 ed[3] = {bA, gsub(cA, bA), {-cA.x, -cA.y, -cA.z}};
  const G3 st[3] = {{0.f, 0.f, 0.f}, bA, cA};
  bool inside = true;
  for (int q = 0; q < 3; q++) {  // counter-clockwise about n: inside is to the left of every edge
    const float side = gdot(gcross(ed[q], gsub(P, st[q])), n) * rsqrtf(gdot(ed[q], ed[q]));
    if (side < -tol) return -1;  // projection outside the triangle: even crossing number in FP64 too
    inside = inside && side > tol;
  }
  return inside && alim > 0.f && fabsf(dist) <= alim ? 1 : 0;
}
__device__ __forceinline__ int classify_ee(G3 pi0, G3 pi1, G3 pj0, G3 pj1, float alim, float mag) {
  const G3 Ei = gsub(pi1, pi0), Ej = gsub(pj1, pj0), w = gsub(pi0, pj0);
  const float c = gdot(Ei, Ei), d = gdot(Ej, Ej), e = gdot(Ei, Ej);
  const float f = c * d - e * e;
  // well away from the FP64 test's parallel threshold (1e-12) and from
  // parallel edges (the sine of their angle above 0.1)
  if (!(f > 2e-12f + 0.01f * c * d)) return 0;
  const float a = gdot(Ei, w), b = gdot(Ej, w);
  const float fi = 1.f / f;
  const float ss = (e * b - a * d) * fi, tt = (c * b - e * a) * fi;
  const float tol = 1e-5f + 4e-5f * mag * rsqrtf(fminf(c, d)) * (1.f + fabsf(ss) + fabsf(tt));
  if (ss < -tol || ss > 1.f + tol || tt < -tol || tt > 1.f + tol) return -1;  // closest points off an edge
  if (!(alim > 0.f) || !(ss >= tol && ss <= 1.f - tol && tt >= tol && tt <= 1.f - tol)) return 0;
  const G3 n = gsub(gmad(pi0, ss, Ei), gmad(pj0, tt, Ej));
  return gdot(n, n) <= alim * alim ? 1 : 0;
}

// squared distance of two segments: the closest-point parameters minimise
// |p1 + s d1 - p2 - t d2| over [0,1]^2 (interior stationary point, else the
// best clamped edge of the square)
__device__ __forceinline__ float seg_seg_d2(G3 p1, G3 q1, G3 p2, G3 q2) {
  const G3 d1 = gsub(q1, p1), d2 = gsub(q2, p2), r = gsub(p1, p2);
  const float a = gdot(d1, d1), e = gdot(d2, d2), f = gdot(d2, r), c = gdot(d1, r), b = gdot(d1, d2);
  float s = 0.f, t = 0.f;
  if (a <= 1e-30f && e <= 1e-30f) {
    s = t = 0.f;
  } else if (a <= 1e-30f) {
    t = clamp01(f / e);
  } else if (e <= 1e-30f) {
    s = clamp01(-c / a);
  } else {
    const float den = a * e - b * b;
    s = den > 0.f ? clamp01((b * f - c * e) / den) : 0.f;
    t = (b * s + f) / e;
    if (t < 0.f) {
      t = 0.f;
      s = clamp01(-c / a);
    } else if (t > 1.f) {
      t = 1.f;
      s = clamp01((b - c) / a);
    }
  }
  const G3 w = gsub(gmad(p1, s, d1), gmad(p2, t, d2));
  return gdot(w, w);
}

// squared distance of a point to a planar polygon (vertices in order)
__device__ __forceinline__ float pt_poly_d2(const Scene& s, const float4* sp, int sh, int f, G3 p) {
  const int fo = s.face_ofs[sh] + f;
  const int v0 = s.face_vofs[fo], nbv = s.face_vofs[fo + 1] - v0;
  const int* fv = s.face_verts + v0;
  const G3 A = gpt(sp[fv[0]]), B = gpt(sp[fv[1]]), C = gpt(sp[fv[nbv - 1]]);
  G3 n = gcross(gsub(B, A), gsub(C, A));
  const float nn = gdot(n, n);
  float best = 3.0e38f;
  if (nn > 0.f) {
    const float inv = rsqrtf(nn);
    n = {n.x * inv, n.y * inv, n.z * inv};
    const float dist = gdot(gsub(p, A), n);
    // crossing number of the projection, in the plane
    const G3 u = gsub(B, A);
    const float iu = rsqrtf(fmaxf(gdot(u, u), 1e-30f));
    const G3 e1 = {u.x * iu, u.y * iu, u.z * iu};
    const G3 e2 = gcross(n, e1);
    const G3 q = gsub(p, A);
    const float o1 = gdot(q, e1), o2 = gdot(q, e2);
    int odd = 0;
    for (int k = 0; k < nbv; k++) {
      const G3 pa = gsub(gpt(sp[fv[k]]), A), pb = gsub(gpt(sp[fv[k + 1 == nbv ? 0 : k + 1]]), A);
      const float a1 = gdot(pa, e1), b1 = gdot(pb, e1), a2 = gdot(pa, e2), b2 = gdot(pb, e2);
      if ((a2 < o2 && b2 >= o2) || (b2 < o2 && a2 >= o2))
        if (a1 + (o2 - a2) / (b2 - a2) * (b1 - a1) < o1) odd = 1 - odd;
    }
    if (odd) best = dist * dist;
  }
  for (int k = 0; k < nbv; k++)
    best = fminf(best, pt_seg_d2(p, gpt(sp[fv[k]]), gpt(sp[fv[k + 1 == nbv ? 0 : k + 1]])));
  return best;
}

// classify_vf_tri on a face of the partner's shape (triangles only: other
// polygons go to the FP64 predicate)
__device__ __forceinline__ int classify_vf(const Scene& s, const float4* sp, int sh, int f, G3 p, float alim,
                                           float mag) {
  const int fo = s.face_ofs[sh] + f;
  const int v0 = s.face_vofs[fo], nbv = s.face_vofs[fo + 1] - v0;
  if (nbv != 3) return 0;
  const int* fv = s.face_verts + v0;
  return classify_vf_tri(p, gpt(sp[fv[0]]), gpt(sp[fv[1]]), gpt(sp[fv[2]]), alim, mag);
}

// the float class decides unless it is 0
#define RK_DECIDE(cls, exact) ([&] { const int c_ = (cls); return c_ > 0 || (c_ == 0 && (exact)); }())

// Candidate sub-contacts of the half-pairs: one warp per half-pair (owner b
// -> partner p).  The lanes first compute, in parallel, the owner vertices
// that pass the OBB cull (FP64 SAT of the vertex cube against p's box
// enlarged by dVerlet; this mask also tells the old-entry pass which
// candidates were tested) and the sub-elements of each body that a
// conservative float bounding-sphere test leaves within reach of the other
// body; those index lists go to shared memory.  The lanes then sweep the
// products of the lists 32 candidates at a time: float sphere prefilter,
// then the FP64 NEAR predicate, and the survivors are appended with one
// atomic per warp and ballot.  Appending leaves the keys unordered; they are
// sorted afterwards.  The float tests only skip candidates that cannot be
// NEAR, so the NEAR set is exactly the one of testing every candidate.
constexpr int kCandWarps = 4;  // warps per block

// Root-versus-leaf test of the two-level pruning: true when a sub-element
// sphere (centre, radius in .w) lies farther than `reach` from the other
// body's vertex box bx (float: centre, 3 axes, half extents).  The box holds
// that body's core, so such an element is farther than `reach` from every
// sub-element of it; the margin covers the float rounding of the box, the
// centre and the projections.
__device__ __forceinline__ bool box_far(const float* bx, float4 c, float reach, float slack) {
  const float dx = c.x - bx[0], dy = c.y - bx[1], dz = c.z - bx[2];
  float d2 = 0.f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float t = fabsf(dx * bx[3 + 3 * k] + dy * bx[4 + 3 * k] + dz * bx[5 + 3 * k]) - bx[12 + k];
    if (t > 0.f) d2 += t * t;
  }
  float lim = c.w + reach;
  lim = lim + 1e-4f * lim + slack + 1e-6f * (fabsf(dx) + fabsf(dy) + fabsf(dz) + bx[12] + bx[13] + bx[14]);
  return d2 > lim * lim;
}

// The owner-vertex cull's FP64 test (Rockable.cpp:1385-1391): the cube of
// half-size r around vertex v against the partner's OBB enlarged by dmax.
// Not inlined: inlined, the compiler evaluated it for every vertex and
// selected the result (about 300 FP64 operations per vertex), although the
// float pre-test leaves it to fewer than one vertex in 4000.
__device__ __noinline__ bool cull_fp64(const double* obb, double dmax, const double* gb, int v, double r) {
  Obb op = load_obb(obb);
  enlarge(op, dmax);
  Obb sub;
  sub.c = g3(gb, v);
  sub.e0 = v3(1, 0, 0);
  sub.e1 = v3(0, 1, 0);
  sub.e2 = v3(0, 0, 1);
  sub.ext = v3(r, r, r);
  return obb_intersect(op, sub);
}

struct CandLists {
  uint16_t bv[64], pv[64];                   // owner / partner vertices
  uint16_t be[kMaxSub], pe[kMaxSub], pf[kMaxSub];  // owner edges, partner edges and faces
};

// Indices k < n with pred(k), in increasing order, written by the warp.
template <class Pred>
__device__ __forceinline__ int warp_list(uint16_t* list, int n, int lane, Pred pred) {
  int cnt = 0;
  for (int base = 0; base < n; base += 32) {
    const int k = base + lane;
    const bool ok = k < n && pred(k);
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    if (ok) list[cnt + __popc(bal & ((1u << lane) - 1u))] = (uint16_t)k;
    cnt += __popc(bal);
  }
  __syncwarp();
  return cnt;
}

__device__ __forceinline__ void warp_emit(bool ok, uint64_t key, int lane, uint64_t* out, int64_t cap,
                                          unsigned long long* counter) {
  const unsigned bal = __ballot_sync(0xffffffffu, ok);
  if (!bal) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(counter, (unsigned long long)__popc(bal));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (ok) {
    const unsigned long long at = base + __popc(bal & ((1u << lane) - 1u));
    if ((int64_t)at < cap) out[at] = key;
  }
}

// The FP64 variant asks for 4 blocks per SM (128 registers, a few spills to
// L1) instead of 3 at 166 registers: it is latency-bound.
template <bool GEOM>
__global__ void __launch_bounds__(32 * kCandWarps, GEOM ? 1 : 4)
k_candidates(Scene s, const uint64_t* hp, int64_t nhp, uint32_t* mask, uint64_t* out, int64_t cap,
             unsigned long long* counter) {
  __shared__ CandLists lists[kCandWarps];
  const int lane = threadIdx.x & 31;
  CandLists& L = lists[threadIdx.x >> 5];
  const int64_t stride = (int64_t)gridDim.x * kCandWarps;
  for (int64_t h = (int64_t)blockIdx.x * kCandWarps + (threadIdx.x >> 5); h < nhp; h += stride) {
    __syncwarp();  // the previous half-pair's lists have been read
    const uint64_t key = hp[h];
    const int b = (int)(key >> 21), p = (int)(key & ((1u << 21) - 1));
    PairView P;
    P.gb = s.gv + 3 * s.gv_ofs[b];
    P.gp = s.gv + 3 * s.gv_ofs[p];
    P.sb = s.shape[b];
    P.sp = s.shape[p];
    P.Rb = s.rad[b];
    P.Rp = s.rad[p];
    P.dmax = s.dVerlet;
    const int nvb = s.vert_ofs[P.sb + 1] - s.vert_ofs[P.sb];
    const int nvp = s.vert_ofs[P.sp + 1] - s.vert_ofs[P.sp];
    const int neb = s.edge_ofs[P.sb + 1] - s.edge_ofs[P.sb];
    const int nep = s.edge_ofs[P.sp + 1] - s.edge_ofs[P.sp];
    const int nfp = s.face_ofs[P.sp + 1] - s.face_ofs[P.sp];
    // owner-vertex cull (Rockable.cpp:1385-1391): the vertex cube against
    // the partner's OBB enlarged by dVerlet.  With the distance-only tests a
    // conservative float test does (a vertex out of reach of the partner's
    // bounding sphere), since an untested candidate only keeps its old entry.
    uint32_t m0, m1;
    if (GEOM) {
      const float4* sbv = s.sph + s.sph_ofs[b];
      const float4 cpp = make_float4(d2f(s.pos[3 * p]), d2f(s.pos[3 * p + 1]), d2f(s.pos[3 * p + 2]), s.bnd[p]);
      const float reach = d2f(P.Rb + P.Rp + P.dmax);
      bool hit0 = false, hit1 = false;
      for (int half = 0; half < 2; half++) {
        const int v = lane + 32 * half;
        if (v < nvb) {
          const float4 a = sbv[v];
          const float dx = a.x - cpp.x, dy = a.y - cpp.y, dz = a.z - cpp.z;
          const float mg = fmaxf(fmaxf(fmaxf(fabsf(cpp.x), fabsf(cpp.y)), fabsf(cpp.z)) + cpp.w,
                                 fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)));
          float lim = reach + cpp.w;
          lim = lim + 1e-4f * lim + 1e-6f * mg + 2e-6f;
          const bool hit = dx * dx + dy * dy + dz * dz <= lim * lim;
          if (half == 0) hit0 = hit;
          else hit1 = hit;
        }
      }
      m0 = __ballot_sync(0xffffffffu, hit0);
      m1 = __ballot_sync(0xffffffffu, hit1);
    } else {
      Obb op = load_obb(s.bobb + 15 * p);
      enlarge(op, P.dmax);
      const double r = P.Rb + P.dmax;
      // Float pre-test of the fifteen axes of the separating-axis test (the
      // partner box's axes, the cube's -- the world axes -- and their
      // cross products): separated along one by more than the rounding
      // margin -> the FP64 test is false as well; the vertex inside the box
      // shrunk by the margin, or an overlap by more than the margin along
      // all fifteen -> the FP64 test is true as well; only the cases in
      // between run the FP64 test, so the mask is unchanged.
      const float fcx = d2f(op.c.x), fcy = d2f(op.c.y), fcz = d2f(op.c.z);
      const float fe[3][3] = {{d2f(op.e0.x), d2f(op.e0.y), d2f(op.e0.z)},
                              {d2f(op.e1.x), d2f(op.e1.y), d2f(op.e1.z)},
                              {d2f(op.e2.x), d2f(op.e2.y), d2f(op.e2.z)}};
      const float fext[3] = {d2f(op.ext.x), d2f(op.ext.y), d2f(op.ext.z)};
      const float fr = d2f(r);
      const float4* sbv = s.sph + s.sph_ofs[b];
      const float mag = fmaxf(fmaxf(fabsf(fcx), fabsf(fcy)), fabsf(fcz)) + fext[0] + fext[1] + fext[2] + fr;
      bool hit0 = false, hit1 = false;
      for (int half = 0; half < 2; half++) {
        const int v = lane + 32 * half;
        if (v < nvb) {
          const float4 pv = sbv[v];
          const float dw[3] = {pv.x - fcx, pv.y - fcy, pv.z - fcz};
          bool out = false, in = true, clear = true;
          float tb[3];
          for (int i = 0; i < 3; i++) {  // the box's axes
            tb[i] = dw[0] * fe[i][0] + dw[1] * fe[i][1] + dw[2] * fe[i][2];
            const float t = fabsf(tb[i]);
            const float lim = fext[i] + fr * (fabsf(fe[i][0]) + fabsf(fe[i][1]) + fabsf(fe[i][2]));
            const float m = 1e-6f * (mag + t) + 1e-9f;
            out = out || t > lim + m;
            in = in && t < fext[i] - m;
            clear = clear && t < lim - m;
          }
          if (!out && !in) {
            const float m = 1e-6f * mag + 1e-9f, mc = 4e-6f * mag + 1e-9f;
            for (int j = 0; j < 3; j++) {  // the world axes
              const float t = fabsf(dw[j]);
              const float lim = fext[0] * fabsf(fe[0][j]) + fext[1] * fabsf(fe[1][j]) + fext[2] * fabsf(fe[2][j]) + fr;
              out = out || t > lim + m;
              clear = clear && t < lim - m;
            }
            for (int i = 0; i < 3; i++) {  // box axis i x world axis j
              const int i1 = i == 2 ? 0 : i + 1, i2 = i == 0 ? 2 : i - 1;
              for (int j = 0; j < 3; j++) {
                const int j1 = j == 2 ? 0 : j + 1, j2 = j == 0 ? 2 : j - 1;
                const float t = fabsf(tb[i2] * fe[i1][j] - tb[i1] * fe[i2][j]);
                const float lim = fext[i1] * fabsf(fe[i2][j]) + fext[i2] * fabsf(fe[i1][j]) +
                                  fr * (fabsf(fe[i][j2]) + fabsf(fe[i][j1]));
                out = out || t > lim + mc;
                clear = clear && t < lim - mc;
              }
            }
          }
          bool hit;
          if (out) {
            hit = false;
          } else if (in || clear) {
            hit = true;
          } else {
            hit = cull_fp64(s.bobb + 15 * p, P.dmax, P.gb, v, r);
          }
          if (half == 0) hit0 = hit;
          else hit1 = hit;
        }
      }
      m0 = __ballot_sync(0xffffffffu, hit0);
      m1 = __ballot_sync(0xffffffffu, hit1);
    }
    if (lane == 0) {
      mask[kMaskWords * h] = m0;
      mask[kMaskWords * h + 1] = m1;
    }
    // conservative float filter: a candidate whose bounding spheres are
    // farther apart than the NEAR distance allows cannot be NEAR
    const float4* sb = s.sph + s.sph_ofs[b];
    const float4* sp = s.sph + s.sph_ofs[p];
    const float sum = d2f(P.Rb + P.Rp + P.dmax);
    const float4 cb = make_float4(d2f(s.pos[3 * b]), d2f(s.pos[3 * b + 1]), d2f(s.pos[3 * b + 2]), s.bnd[b]);
    const float4 cp = make_float4(d2f(s.pos[3 * p]), d2f(s.pos[3 * p + 1]), d2f(s.pos[3 * p + 2]), s.bnd[p]);
    // margin for the float rounding of coordinates of magnitude up to `mag`
    // (about 16 ulps of it) on top of a relative 1e-4
    const float mag = fmaxf(fmaxf(fmaxf(fabsf(cb.x), fabsf(cb.y)), fabsf(cb.z)) + cb.w,
                            fmaxf(fmaxf(fabsf(cp.x), fabsf(cp.y)), fabsf(cp.z)) + cp.w);
    const float slack = 1e-6f * mag + 2e-6f;
    auto far = [&](float4 a, float4 c, float extent) {
      float dx = a.x - c.x, dy = a.y - c.y, dz = a.z - c.z;
      float lim = sum + extent;
      lim = lim + 1e-4f * lim + slack;
      return dx * dx + dy * dy + dz * dz > lim * lim;
    };
    const float ve_ext = d2f(1.0 + 2.0 * P.dmax);
    const float glim = sum + 1e-4f * sum + slack;
    const float glim2 = glim * glim;
    const float alim = sum - (1e-4f * sum + slack);  // float acceptance: the NEAR distance shrunk by the margin
    const float dmaxf = d2f(P.dmax);
    const bool lower = b < p;  // vertex-vertex and edge-edge pairs are tested in the i < j direction only
    // Two-level pruning (the role of Rockable's per-shape OBB trees,
    // Rockable.cpp:1440-1541, Shape.cpp:628-670): a sub-element stays in
    // its list only when its sphere reaches the other body's bounding
    // sphere and its vertex box (root against leaf); the products of the
    // lists then test sphere against sphere (leaf against leaf) before the
    // NEAR predicate.  Only elements that cannot be NEAR are dropped.
    const float* bxb = s.bbox + 15 * b;
    const float* bxp = s.bbox + 15 * p;
    // an owner vertex meets the partner's edges up to dmax x their length
    // beyond their ends (the vertex-edge projection test), so its reach
    // grows by that much (an edge is at most the partner's diameter long)
    const float vreach = sum + 2.f * dmaxf * cp.w;
    const int nbv = warp_list(L.bv, nvb, lane, [&](int v) {
      return (((v < 32 ? m0 : m1) >> (v & 31)) & 1u) != 0u && !box_far(bxp, sb[v], vreach, slack);
    });
    const int npv = lower ? warp_list(L.pv, nvp, lane, [&](int w) {
      return !far(sp[w], cb, cb.w) && !box_far(bxb, sp[w], sum, slack);
    }) : 0;
    const int npe = warp_list(L.pe, nep, lane, [&](int e) {
      const float4 se = sp[nvp + e];
      const float4 sx = make_float4(se.x, se.y, se.z, ve_ext * se.w);  // the vertex-edge test's extended edge
      return !far(se, cb, cb.w + sx.w) && !box_far(bxb, sx, sum, slack);
    });
    const int npf = warp_list(L.pf, nfp, lane, [&](int f) {
      const float4 sf = sp[nvp + nep + f];
      return !far(sf, cb, cb.w + sf.w) && !box_far(bxb, sf, sum, slack);
    });
    const int nbe = lower ? warp_list(L.be, neb, lane, [&](int e) {
      const float4 se = sb[nvb + e];
      return !far(se, cp, cp.w + se.w) && !box_far(bxp, se, sum, slack);
    }) : 0;
    // vertex-vertex
    for (int base = 0, tot = nbv * npv; base < tot; base += 32) {
      const int c = base + lane;
      bool ok = false;
      int v = 0, w = 0;
      if (c < tot) {
        v = L.bv[c / npv];
        w = L.pv[c % npv];
        if (GEOM) {
          const G3 d = gsub(gpt(sb[v]), gpt(sp[w]));
          ok = gdot(d, d) <= glim2;
        } else {
          ok = !far(sb[v], sp[w], 0.f) && (accept_vv(gpt(sb[v]), gpt(sp[w]), alim) || near_vv(P, v, w));
        }
      }
      warp_emit(ok, entry_key((uint32_t)b, (uint32_t)p, 0u, (uint32_t)v, (uint32_t)w), lane, out, cap, counter);
    }
    // vertex-edge
    for (int base = 0, tot = nbv * npe; base < tot; base += 32) {
      const int c = base + lane;
      bool ok = false;
      int v = 0, e = 0;
      if (c < tot) {
        v = L.bv[c / npe];
        e = L.pe[c % npe];
        const float4 se = sp[nvp + e];
        if (GEOM) {
          const int eo = s.edge_ofs[P.sp] + e;
          ok = !far(sb[v], se, se.w) &&
               pt_seg_d2(gpt(sb[v]), gpt(sp[s.edges[2 * eo]]), gpt(sp[s.edges[2 * eo + 1]])) <= glim2;
        } else {
          // exact rejection first: Rockable's vertex-edge test accepts a
          // projection slightly off the edge, never a line distance above it
          const int eo = s.edge_ofs[P.sp] + e;
          const G3 pv = gpt(sb[v]), e0 = gpt(sp[s.edges[2 * eo]]), e1 = gpt(sp[s.edges[2 * eo + 1]]);
          ok = !far(sb[v], se, ve_ext * se.w) && pt_line_d2(pv, e0, e1) <= glim2 &&
               RK_DECIDE(classify_ve(pv, e0, e1, alim, dmaxf, mag), near_ve(s, P, v, e));
        }
      }
      warp_emit(ok, entry_key((uint32_t)b, (uint32_t)p, 1u, (uint32_t)v, (uint32_t)e), lane, out, cap, counter);
    }
    // vertex-face
    for (int base = 0, tot = nbv * npf; base < tot; base += 32) {
      const int c = base + lane;
      bool ok = false;
      int v = 0, f = 0;
      if (c < tot) {
        v = L.bv[c / npf];
        f = L.pf[c % npf];
        const float4 sf = sp[nvp + nep + f];
        if (GEOM) ok = !far(sb[v], sf, sf.w) && pt_poly_d2(s, sp, P.sp, f, gpt(sb[v])) <= glim2;
        else  // exact rejection first: NEAR needs the polygon within reach
          ok = !far(sb[v], sf, sf.w) && pt_poly_d2(s, sp, P.sp, f, gpt(sb[v])) <= glim2 &&
               RK_DECIDE(classify_vf(s, sp, P.sp, f, gpt(sb[v]), alim, mag), near_vf(s, P, v, f));
      }
      warp_emit(ok, entry_key((uint32_t)b, (uint32_t)p, 2u, (uint32_t)v, (uint32_t)f), lane, out, cap, counter);
    }
    // edge-edge
    for (int base = 0, tot = nbe * npe; base < tot; base += 32) {
      const int c = base + lane;
      bool ok = false;
      int e1 = 0, e2 = 0;
      if (c < tot) {
        e1 = L.be[c / npe];
        e2 = L.pe[c % npe];
        const float4 s1 = sb[nvb + e1], s2 = sp[nvp + e2];
        if (GEOM) {
          // nearly parallel edges (ill-conditioned closest points) within
          // sphere reach are kept: an extra entry is harmless, a missing one not
          const int ob = s.edge_ofs[P.sb] + e1, op = s.edge_ofs[P.sp] + e2;
          const G3 a0 = gpt(sb[s.edges[2 * ob]]), a1 = gpt(sb[s.edges[2 * ob + 1]]);
          const G3 b0 = gpt(sp[s.edges[2 * op]]), b1 = gpt(sp[s.edges[2 * op + 1]]);
          const G3 d1 = gsub(a1, a0), d2 = gsub(b1, b0), nx = gcross(d1, d2);
          const bool parallel = !(gdot(nx, nx) > 1e-6f * gdot(d1, d1) * gdot(d2, d2));
          ok = !far(s1, s2, s1.w + s2.w) && (parallel || seg_seg_d2(a0, a1, b0, b1) <= glim2);
        } else {
          // exact rejection first: NEAR needs the edges' lines within reach
          const int ob = s.edge_ofs[P.sb] + e1, op = s.edge_ofs[P.sp] + e2;
          const G3 a0 = gpt(sb[s.edges[2 * ob]]), a1 = gpt(sb[s.edges[2 * ob + 1]]);
          const G3 b0 = gpt(sp[s.edges[2 * op]]), b1 = gpt(sp[s.edges[2 * op + 1]]);
          ok = !far(s1, s2, s1.w + s2.w) && !lines_far(a0, a1, b0, b1, glim2) &&
               RK_DECIDE(classify_ee(a0, a1, b0, b1, alim, mag), near_ee(s, P, e1, e2));
        }
      }
      warp_emit(ok, entry_key((uint32_t)b, (uint32_t)p, 3u, (uint32_t)e1, (uint32_t)e2), lane, out, cap, counter);
    }
  }
}


// Old entries that were not tested this time are kept as they are.
__global__ void k_stale_flag(const uint64_t* okey, int64_t no, const uint64_t* hp, int64_t nhp, const uint32_t* mask,
                             int64_t* flag) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= no) return;
  const uint64_t k = okey[e];
  const uint64_t i = k >> 43, j = (k >> 22) & ((1u << 21) - 1);
  const int t = (int)((k >> 20) & 3u), isub = (int)((k >> 10) & 1023u);
  const uint64_t hk = (i << 21) | j;
  int64_t h = lower_bound_u64(hp, nhp, hk);
  bool tested = false;
  if (h < nhp && hp[h] == hk) {
    // vertex-vertex and edge-edge candidates exist only in the i < j direction
    if ((t == 0 || t == 3) && i > j) tested = false;
    else tested = (t == 3) || ((mask[kMaskWords * h + (isub >> 5)] >> (isub & 31)) & 1u);
  }
  flag[e] = tested ? 0 : 1;
}

__global__ void k_stale_write(const uint64_t* okey, int64_t no, const int64_t* flag, const int64_t* pos,
                              uint64_t* stale, int64_t* stale_src) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= no || !flag[e]) return;
  stale[pos[e]] = okey[e];
  stale_src[pos[e]] = e;
}

__global__ void k_merge(const uint64_t* stale, const int64_t* stale_src, int64_t ns, const uint64_t* cand, int64_t nc,
                        const uint64_t* okey, int64_t no, uint64_t* fkey, int64_t* fsrc) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < ns) {
    uint64_t x = stale[k];
    int64_t p = k + lower_bound_u64(cand, nc, x);
    fkey[p] = x;
    fsrc[p] = stale_src[k];
  } else if (k < ns + nc) {
    int64_t q = k - ns;
    uint64_t x = cand[q];
    int64_t p = q + lower_bound_u64(stale, ns, x);
    int64_t o = lower_bound_u64(okey, no, x);
    fkey[p] = x;
    fsrc[p] = (o < no && okey[o] == x) ? o : -1;
  }
}

// Fill the next entry buffer: carried history or a fresh sub-contact with
// the damping of Rockable.cpp:1356-1376 (rate per group pair from the host).
__global__ void k_fill(Scene s, int64_t nf, const uint64_t* fkey, const int64_t* fsrc, EntryBuf ob, EntryBuf nb) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nf) return;
  const uint64_t x = fkey[k];
  const int i = (int)(x >> 43), j = (int)((x >> 22) & ((1u << 21) - 1));
  const uint32_t t = (uint32_t)((x >> 20) & 3u), isub = (uint32_t)((x >> 10) & 1023u), jsub = (uint32_t)(x & 1023u);
  nb.ei[k] = i;
  nb.ej[k] = j;
  nb.etsub[k] = pack_tsub(t, isub, jsub);
  nb.ekey[k] = x;
  const int64_t o = fsrc[k];
  if (o >= 0) {
    nb.dn[k] = ob.dn[o];
    nb.fn[k] = ob.fn[o];
    nb.damp[k] = ob.damp[o];
    nb.bond[k] = ob.bond[o];
    for (int d = 0; d < 3; d++) {
      nb.ft[3 * k + d] = ob.ft[3 * o + d];
      nb.mom[3 * k + d] = ob.mom[3 * o + d];
      nb.gn[3 * k + d] = ob.gn[3 * o + d];
      nb.gpos[3 * k + d] = ob.gpos[3 * o + d];
      nb.gvel[3 * k + d] = ob.gvel[3 * o + d];
    }
  } else {
    const double* P = s.table[s.group[i] * s.ngroup + s.group[j]].p;
    double meff;
    if (i < s.n_driven) meff = s.mass[j];
    else if (j < s.n_driven) meff = s.mass[i];
    else meff = (s.mass[i] * s.mass[j]) / (s.mass[i] + s.mass[j]);
    nb.damp[k] = P[22] * 2.0 * sqrt(P[RK_P_KN] * meff);
    nb.dn[k] = 0.0;
    nb.fn[k] = 0.0;
    nb.bond[k] = -1;
    for (int d = 0; d < 3; d++) {
      nb.ft[3 * k + d] = 0.0;
      nb.mom[3 * k + d] = 0.0;
      nb.gn[3 * k + d] = 0.0;
      nb.gpos[3 * k + d] = 0.0;
      nb.gvel[3 * k + d] = 0.0;
    }
  }
}

__global__ void k_iofs(const uint64_t* key, int64_t ne, int64_t nb, int64_t* iofs) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b > nb) return;
  iofs[b] = lower_bound_u64(key, ne, (uint64_t)b << 43);
}

__global__ void k_jkeys(const int* ej, int64_t ne, uint64_t* jk) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  jk[e] = ((uint64_t)ej[e] << 27) | (uint64_t)e;
}

__global__ void k_jlist(const uint64_t* jk, int64_t ne, int* jlist) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  jlist[e] = (int)(jk[e] & ((1ull << 27) - 1));
}

__global__ void k_jofs(const uint64_t* jk, int64_t ne, int64_t nb, int64_t* jofs) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b > nb) return;
  jofs[b] = lower_bound_u64(jk, ne, (uint64_t)b << 27);
}

// ----------------------------------------------------------------- host ----
static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

#define RKCHK(x)                                                              \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      c.err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #x;     \
      return RK_ERR_CUDA;                                                     \
    }                                                                         \
  } while (0)

template <typename T>
static int grow(Ctx& c, T*& p, int64_t n_old, int64_t n_new) {
  (void)n_old;
  if (p) cudaFree(p);
  p = nullptr;
  cudaError_t e = cudaMalloc(&p, (size_t)std::max<int64_t>(n_new, 1) * sizeof(T));
  if (e != cudaSuccess) {
    c.err = std::string("CUDA: ") + cudaGetErrorString(e) + " (neighbour-list scratch)";
    return RK_ERR_CUDA;
  }
  return 0;
}

static int ensure_tmp(Ctx& c, int64_t bytes) {
  if (bytes <= c.w.tmp_bytes) return 0;
  int64_t nb = std::max<int64_t>(bytes, c.w.tmp_bytes * 3 / 2);
  if (c.w.tmp) cudaFree(c.w.tmp);
  c.w.tmp = nullptr;
  if (cudaMalloc(&c.w.tmp, (size_t)nb) != cudaSuccess) {
    c.err = "CUDA: cannot allocate neighbour-list temp";
    return RK_ERR_CUDA;
  }
  c.w.tmp_bytes = nb;
  return 0;
}

// bits of the largest body index: the sorts skip the key bits no body uses
static int body_bits(int64_t n) {
  int b = 1;
  while (b < 21 && ((int64_t)1 << b) < n) b++;
  return b;
}

static int64_t read_i64(Ctx& c, const int64_t* d) {
  int64_t v = 0;
  cudaMemcpyAsync(&v, d, sizeof v, cudaMemcpyDeviceToHost, c.stream);
  cudaStreamSynchronize(c.stream);
  return v;
}

int rebuild_nl(Ctx& c, const uint8_t* only) {
  Scene& s = c.s;
  NLWork& w = c.w;
  cudaStream_t st = c.stream;
  int rc;
  const int64_t N = s.n;
  if (N <= 0) return 0;
  RKCHK(cudaMemsetAsync(s.flags + FLAG_NONFINITE, 0, sizeof(unsigned long long), st));
  // The boxes of every body; the world vertices and the sub-element spheres
  // (the step computed only the listed bodies' vertices) of every body for a
  // full build, of the bodies of the visited pairs for a partial refresh
  // (after the pairs are known).
  const bool defer = only != nullptr;
  const int64_t nsph = c.nsph;
  RKCHK(cudaMemsetAsync(s.bnd, 0, (size_t)N * sizeof(float), st));
  if (!defer) {
    c.kernels += launch_glob_vertices(s, st, true);
    if (nsph > 0) k_spheres<<<nblk(nsph, 256), 256, 0, st>>>(s, nsph, nullptr);
    c.kernels++;
  }
  k_body_obb<<<nblk(N, 128), 128, 0, st>>>(s);
  c.kernels++;
  {  // a body whose state is no longer finite: stop here, loudly
    unsigned long long bad = 0;
    RKCHK(cudaMemcpyAsync(&bad, s.flags + FLAG_NONFINITE, sizeof bad, cudaMemcpyDeviceToHost, st));
    RKCHK(cudaStreamSynchronize(st));
    if (bad) {
      c.err = "non-finite position or orientation of body " + std::to_string(bad - 1) +
              " (unstable time step or exploding contact?)";
      return RK_ERR_NUMERIC;
    }
  }
  // ---- pairs
  if (w.pair_cap < 16 * N + 1024) {
    int64_t nc = 16 * N + 1024;
    if ((rc = grow(c, w.pairs, w.pair_cap, nc))) return rc;
    w.pair_cap = nc;
  }
  if (!w.counter) RKCHK(cudaMalloc(&w.counter, 64));
  int64_t np = -1;
  bool use_grid = (c.broadphase == 2) || (c.broadphase == 0 && N > 4096);
  float cell = 0.f, clo[3] = {0.f, 0.f, 0.f}, chi[3] = {0.f, 0.f, 0.f};
  int64_t nover = 0;
  const bool reuse_grid = use_grid && only != nullptr && c.grid_n == N && c.last_cell > 0.f;
  if (use_grid && w.grid_cap < N) {
    if ((rc = grow(c, w.gkeys, w.grid_cap, N)) || (rc = grow(c, w.gtmp, w.grid_cap, N)) ||
        (rc = grow(c, w.gover, w.grid_cap, N)) || (rc = grow(c, w.gis_over, w.grid_cap, N)))
      return rc;
    w.grid_cap = N;
  }
  if (reuse_grid) {
    cell = c.last_cell;
    for (int a = 0; a < 3; a++) {
      clo[a] = c.grid_lo[a];
      chi[a] = c.grid_hi[a];
    }
  } else if (use_grid) {
    // cell size: the largest extent among bodies not larger than 4x the mean
    if (w.grid_cap < N) {
      if ((rc = grow(c, w.gkeys, w.grid_cap, N)) || (rc = grow(c, w.gtmp, w.grid_cap, N)) ||
          (rc = grow(c, w.gover, w.grid_cap, N)) || (rc = grow(c, w.gis_over, w.grid_cap, N)))
        return rc;
      w.grid_cap = N;
    }
    if (!w.gstat) RKCHK(cudaMalloc(&w.gstat, 64));
    RKCHK(cudaMemsetAsync(w.gstat, 0, 64, st));
    k_grid_sum<<<nblk(N, 256), 256, 0, st>>>(s, (double*)w.gstat);
    double mean_sum = 0.0;
    RKCHK(cudaMemcpyAsync(&mean_sum, w.gstat, 8, cudaMemcpyDeviceToHost, st));
    RKCHK(cudaStreamSynchronize(st));
    const float lim = (float)(4.0 * mean_sum / (double)N);
    // gstat: [8] largest extent bits, [24] centre range (3 ordered minima, 3 maxima)
    RKCHK(cudaMemsetAsync((char*)w.gstat + 24, 0xff, 12, st));
    k_grid_max<<<nblk(N, 256), 256, 0, st>>>(s, lim, (unsigned int*)((char*)w.gstat + 8),
                                             (unsigned int*)((char*)w.gstat + 24), (unsigned int*)((char*)w.gstat + 36));
    unsigned int mb[10] = {};
    RKCHK(cudaMemcpyAsync(mb, (char*)w.gstat + 8, 40, cudaMemcpyDeviceToHost, st));
    RKCHK(cudaStreamSynchronize(st));
    std::memcpy(&cell, &mb[0], 4);
    for (int a = 0; a < 3; a++) {
      clo[a] = float_of_ord(mb[4 + a]);
      chi[a] = float_of_ord(mb[7 + a]);
    }
    cell *= 1.01f;
    c.kernels += 2;
    if (!(cell > 0.f)) use_grid = false;
  }
  if (use_grid) {
    const float inv = 1.0f / cell;
    const CellFormat fmt = make_cell_format(s.scene_of != nullptr, inv, clo, chi);
    RKCHK(cudaMemsetAsync((char*)w.gstat + 16, 0, 8, st));
    RKCHK(cudaMemsetAsync(w.gis_over, 0, N, st));
    k_grid_keys<<<nblk(N, 256), 256, 0, st>>>(s, fmt, cell, inv, w.gkeys, w.gover,
                                              (unsigned long long*)((char*)w.gstat + 16));
    unsigned long long no_ = 0;
    RKCHK(cudaMemcpyAsync(&no_, (char*)w.gstat + 16, 8, cudaMemcpyDeviceToHost, st));
    RKCHK(cudaStreamSynchronize(st));
    nover = (int64_t)no_;
    if ((rc = ensure_tmp(c, (int64_t)sort_temp_bytes(N)))) return rc;
    radix_sort_u64(w.gkeys, w.gtmp, N, 21, 21 + fmt.total, w.tmp, st);
    if (nover > 0) k_mark_over<<<nblk(nover, 256), 256, 0, st>>>(w.gover, (int)nover, w.gis_over);
    c.kernels += 16;
    for (int attempt = 0; attempt < 4; attempt++) {
      RKCHK(cudaMemsetAsync(w.counter, 0, 8, st));
      k_grid_pairs<<<nblk(9 * kGridLanes * (N - nover), 128), 128, 0, st>>>(s, fmt, only, w.gkeys, N - nover,
                                                                             w.pairs, w.pair_cap, w.counter);
      if (nover > 0) {
        dim3 g2(nblk(N, 128), (unsigned)nover);
        k_over_pairs<<<g2, 128, 0, st>>>(s, only, w.gover, w.gis_over, w.pairs, w.pair_cap, w.counter);
      }
      c.kernels += 2;
      unsigned long long cnt = 0;
      RKCHK(cudaMemcpyAsync(&cnt, w.counter, 8, cudaMemcpyDeviceToHost, st));
      RKCHK(cudaStreamSynchronize(st));
      np = (int64_t)cnt;
      if (np <= w.pair_cap) break;
      int64_t nc = np + np / 2 + 1024;
      if ((rc = grow(c, w.pairs, w.pair_cap, nc))) return rc;
      w.pair_cap = nc;
      np = -1;
    }
  } else {
    for (int attempt = 0; attempt < 4; attempt++) {
      RKCHK(cudaMemsetAsync(w.counter, 0, 8, st));
      k_pairs<<<nblk(N, kPairTile), kPairTile, 0, st>>>(s, only, w.pairs, w.pair_cap, w.counter);
      c.kernels++;
      unsigned long long cnt = 0;
      RKCHK(cudaMemcpyAsync(&cnt, w.counter, 8, cudaMemcpyDeviceToHost, st));
      RKCHK(cudaStreamSynchronize(st));
      np = (int64_t)cnt;
      if (np <= w.pair_cap) break;
      int64_t nc = np + np / 2 + 1024;
      if ((rc = grow(c, w.pairs, w.pair_cap, nc))) return rc;
      w.pair_cap = nc;
      np = -1;
    }
  }
  if (np < 0) { c.err = "pair buffer kept overflowing"; return RK_ERR_CAPACITY; }
  if (defer) {  // the bodies of the visited pairs: world vertices and spheres
    if (w.mark_cap < N) {
      if ((rc = grow(c, w.gmark, w.mark_cap, N))) return rc;
      w.mark_cap = N;
    }
    RKCHK(cudaMemsetAsync(w.gmark, 0, (size_t)N, st));
    if (np > 0) k_mark_pair_bodies<<<nblk(np, 256), 256, 0, st>>>(w.pairs, np, w.gmark);
    c.kernels += 1 + launch_glob_vertices(s, st, true, w.gmark);
    if (nsph > 0) k_spheres<<<nblk(nsph, 256), 256, 0, st>>>(s, nsph, w.gmark);
    c.kernels++;
  }
  c.last_cell = cell;
  c.last_nover = nover;
  if (use_grid && !reuse_grid) {
    for (int a = 0; a < 3; a++) {
      c.grid_lo[a] = clo[a];
      c.grid_hi[a] = chi[a];
    }
    c.grid_n = N;
  }
  if (w.timing_split && w.split) RKCHK(cudaEventRecord(w.split, st));
  const int64_t nhp = 2 * np;
  if (w.hp_cap < nhp + 1) {
    int64_t nc = nhp + nhp / 2 + 1024;
    if ((rc = grow(c, w.hp, w.hp_cap, nc))) return rc;
    if ((rc = grow(c, w.hp_tmp, w.hp_cap, nc))) return rc;
    if ((rc = grow(c, w.hp_mask, w.hp_cap, kMaskWords * nc))) return rc;
    w.hp_cap = nc;
  }
  const EntryBuf& ob = c.eb[c.cur];
  const int64_t no = s.ne;
  int64_t need_tmp = (int64_t)std::max(sort_temp_bytes(nhp), scan_temp_bytes(no + 1));
  if ((rc = ensure_tmp(c, need_tmp))) return rc;
  if (np > 0) {
    k_half_pairs<<<nblk(np, 256), 256, 0, st>>>(w.pairs, np, w.hp);
    c.kernels++;
    radix_sort_u64(w.hp, w.hp_tmp, nhp, 0, 21 + body_bits(N), w.tmp, st);  // (owner << 21) | partner
    c.kernels += 13;
  }
  // ---- candidates: appended by one warp per half-pair, then sorted by key
  int64_t ncand = 0;
  if (nhp > 0) {
    const int64_t want = std::max<int64_t>(w.cand_hint, 4 * nhp) + 1024;
    if (w.cand_cap < want) {
      int64_t nc = want + want / 4;
      if ((rc = grow(c, w.cand, w.cand_cap, nc)) || (rc = grow(c, w.cand_tmp, w.cand_cap, nc))) return rc;
      w.cand_cap = nc;
    }
    const unsigned grid = (unsigned)std::min<int64_t>((nhp + kCandWarps - 1) / kCandWarps, 152 * 16);
    for (int attempt = 0; attempt < 4; attempt++) {
      RKCHK(cudaMemsetAsync(w.counter + 3, 0, 8, st));
      if (s.near_geometric)
        k_candidates<true><<<grid, 32 * kCandWarps, 0, st>>>(s, w.hp, nhp, w.hp_mask, w.cand, w.cand_cap, w.counter + 3);
      else
        k_candidates<false><<<grid, 32 * kCandWarps, 0, st>>>(s, w.hp, nhp, w.hp_mask, w.cand, w.cand_cap,
                                                              w.counter + 3);
      c.kernels++;
      unsigned long long cnt = 0;
      RKCHK(cudaMemcpyAsync(&cnt, w.counter + 3, 8, cudaMemcpyDeviceToHost, st));
      RKCHK(cudaStreamSynchronize(st));
      ncand = (int64_t)cnt;
      if (ncand <= w.cand_cap) break;
      int64_t nc = ncand + ncand / 4 + 1024;
      if ((rc = grow(c, w.cand, w.cand_cap, nc)) || (rc = grow(c, w.cand_tmp, w.cand_cap, nc))) return rc;
      w.cand_cap = nc;
      ncand = -1;
    }
    if (ncand < 0) { c.err = "candidate buffer kept overflowing"; return RK_ERR_CAPACITY; }
    w.cand_hint = ncand + ncand / 8;
    if (ncand > 1) {
      if ((rc = ensure_tmp(c, (int64_t)sort_temp_bytes(ncand)))) return rc;
      // A stable sort by (owner, partner) alone orders the keys completely:
      // one warp appends a half-pair's candidates, in its sweeps' order
      // (vertex-vertex, vertex-edge, vertex-face, edge-edge, each by
      // ascending sub-element indices, i.e. by ascending key), chunk after
      // chunk with increasing atomically reserved offsets.
      radix_sort_u64(w.cand, w.cand_tmp, ncand, 22, 43 + body_bits(N), w.tmp, st);
      c.kernels += 25;
    }
  }
  // ---- old entries kept untouched
  if (w.old_cap < no + 1) {
    int64_t nc = no + no / 2 + 1024;
    if ((rc = grow(c, w.flag, w.old_cap, nc + 1))) return rc;
    if ((rc = grow(c, w.stale, w.old_cap, nc))) return rc;
    if ((rc = grow(c, w.stale_src, w.old_cap, nc))) return rc;
    w.old_cap = nc;
  }
  int64_t nstale = 0;
  if (no > 0) {
    k_stale_flag<<<nblk(no, 256), 256, 0, st>>>(ob.ekey, no, w.hp, nhp, w.hp_mask, w.flag);
    RKCHK(cudaMemsetAsync(w.flag + no, 0, sizeof(int64_t), st));
    // positions in place of the flags, keeping a copy of the flags in stale_src
    RKCHK(cudaMemcpyAsync(w.stale_src, w.flag, (size_t)no * sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    exclusive_scan_i64(w.flag, w.flag, no + 1, w.tmp, st);
    c.kernels += 3;
    nstale = read_i64(c, w.flag + no);
  }
  // compact (flags copied to stale_src: use a separate pass into stale / cand_src)
  if (w.fin_cap < nstale + ncand + 1) {
    int64_t nc = nstale + ncand + (nstale + ncand) / 2 + 1024;
    if ((rc = grow(c, w.fkey, w.fin_cap, nc))) return rc;
    if ((rc = grow(c, w.fsrc, w.fin_cap, nc))) return rc;
    if ((rc = grow(c, w.jkeys, w.fin_cap, nc))) return rc;
    if ((rc = grow(c, w.jtmp, w.fin_cap, nc))) return rc;
    w.fin_cap = nc;
  }
  if (no > 0) {
    // fsrc doubles as the compacted old-index buffer before the merge
    k_stale_write<<<nblk(no, 256), 256, 0, st>>>(ob.ekey, no, w.stale_src, w.flag, w.stale, w.fsrc);
    c.kernels++;
    RKCHK(cudaMemcpyAsync(w.stale_src, w.fsrc, (size_t)std::max<int64_t>(nstale, 1) * sizeof(int64_t),
                          cudaMemcpyDeviceToDevice, st));
  }
  const int64_t nf = nstale + ncand;
  if ((rc = ensure_entry_capacity(c, 1 - c.cur, nf))) return rc;
  if (nf > 0) {
    k_merge<<<nblk(nf, 256), 256, 0, st>>>(w.stale, w.stale_src, nstale, w.cand, ncand, ob.ekey, no, w.fkey, w.fsrc);
    k_fill<<<nblk(nf, 256), 256, 0, st>>>(s, nf, w.fkey, w.fsrc, c.eb[c.cur], c.eb[1 - c.cur]);
    c.kernels += 2;
  }
  c.cur = 1 - c.cur;
  s.ne = nf;
  bind_entries(c);
  // ---- index structures
  need_tmp = (int64_t)sort_temp_bytes(nf);
  if ((rc = ensure_tmp(c, need_tmp))) return rc;
  k_iofs<<<nblk(N + 1, 256), 256, 0, st>>>(s.ekey, nf, N, s.iofs);
  c.kernels++;
  if (nf > 0) {
    k_jkeys<<<nblk(nf, 256), 256, 0, st>>>(s.ej, nf, w.jkeys);
    radix_sort_u64(w.jkeys, w.jtmp, nf, 27, 51, w.tmp, st);
    k_jlist<<<nblk(nf, 256), 256, 0, st>>>(w.jkeys, nf, s.jlist);
    c.kernels += 11;
  }
  k_jofs<<<nblk(N + 1, 256), 256, 0, st>>>(w.jkeys, nf, N, s.jofs);
  c.kernels++;
  RKCHK(cudaGetLastError());
  return heavy_list(c);
}

__global__ void k_type_keys(const uint32_t* etsub, int64_t ne, uint64_t* keys) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  keys[e] = ((uint64_t)tsub_type(etsub[e]) << 40) | (uint64_t)e;
}
// perm, and the first position of each type in it (tofs[4] = ne)
__global__ void k_type_perm(const uint64_t* keys, int64_t ne, int* perm, unsigned long long* tofs) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ne) return;
  perm[k] = (int)(keys[k] & ((1ull << 40) - 1));
  const int t = (int)(keys[k] >> 40), tp = k > 0 ? (int)(keys[k - 1] >> 40) : -1;
  for (int u = tp + 1; u <= t; u++) tofs[u] = (unsigned long long)k;
  if (k == ne - 1)
    for (int u = t + 1; u <= 4; u++) tofs[u] = (unsigned long long)ne;
}

// Order in which the narrow phase visits the entries: by sub-contact type,
// entry order within a type (after the index build; uses its scratch).
static int entry_order(Ctx& c) {
  Scene& s = c.s;
  NLWork& w = c.w;
  const int64_t ne = s.ne;
  if (ne <= 0) return 0;
  if (w.fin_cap < ne || w.tmp_bytes < (int64_t)sort_temp_bytes(ne)) {
    c.err = "entry order: scratch smaller than the neighbour list";
    return RK_ERR_STATE;
  }
  k_type_keys<<<nblk(ne, 256), 256, 0, c.stream>>>(s.etsub, ne, w.jkeys);
  radix_sort_u64(w.jkeys, w.jtmp, ne, 40, 42, w.tmp, c.stream);
  k_type_perm<<<nblk(ne, 256), 256, 0, c.stream>>>(w.jkeys, ne, s.nperm, s.flags + FLAG_TOFS);
  c.kernels += 5;
  return 0;
}

// Global vertex indices of each entry's sub-elements (see Scene::egv): the
// mixed narrow phase loads its vertices without the shape tables' chain of
// dependent loads.
__global__ void k_entry_gv(Scene s) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.ne) return;
  const int i = s.ei[e], j = s.ej[e];
  const uint32_t ts = s.etsub[e];
  const int type = tsub_type(ts), isub = tsub_isub(ts), jsub = tsub_jsub(ts);
  const int oi = (int)s.gv_ofs[i], oj = (int)s.gv_ofs[j];
  int4 g = make_int4(-1, -1, -1, -1);
  if (type == 0) {
    g = make_int4(oi + isub, oj + jsub, -1, -1);
  } else if (type == 1) {
    const int eo = s.edge_ofs[s.shape[j]] + jsub;
    g = make_int4(oi + isub, oj + s.edges[2 * eo], oj + s.edges[2 * eo + 1], -1);
  } else if (type == 2) {
    const int fo = s.face_ofs[s.shape[j]] + jsub;
    const int v0 = s.face_vofs[fo], nbv = s.face_vofs[fo + 1] - v0;
    const int* fv = s.face_verts + v0;
    g = nbv == 3 ? make_int4(oi + isub, oj + fv[0], oj + fv[1], oj + fv[2]) : make_int4(oi + isub, -1, -1, -1);
  } else {
    const int eoi = s.edge_ofs[s.shape[i]] + isub, eoj = s.edge_ofs[s.shape[j]] + jsub;
    g = make_int4(oi + s.edges[2 * eoi], oi + s.edges[2 * eoi + 1], oj + s.edges[2 * eoj], oj + s.edges[2 * eoj + 1]);
  }
  s.egv[e] = g;
}

int heavy_list(Ctx& c) {
  Scene& s = c.s;
  {
    const int rc = entry_order(c);
    if (rc) return rc;
  }
  s.egv_ok = 0;
  if (s.ne > 0 && s.nvert < (int64_t)0x7fffffff) {
    k_entry_gv<<<nblk(s.ne, 256), 256, 0, c.stream>>>(s);
    c.kernels++;
    s.egv_ok = 1;
  }
  // counter slots 1, 2: heavy bodies, deferred heavy bodies; 4: listed vertices
  RKCHK(cudaMemsetAsync(c.w.counter + 1, 0, 32, c.stream));
  k_heavy<<<nblk(s.n, 256), 256, 0, c.stream>>>(s, c.w.counter + 1);
  c.kernels++;
  unsigned long long nh[4] = {0, 0, 0, 0};
  RKCHK(cudaMemcpyAsync(nh, c.w.counter + 1, 32, cudaMemcpyDeviceToHost, c.stream));
  RKCHK(cudaStreamSynchronize(c.stream));
  s.nheavy = (int)nh[0];
  s.nheavy_lazy = (int)nh[1];
  s.nlv = (int64_t)nh[3];
  return 0;
}

}  // namespace rk
