// rk_prims.cu -- device-wide primitives used by the neighbour-list rebuild:
// exclusive prefix sum of int64 counts and a stable LSD radix sort of 64-bit
// keys (8 bits per pass, block-local stable ranking with warp match masks).
#include <cstdint>

#include "rk_engine.cuh"

namespace rk {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

static inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

__device__ __forceinline__ int64_t warp_incl_scan(int64_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__global__ void k_tile_sums(const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  __shared__ int64_t ws[32];
  const int64_t base = blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int64_t idx = base + k;
    if (idx < n) t += in[idx];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x < 32) {
    int64_t v = ws[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = v;
  }
}

__global__ void k_tile_scan(const int64_t* in, int64_t* out, int64_t n, const int64_t* __restrict__ block_ofs) {
  __shared__ int64_t ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int64_t idx = base + k;
    v[k] = idx < n ? in[idx] : 0;
    t += v[k];
  }
  int64_t x = warp_incl_scan(t);
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = ws[lane];
    w = warp_incl_scan(w);
    ws[lane] = w;
  }
  __syncthreads();
  int64_t excl = x - t + (warp > 0 ? ws[warp - 1] : 0) + (block_ofs ? block_ofs[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int64_t idx = base + k;
    if (idx < n) out[idx] = excl;
    excl += v[k];
  }
}

size_t scan_temp_bytes(int64_t n) {
  size_t total = 0;
  while (n > kScanTile) {
    int64_t nb = cdiv(n, kScanTile);
    total += (size_t)nb * sizeof(int64_t);
    n = nb;
  }
  return total + 256;
}

// out[k] = sum_{m<k} in[m]; in and out may alias.
void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* temp, cudaStream_t st) {
  if (n <= 0) return;
  if (n <= kScanTile) {
    k_tile_scan<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
    return;
  }
  int64_t nb = cdiv(n, kScanTile);
  int64_t* sums = (int64_t*)temp;
  void* rest = (void*)(sums + nb);
  k_tile_sums<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, sums);
  exclusive_scan_i64(sums, sums, nb, rest, st);
  k_tile_scan<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, sums);
}

// ------------------------------------------------------------ radix sort ----
constexpr int kSortThreads = 256;
constexpr int kSortChunks = 16;
constexpr int64_t kSortTile = (int64_t)kSortThreads * kSortChunks;

// One pass of the LSD radix sort on the digit (key >> sh) & mask: 8 bits,
// fewer in the last pass when hi_bit - lo_bit is not a multiple of 8 (the
// bits at and above hi_bit must not take part in the order).
__global__ void k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int sh, unsigned mask, int64_t nblocks,
                             int64_t* __restrict__ hist) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = blockIdx.x * kSortTile;
  for (int c = 0; c < kSortChunks; c++) {
    int64_t idx = base + (int64_t)c * kSortThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(unsigned)((keys[idx] >> sh) & mask)], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_radix_scatter(const uint64_t* __restrict__ keys, uint64_t* __restrict__ out, int64_t n, int sh,
                                unsigned mask, int64_t nblocks, const int64_t* __restrict__ ofs) {
  __shared__ unsigned run[256];
  __shared__ unsigned wcnt[kSortThreads / 32][256];
  __shared__ int64_t base_ofs[256];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  run[t] = 0;
  base_ofs[t] = ofs[(int64_t)t * nblocks + blockIdx.x];
  const unsigned lt = (1u << lane) - 1u;
  const int64_t tile = blockIdx.x * kSortTile;
  for (int c = 0; c < kSortChunks; c++) {
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; w++) wcnt[w][t] = 0;
    __syncthreads();
    const int64_t idx = tile + (int64_t)c * kSortThreads + t;
    const bool valid = idx < n;
    const uint64_t key = valid ? keys[idx] : 0ull;
    const unsigned d = valid ? (unsigned)((key >> sh) & mask) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lt);
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      unsigned before = 0;
      for (int w = 0; w < warp; w++) before += wcnt[w][d];
      out[base_ofs[d] + run[d] + before + rank] = key;
    }
    __syncthreads();
    unsigned tot = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; w++) tot += wcnt[w][t];
    run[t] += tot;
    __syncthreads();
  }
}

size_t sort_temp_bytes(int64_t n) {
  int64_t nb = cdiv(n > 0 ? n : 1, kSortTile);
  int64_t h = 256 * nb;
  return (size_t)h * sizeof(int64_t) + scan_temp_bytes(h) + 256;
}

// Stable sort of keys on bits [lo_bit, hi_bit); tmp has n slots.  The
// result ends in keys.
void radix_sort_u64(uint64_t* keys, uint64_t* tmp, int64_t n, int lo_bit, int hi_bit, void* temp,
                    cudaStream_t st) {
  if (n <= 1) return;
  const int64_t nb = cdiv(n, kSortTile);
  int64_t* hist = (int64_t*)temp;
  void* scan_tmp = (void*)(hist + 256 * nb);
  uint64_t* src = keys;
  uint64_t* dst = tmp;
  int passes = 0;
  for (int sh = lo_bit; sh < hi_bit; sh += 8) {
    const unsigned mask = (1u << (hi_bit - sh < 8 ? hi_bit - sh : 8)) - 1u;
    k_radix_hist<<<(unsigned)nb, kSortThreads, 0, st>>>(src, n, sh, mask, nb, hist);
    exclusive_scan_i64(hist, hist, 256 * nb, scan_tmp, st);
    k_radix_scatter<<<(unsigned)nb, kSortThreads, 0, st>>>(src, dst, n, sh, mask, nb, hist);
    uint64_t* x = src;
    src = dst;
    dst = x;
    passes++;
  }
  if (passes & 1) cudaMemcpyAsync(keys, src, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
}

}  // namespace rk
