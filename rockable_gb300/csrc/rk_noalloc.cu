// rk_noalloc.cu -- rk_sort_keys_noalloc: the neighbour-list key sort for
// callers that cannot allocate device memory.
//
// rk_sort_keys allocates two temporary buffers with cudaMalloc on every call
// and frees them afterwards.  Some callers cannot accept that: a host whose
// device memory is already held by its own caching allocator (cudaMalloc
// then fails with out-of-memory although the memory is only reserved, not in
// use), a serving loop that must run with a memory footprint fixed at start-up
// and cannot meet an out-of-memory error halfway through a step, and code that
// shares the device with other streams and cannot afford the device-wide
// synchronisation that cudaFree implies.  This variant runs the same radix-sort
// passes on a scratch array that lives in this file for the life of the
// process, and calls no allocating routine.
//
// The scratch is one file-scope __device__ array (kScratchBytes, about
// 4.5 MB), present on every GPU that loads the library until the process
// exits.  It bounds the problem size: at most kNoAllocMaxKeys keys per call;
// larger calls return RK_ERR_CAPACITY and touch nothing.  Every call uses the
// whole array, so calls that overlap on the GPU (two streams, or two host
// threads on one device) overwrite each other's data: the caller must order
// them.  Calls in sequence share the array, which keeps what the last call
// left; no part of it has to start at zero, because each radix pass writes
// its histogram, offsets and output keys before reading them.
//
// The first call on each device does a one-time set-up: it looks up the
// device address of the array (cudaGetSymbolAddress) with that device current.
// Make that first call before any stream capture begins.  The address is kept
// for the life of the process: do not use the entry point on a device after
// cudaDeviceReset (or anything else that tears down and recreates its primary
// context), since the module, and with it the array, may then load elsewhere.
//
// Errors: the call returns RK_ERR_CUDA without sorting when a CUDA error is
// already pending on the calling thread (it leaves that error in place for
// its owner), and RK_ERR_CUDA when one of its own launches fails.
#include <cstdint>
#include <mutex>

#include "../../include/rk_gpu.h"
#include "rk_engine.cuh"

namespace rk {

constexpr int64_t kNoAllocMaxKeys = int64_t(1) << 19;                 // 524,288 keys
constexpr size_t kNoAllocKeyBytes = size_t(kNoAllocMaxKeys) * sizeof(uint64_t);
constexpr size_t kNoAllocTempBytes = size_t(512) << 10;              // histograms + scan partials
constexpr size_t kScratchBytes = kNoAllocKeyBytes + kNoAllocTempBytes;

// The scratch itself.  In host code this name is only a stand-in for the
// device symbol: host code never uses it as a device address, it asks the
// runtime for the address (scratch_address below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch on the current device, looked up once per
// device (a symbol lookup: nothing is allocated).
static int scratch_address(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RK_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return RK_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return RK_OK;
}

}  // namespace rk

extern "C" int rk_sort_keys_noalloc(uint64_t* keys, int64_t n, int lo_bit, int hi_bit, void* stream) {
  using namespace rk;
  if (n < 0 || (n > 0 && !keys) || lo_bit < 0 || hi_bit > 64 || lo_bit >= hi_bit) return RK_ERR_ARG;
  if (n > kNoAllocMaxKeys) return RK_ERR_CAPACITY;  // larger than the fixed scratch
  if (sort_temp_bytes(n) > kNoAllocTempBytes) return RK_ERR_CAPACITY;
  if (cudaPeekAtLastError() != cudaSuccess) return RK_ERR_CUDA;  // an earlier error, not ours to clear
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);  // first call on a device: the one-time lookup
  if (rc != RK_OK) return rc;
  if (n <= 1) return RK_OK;
  uint64_t* tmp = reinterpret_cast<uint64_t*>(base);
  void* temp = base + kNoAllocKeyBytes;
  radix_sort_u64(keys, tmp, n, lo_bit, hi_bit, temp, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? RK_OK : RK_ERR_CUDA;  // nothing was pending before: any error is ours
}
