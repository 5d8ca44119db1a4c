// rk_fast.cu -- the per-body kernels of rk_body.cuh compiled with fused
// multiply-adds allowed, for the mixed form (see rk_body.cuh).
#include "../../include/rk_gpu.h"
#include "rk_engine.cuh"
#include "rk_guard.cuh"
#define RK_BODY_NS fused
#include "rk_body.cuh"

namespace rk {

int launch_fused_drift(const Scene& s, unsigned blocks, int threads, cudaStream_t st) {
  fused::k_drift<<<blocks, threads, 0, st>>>(s);
  return 1;
}
int launch_fused_glob(const Scene& s, unsigned blocks, int threads, int only_listed, cudaStream_t st) {
  fused::k_glob_vertices<<<blocks, threads, 0, st>>>(s, only_listed);
  return 1;
}
int launch_fused_gather(const Scene& s, unsigned blocks, int threads, int apply_kick, cudaStream_t st) {
  fused::k_gather_accel<<<blocks, threads, 0, st>>>(s, apply_kick);
  return 1;
}
cudaError_t fused_attributes(int which, cudaFuncAttributes* a) {
  if (which == 1) return cudaFuncGetAttributes(a, fused::k_gather_accel);
  if (which == 2) return cudaFuncGetAttributes(a, fused::k_glob_vertices);
  return cudaFuncGetAttributes(a, fused::k_drift);
}

}  // namespace rk
