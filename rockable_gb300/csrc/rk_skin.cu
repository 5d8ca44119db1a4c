// rk_skin.cu -- learned Verlet skin: exact displacement guard and the small
// MLP (16 -> 64 -> 64 -> 2) that proposes the skin and the rebuild interval.
//
// No reference counterpart: Rockable uses a fixed interVerlet and DVerlet /
// dVerlet, or its dynamic guard on centre displacement and angle
// (Rockable.cpp:1571-1596).  Here the guard is exact: the motion of any point
// of body b since the last rebuild is bounded by
//     delta_b = |x_b - x_b0| + theta_b * rsw_b
// (theta_b a bound of the rotation angle between Q_b0 and Q_b, rsw_b the
// largest vertex distance from the centre).  Two sub-elements can only have come closer by
// delta_i + delta_j, so while max_b delta_b < dVerlet / 2 every sub-contact
// that was not NEAR at the rebuild is still separated, and a refresh is
// forced as soon as the bound reaches dVerlet / 2.
//
// The MLP runs in FP16 storage with FP32 accumulation, trained by one CTA
// (batch <= 128 windows) with Adam on FP32 master weights.
#include <cuda_fp16.h>

#include "../../include/rk_gpu.h"
#include "rk_engine.cuh"
#include "rk_guard.cuh"

namespace rk {

// ---------------------------------------------------------------- guard ----
// Partial refresh: when only a few bodies have used up their budget, only
// their pairs are refreshed (the neighbour-list rebuild restricted to pairs
// with at least one flagged body) and only their snapshots are reset.  A
// pair (i, j) is then last tested at T_ij = the later of the two bodies'
// last refreshes, and the motion of i since T_ij is no longer bounded by
// delta_i (measured from i's own refresh, possibly earlier).  Two monotone
// bounds still hold for any T_ij after i's refresh:
//   path_i   = the accumulated per-step motion (drift kernel), and
//   2 maxd_i = twice the largest delta_i seen since i's refresh
// (|x(now) - x(T)| <= delta(now) + delta(T)).  So once a partial refresh has
// happened, g_b = min(path_b, 2 maxd_b) < dVerlet / 2 for every body keeps
// every missed sub-contact separated; before it, max delta_b suffices.
// Histogram of delta_b over the bodies in quarter-octave bins of
// log2(delta / unit), bins 0..63 covering 2^-14 .. 2^2 units (the skin's
// displacement-rate percentile at a full rebuild).
__global__ void k_skin_hist(Scene s, const double* ref_pos, const double* ref_q, const float* rsw, float unit,
                            unsigned int* hist) {
  __shared__ unsigned int h[64];
  if (threadIdx.x < 64) h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < s.n) {
    const double dx = s.pos[3 * b] - ref_pos[3 * b], dy = s.pos[3 * b + 1] - ref_pos[3 * b + 1],
                 dz = s.pos[3 * b + 2] - ref_pos[3 * b + 2];
    const float delta =
        (float)(sqrt(dx * dx + dy * dy + dz * dz) + rot_bound(s.Q + 4 * b, ref_q + 4 * b) * (double)rsw[b]);
    int bin = 0;
    if (delta > 0.f) bin = (int)floorf(4.f * (log2f(delta / unit) + 14.f));
    bin = min(max(bin, 0), 63);
    atomicAdd(&h[bin], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 64 && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

int launch_skin_hist(const Scene& s, const double* rp, const double* rq, const float* rsw, float unit,
                     unsigned int* hist, cudaStream_t st) {
  k_skin_hist<<<(unsigned)((s.n + 255) / 256), 256, 0, st>>>(s, rp, rq, rsw, unit, hist);
  return 1;
}

__global__ void k_skin_reset(Scene s, const uint8_t* only, double* ref_pos, double* ref_q, float* maxd, float* path) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= s.n) return;
  if (only && !only[b]) return;
  for (int d = 0; d < 3; d++) ref_pos[3 * b + d] = s.pos[3 * b + d];
  for (int d = 0; d < 4; d++) ref_q[4 * b + d] = s.Q[4 * b + d];
  maxd[b] = 0.f;
  path[b] = 0.f;
}

int launch_skin_reset(const Scene& s, const uint8_t* only, double* rp, double* rq, float* maxd, float* path,
                      cudaStream_t st) {
  k_skin_reset<<<(unsigned)((s.n + 255) / 256), 256, 0, st>>>(s, only, rp, rq, maxd, path);
  return 1;
}

// ------------------------------------------------------ batched steps ----
// A batch of steps runs as one graph without a host round trip per step:
// k_skin_begin opens the batch, and the last block of each step's resultant
// kernel reads the exact guard the kernel just reduced (skin_batch_step_end,
// rk_guard.cuh) and halts the rest of the batch when the host has to act (a
// refresh is due, or the batch's step budget is spent); a halted step's
// kernels return at once.  Control block sk_ctl (words, set by the host
// before the batch):
//   [0] halt  [1] steps executed  [2] steps since the last refresh
//   [3] step budget  [4] refresh interval (steps)  [5] trigger (float bits,
//   the smallest float >= skin/2)  [6] 1: the trigger compares the path bound
//   g, 0: the displacement bound delta  [7] arrival ticket of the resultant
//   kernel's blocks  [8..15] guard words of the last executed step (the
//   layout of sk_out).
__global__ void k_skin_begin(Scene s) {
  if (step_halted(s)) return;
  const int t = threadIdx.x;
  if (t == 0) s.flags[FLAG_NACTIVE] = 0ull;
  if (t < 8) s.sk_out[t] = 0u;
}

int launch_skin_begin(const Scene& s, cudaStream_t st) {
  k_skin_begin<<<1, 32, 0, st>>>(s);
  return 1;
}

// ------------------------------------------------------------------ MLP ----
// Parameter layout (floats): W1[64][16] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
constexpr int kIn = 16, kH = 64, kOut = 2;
constexpr int kW1 = 0, kB1 = kW1 + kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kOut * kH, kNP = kB3 + kOut;

int mlp_num_params() { return kNP; }

// forward of one sample by one thread group; x in registers, weights as half
__device__ __forceinline__ float hw(const __half* w, int k) { return __half2float(w[k]); }

// Inference: one sample, 64 threads.
__global__ void k_mlp_infer(const __half* w, const float* x, float* y) {
  __shared__ float h1[kH], h2[kH], xs[kIn];
  const int t = threadIdx.x;
  if (t < kIn) xs[t] = __half2float(__float2half(x[t]));
  __syncthreads();
  float a = hw(w, kB1 + t);
  for (int k = 0; k < kIn; k++) a += hw(w, kW1 + t * kIn + k) * xs[k];
  h1[t] = __half2float(__float2half(fmaxf(a, 0.f)));
  __syncthreads();
  a = hw(w, kB2 + t);
  for (int k = 0; k < kH; k++) a += hw(w, kW2 + t * kH + k) * h1[k];
  h2[t] = __half2float(__float2half(fmaxf(a, 0.f)));
  __syncthreads();
  if (t < kOut) {
    a = hw(w, kB3 + t);
    for (int k = 0; k < kH; k++) a += hw(w, kW3 + t * kH + k) * h2[k];
    y[t] = a;
  }
}

// One training step on a batch: forward (FP16 activations, FP32 accumulate),
// MSE loss gradient, backward, gradient averaged over the batch in FP32.
// grad[] receives the gradient (kNP floats); loss[0] the mean loss.
// 256 threads; batch <= 128.
constexpr int kMaxBatch = 128;
__global__ void __launch_bounds__(256) k_mlp_grad(const __half* w, const float* X, const float* T, int nb,
                                                  float* grad, float* loss) {
  extern __shared__ float sm[];
  float* xs = sm;                       // nb*kIn
  float* h1 = xs + kMaxBatch * kIn;     // nb*kH (post-ReLU, rounded to half)
  float* h2 = h1 + kMaxBatch * kH;      // nb*kH
  float* d2 = h2 + kMaxBatch * kH;      // nb*kH  dL/d(pre-activation 2)
  float* d1 = d2 + kMaxBatch * kH;      // nb*kH  dL/d(pre-activation 1)
  float* dy = d1 + kMaxBatch * kH;      // nb*kOut
  const int t = threadIdx.x, nt = blockDim.x;
  for (int k = t; k < nb * kIn; k += nt) xs[k] = __half2float(__float2half(X[k]));
  __syncthreads();
  for (int k = t; k < nb * kH; k += nt) {
    int s = k / kH, u = k % kH;
    float a = hw(w, kB1 + u);
    for (int q = 0; q < kIn; q++) a += hw(w, kW1 + u * kIn + q) * xs[s * kIn + q];
    h1[k] = __half2float(__float2half(fmaxf(a, 0.f)));
  }
  __syncthreads();
  for (int k = t; k < nb * kH; k += nt) {
    int s = k / kH, u = k % kH;
    float a = hw(w, kB2 + u);
    for (int q = 0; q < kH; q++) a += hw(w, kW2 + u * kH + q) * h1[s * kH + q];
    h2[k] = __half2float(__float2half(fmaxf(a, 0.f)));
  }
  __syncthreads();
  __shared__ float lsum;
  if (t == 0) lsum = 0.f;
  __syncthreads();
  for (int k = t; k < nb * kOut; k += nt) {
    int s = k / kOut, o = k % kOut;
    float a = hw(w, kB3 + o);
    for (int q = 0; q < kH; q++) a += hw(w, kW3 + o * kH + q) * h2[s * kH + q];
    float r = a - T[k];
    dy[k] = 2.f * r / (float)(nb * kOut);
    atomicAdd(&lsum, r * r);
  }
  __syncthreads();
  if (t == 0) loss[0] = lsum / (float)(nb * kOut);
  // dL/d pre2 = (W3^T dy) * relu'(pre2)
  for (int k = t; k < nb * kH; k += nt) {
    int s = k / kH, u = k % kH;
    float a = 0.f;
    for (int o = 0; o < kOut; o++) a += hw(w, kW3 + o * kH + u) * dy[s * kOut + o];
    d2[k] = h2[k] > 0.f ? a : 0.f;
  }
  __syncthreads();
  for (int k = t; k < nb * kH; k += nt) {
    int s = k / kH, u = k % kH;
    float a = 0.f;
    for (int v = 0; v < kH; v++) a += hw(w, kW2 + v * kH + u) * d2[s * kH + v];
    d1[k] = h1[k] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // parameter gradients, summed over the batch in FP32
  for (int p = t; p < kNP; p += nt) {
    float g = 0.f;
    if (p < kB1) {
      int u = p / kIn, q = p % kIn;
      for (int s = 0; s < nb; s++) g += d1[s * kH + u] * xs[s * kIn + q];
    } else if (p < kW2) {
      int u = p - kB1;
      for (int s = 0; s < nb; s++) g += d1[s * kH + u];
    } else if (p < kB2) {
      int u = (p - kW2) / kH, q = (p - kW2) % kH;
      for (int s = 0; s < nb; s++) g += d2[s * kH + u] * h1[s * kH + q];
    } else if (p < kW3) {
      int u = p - kB2;
      for (int s = 0; s < nb; s++) g += d2[s * kH + u];
    } else if (p < kB3) {
      int o = (p - kW3) / kH, q = (p - kW3) % kH;
      for (int s = 0; s < nb; s++) g += dy[s * kOut + o] * h2[s * kH + q];
    } else {
      int o = p - kB3;
      for (int s = 0; s < nb; s++) g += dy[s * kOut + o];
    }
    grad[p] = g;
  }
}

// Adam on FP32 master weights, refreshed FP16 copy.
__global__ void k_mlp_adam(float* master, __half* w, float* m, float* v, const float* grad, float lr, float b1,
                           float b2, float eps, int step) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNP) return;
  float g = grad[p];
  m[p] = b1 * m[p] + (1.f - b1) * g;
  v[p] = b2 * v[p] + (1.f - b2) * g * g;
  float mh = m[p] / (1.f - powf(b1, (float)step));
  float vh = v[p] / (1.f - powf(b2, (float)step));
  master[p] -= lr * mh / (sqrtf(vh) + eps);
  w[p] = __float2half(master[p]);
}

__global__ void k_mlp_to_half(const float* master, __half* w) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kNP) w[p] = __float2half(master[p]);
}

size_t mlp_grad_smem() { return (size_t)(kMaxBatch * kIn + 4 * kMaxBatch * kH + kMaxBatch * kOut) * sizeof(float); }
int mlp_max_batch() { return kMaxBatch; }

void launch_mlp_infer(const void* w, const float* x, float* y, cudaStream_t st) {
  k_mlp_infer<<<1, kH, 0, st>>>((const __half*)w, x, y);
}
void launch_mlp_grad(const void* w, const float* X, const float* T, int nb, float* grad, float* loss,
                     cudaStream_t st) {
  // the attribute belongs to the current device's context: set it before
  // every launch (a few host instructions), so a context on any device has it
  cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_grad_smem());
  k_mlp_grad<<<1, 256, mlp_grad_smem(), st>>>((const __half*)w, X, T, nb, grad, loss);
}
void launch_mlp_adam(float* master, void* w, float* m, float* v, const float* grad, float lr, int step,
                     cudaStream_t st) {
  k_mlp_adam<<<(kNP + 255) / 256, 256, 0, st>>>(master, (__half*)w, m, v, grad, lr, 0.9f, 0.999f, 1e-8f, step);
}
void launch_mlp_to_half(const float* master, void* w, cudaStream_t st) {
  k_mlp_to_half<<<(kNP + 255) / 256, 256, 0, st>>>(master, (__half*)w);
}

}  // namespace rk
