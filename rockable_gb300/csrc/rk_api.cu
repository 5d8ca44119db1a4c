// rk_api.cu -- the C ABI of librk_gpu.so: context, uploads, the step loop
// (Rockable::integrate bookkeeping around rk::velocity-Verlet kernels) and
// downloads.  See include/rk_gpu.h for the reference seams each call replaces.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rk_conf.cuh"
#include "rk_extract.cuh"
#include "rk_ctx.cuh"

using namespace rk;

struct rk_ctx {
  Ctx c;
};

namespace {

#define CK(x)                                                            \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) {                                             \
      c.err = std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #x; \
      return RK_ERR_CUDA;                                                \
    }                                                                    \
  } while (0)

template <typename T>
int dalloc(Ctx& c, T*& p, int64_t n) {
  if (p) cudaFree(p);
  p = nullptr;
  CK(cudaMalloc(&p, (size_t)std::max<int64_t>(n, 1) * sizeof(T)));
  return 0;
}
template <typename T>
int dupload(Ctx& c, T*& p, const T* h, int64_t n) {
  int rc = dalloc(c, p, n);
  if (rc) return rc;
  if (n > 0 && h) CK(cudaMemcpyAsync(p, h, (size_t)n * sizeof(T), cudaMemcpyHostToDevice, c.stream));
  else if (n > 0) CK(cudaMemsetAsync(p, 0, (size_t)n * sizeof(T), c.stream));
  return 0;
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

int fail(Ctx& c, int code, const std::string& msg) {
  c.err = msg;
  return code;
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

namespace rk {

void bind_entries(Ctx& c) {
  EntryBuf& b = c.eb[c.cur];
  Scene& s = c.s;
  s.ei = b.ei; s.ej = b.ej; s.etsub = b.etsub; s.ekey = b.ekey;
  s.dn = b.dn; s.fn = b.fn; s.ft = b.ft; s.mom = b.mom; s.damp = b.damp; s.bond = b.bond;
  s.gn = b.gn; s.gpos = b.gpos; s.gvel = b.gvel;
}

static void free_entrybuf(EntryBuf& b) {
  dfree(b.ei); dfree(b.ej); dfree(b.etsub); dfree(b.ekey); dfree(b.dn); dfree(b.fn); dfree(b.ft); dfree(b.mom);
  dfree(b.damp); dfree(b.bond); dfree(b.gn); dfree(b.gpos); dfree(b.gvel);
  b.cap = 0;
}

// Grow entry buffer `which` (and the single-buffered per-step arrays) to
// hold n entries; contents of a grown buffer are not preserved.
int ensure_entry_capacity(Ctx& c, int which, int64_t n) {
  EntryBuf& b = c.eb[which];
  int rc;
  if (b.cap < n || b.cap == 0) {
    int64_t cap = std::max<int64_t>(n + n / 2, 1024);
    free_entrybuf(b);
    if ((rc = dalloc(c, b.ei, cap)) || (rc = dalloc(c, b.ej, cap)) || (rc = dalloc(c, b.etsub, cap)) ||
        (rc = dalloc(c, b.ekey, cap)) || (rc = dalloc(c, b.dn, cap)) || (rc = dalloc(c, b.fn, cap)) ||
        (rc = dalloc(c, b.ft, 3 * cap)) || (rc = dalloc(c, b.mom, 3 * cap)) || (rc = dalloc(c, b.damp, cap)) ||
        (rc = dalloc(c, b.bond, cap)) || (rc = dalloc(c, b.gn, 3 * cap)) || (rc = dalloc(c, b.gpos, 3 * cap)) ||
        (rc = dalloc(c, b.gvel, 3 * cap)))
      return rc;
    b.cap = cap;
  }
  if (c.contrib_cap < n || c.contrib_cap == 0) {
    int64_t cap = std::max<int64_t>(n + n / 2, 1024);
    Scene& s = c.s;
    if ((rc = dalloc(c, s.act, cap)) || (rc = dalloc(c, s.cf, 3 * cap)) || (rc = dalloc(c, s.cmi, 3 * cap)) ||
        (rc = dalloc(c, s.cmj, 3 * cap)) || (rc = dalloc(c, s.jlist, cap)) || (rc = dalloc(c, s.nperm, cap)) ||
        (rc = dalloc(c, s.egv, cap)) || (rc = dalloc(c, s.slow, cap)))
      return rc;
    c.contrib_cap = cap;
  }
  return 0;
}

}  // namespace rk

namespace {

__global__ void k_upload_keys(Scene s, int64_t ne, const int* t, const int* isub, const int* jsub, int* bad) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int i = s.ei[e], j = s.ej[e];
  if (i < 0 || j < 0 || i >= s.n || j >= s.n || t[e] < 0 || t[e] > 3 || isub[e] < 0 || jsub[e] < 0 ||
      isub[e] >= kMaxSub || jsub[e] >= kMaxSub) {
    atomicExch(bad, 1);
    return;
  }
  s.etsub[e] = pack_tsub(t[e], isub[e], jsub[e]);
  s.ekey[e] = entry_key(i, j, t[e], isub[e], jsub[e]);
}

__global__ void k_check_sorted(const uint64_t* k, int64_t n, int* bad) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e + 1 >= n) return;
  if (!(k[e] < k[e + 1])) atomicExch(bad, 2);
}

__global__ void k_iofs2(const uint64_t* key, int64_t ne, int64_t nb, int64_t* iofs) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b > nb) return;
  int64_t lo = 0, hi = ne;
  uint64_t x = (uint64_t)b << 43;
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (key[m] < x) lo = m + 1;
    else hi = m;
  }
  iofs[b] = lo;
}
__global__ void k_jkeys2(const int* ej, int64_t ne, uint64_t* jk) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  jk[e] = ((uint64_t)ej[e] << 27) | (uint64_t)e;
}
__global__ void k_jlist2(const uint64_t* jk, int64_t ne, int* jlist) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  jlist[e] = (int)(jk[e] & ((1ull << 27) - 1));
}
__global__ void k_jofs2(const uint64_t* jk, int64_t ne, int64_t nb, int64_t* jofs) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b > nb) return;
  int64_t lo = 0, hi = ne;
  uint64_t x = (uint64_t)b << 27;
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (jk[m] < x) lo = m + 1;
    else hi = m;
  }
  jofs[b] = lo;
}

// i-side offsets and j-side list of the current entries (after an upload).
int build_index(Ctx& c) {
  Scene& s = c.s;
  NLWork& w = c.w;
  const int64_t ne = s.ne, N = s.n;
  if (w.fin_cap < ne + 1) {
    int64_t cap = ne + ne / 2 + 1024;
    dfree(w.jkeys);
    dfree(w.jtmp);
    dfree(w.fkey);
    dfree(w.fsrc);
    int rc;
    if ((rc = dalloc(c, w.jkeys, cap)) || (rc = dalloc(c, w.jtmp, cap)) || (rc = dalloc(c, w.fkey, cap)) ||
        (rc = dalloc(c, w.fsrc, cap)))
      return rc;
    w.fin_cap = cap;
  }
  int64_t need = (int64_t)sort_temp_bytes(ne);
  if (need > w.tmp_bytes) {
    dfree(w.tmp);
    int64_t nb = need + need / 2;
    CK(cudaMalloc(&w.tmp, (size_t)nb));
    w.tmp_bytes = nb;
  }
  k_iofs2<<<nblk(N + 1, 256), 256, 0, c.stream>>>(s.ekey, ne, N, s.iofs);
  if (ne > 0) {
    k_jkeys2<<<nblk(ne, 256), 256, 0, c.stream>>>(s.ej, ne, w.jkeys);
    radix_sort_u64(w.jkeys, w.jtmp, ne, 27, 51, w.tmp, c.stream);
    k_jlist2<<<nblk(ne, 256), 256, 0, c.stream>>>(w.jkeys, ne, s.jlist);
  }
  k_jofs2<<<nblk(N + 1, 256), 256, 0, c.stream>>>(w.jkeys, ne, N, s.jofs);
  CK(cudaGetLastError());
  return heavy_list(c);
}

int read_flags(Ctx& c) {
  CK(cudaMemcpyAsync(c.h_flags, c.s.flags, FLAG_COUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (c.h_flags[FLAG_ERROR]) {
    c.err = "mixed narrow phase: an entry's type run disagrees with the entry order (entries skipped)";
    return RK_ERR_STATE;
  }
  return 0;
}

}  // namespace


// Resultants of driven bodies that feed no state are summed on demand, from
// the contributions of the last narrow phase (before they are overwritten or
// re-ordered by a rebuild).
static void settle_lazy_forces(Ctx& c) {
  if (c.forces_stale) {
    c.kernels += launch_gather_heavy_lazy(c.s, c.stream);
    c.forces_stale = false;
  }
}

// Before a neighbour-list update inside rk_step: the deferred resultants
// must be summed from the current list only when no step of this call
// follows (a step recomputes every contribution of the new list, and the
// resultants it leaves are the ones a download must see).
static void settle_before_update(Ctx& c) {
  if (!c.more_steps_follow) settle_lazy_forces(c);
}

// ------------------------------------------------------------ learned skin ----
// Windows in the replay buffer before the network trains and predicts.  Its
// output layer starts at zero (it then predicts what the method without it
// does), so it can act from the first windows and departs from that method
// only as far as its training carries it.
static const int kMinWindows = 2;

static double to_f(unsigned int bits) {
  float f;
  std::memcpy(&f, &bits, 4);
  return (double)f;
}

static int skin_train(Ctx& c) {
  Skin& k = c.skin;
  const int nb = (int)std::min<size_t>(k.rx.size(), (size_t)mlp_max_batch());
  if (nb < kMinWindows) return 0;
  std::vector<float> X(16 * nb), T(2 * nb);
  for (int i = 0; i < nb; i++) {
    for (int q = 0; q < 16; q++) X[16 * i + q] = k.rx[i][q];
    T[2 * i] = k.ry[i][0];
    T[2 * i + 1] = k.ry[i][1];
  }
  CK(cudaMemcpyAsync(k.X, X.data(), X.size() * 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(k.T, T.data(), T.size() * 4, cudaMemcpyHostToDevice, c.stream));
  for (int it = 0; it < std::max(1, k.cfg.train_steps); it++) {
    launch_mlp_grad(k.w, k.X, k.T, nb, k.grad, k.loss, c.stream);
    launch_mlp_adam(k.master, k.w, k.m, k.v, k.grad, (float)k.cfg.learning_rate, ++k.adam_step, c.stream);
    c.kernels += 2;
  }
  float l = 0.f;
  CK(cudaMemcpyAsync(&l, k.loss, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  k.last_loss = l;
  return 0;
}

// Device staging buffer of the packed kinematics transfers (19 doubles per body).
static int ensure_kin_stage(Ctx& c) {
  if (c.kin_stage_n < c.s.n) {
    int rc;
    if ((rc = dalloc(c, c.kin_stage, 19 * c.s.n))) return rc;
    c.kin_stage_n = c.s.n;
  }
  return 0;
}

// Scene fields of the fused guard (null when the skin is off).  Bodies past
// half of their budget are flagged, to be refreshed together with the one
// that reached it.
static void skin_bind(Ctx& c, bool on) {
  Skin& k = c.skin;
  Scene& s = c.s;
  s.sk_path = on ? k.path : nullptr;
  s.sk_rsw = on ? k.rsw : nullptr;
  s.sk_ref_pos = on ? k.ref_pos : nullptr;
  s.sk_ref_q = on ? k.ref_q : nullptr;
  s.sk_maxd = on ? k.maxd : nullptr;
  s.sk_flag = on ? k.flag : nullptr;
  s.sk_out = on ? k.d_guard : nullptr;
  s.sk_flag_at = on ? (float)(0.25 * k.skin) : 0.f;
}

static int skin_rebuild(Ctx& c, double dmax, double vmax, bool forced) {
  {  // the flags are not read every step when the guard is pipelined
    const int rf = read_flags(c);
    if (rf) return rf;
  }
  Skin& k = c.skin;
  Scene& s = c.s;
  const double N = (double)std::max<int64_t>(1, s.n - s.n_driven);
  const double ref = k.cfg.skin_max;
  // displacement rate that sets the next full rebuild: the largest body's
  // without partial refreshes; with them (the fastest bodies are refreshed on
  // their own), the 80th percentile of the bodies' guard values
  const double rate_max = dmax / (double)std::max<int64_t>(1, k.since);
  double rate = rate_max;
  if (k.cfg.partial_fraction > 0.0) {
    unsigned int h[64];
    CK(cudaMemsetAsync(k.d_hist, 0, sizeof h, c.stream));
    c.kernels += launch_skin_hist(s, k.ref_pos, k.ref_q, k.rsw, (float)k.skin, k.d_hist, c.stream);
    CK(cudaMemcpyAsync(h, k.d_hist, sizeof h, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    const double want = 0.8 * (double)s.n;
    double acc = 0.0;
    int bin = 63;
    for (int q = 0; q < 64; q++) {
      acc += h[q];
      if (acc >= want) { bin = q; break; }
    }
    const double d80 = k.skin * std::pow(2.0, (bin + 1) / 4.0 - 14.0);  // upper edge of the bin
    rate = std::max(d80 / (double)std::max<int64_t>(1, k.since), 1e-30);
  }
  const int64_t ne0 = s.ne;
  const double active = (double)c.h_flags[FLAG_NACTIVE];
  if (k.since > 0) {  // measured cost of the window
    float ms = 0.f;
    CK(cudaEventRecord(k.eb, c.stream));
    CK(cudaEventSynchronize(k.eb));
    CK(cudaEventElapsedTime(&ms, k.ea, k.eb));
    double per = ms / (double)k.since;
    k.step_ms = k.step_ms > 0 ? 0.7 * k.step_ms + 0.3 * per : per;
  }
  k.last_rate = rate;
  for (int q = 3; q > 0; q--) k.rates[q] = k.rates[q - 1];
  k.rates[0] = rate;
  auto lg = [](double x) { return (float)std::log10(std::max(x, 1e-30)); };
  std::array<float, 16> f{};
  f[0] = lg(rate / ref);
  f[1] = lg(k.rates[1] / ref);
  f[2] = lg(k.rates[2] / ref);
  f[3] = lg(k.rates[3] / ref);
  f[4] = lg(vmax * s.dt / ref);
  f[5] = (float)(active / N);
  f[6] = (float)((double)ne0 / (N * 50.0));
  f[7] = lg(k.skin / ref);
  f[8] = (float)(std::log10((double)k.since + 1.0) / 3.0);
  f[9] = forced ? 1.f : 0.f;
  f[10] = (float)std::min(1.0, k.pred_churn);
  f[11] = lg(k.step_ms + 1e-3);
  f[12] = lg(k.rebuild_ms + 1e-3);
  f[13] = (float)std::max(-3.0, std::min(3.0, std::log10(std::max(rate, 1e-30) / std::max(k.rates[1], 1e-30))));
  f[14] = 1.f;
  f[15] = (float)std::max(-3.0, std::min(3.0, std::log10(std::max(rate_max, 1e-30) / std::max(rate, 1e-30))));
  // prediction of the next window's displacement rate
  // The network predicts corrections to the method without it, as log10
  // ratios: next rate / this window's rate, next churn / the last observed
  // churn.  Its output layer starts at zero, so it starts as that method
  // and departs from it only as far as its training supports.
  const double churn_base = k.pred_churn;
  double u = rate, churn = churn_base;
  if (k.cfg.use_mlp && k.rx.size() >= (size_t)kMinWindows) {
    float y[2];
    CK(cudaMemcpyAsync(k.io, f.data(), 64, cudaMemcpyHostToDevice, c.stream));
    launch_mlp_infer(k.w, k.io, k.io + 16, c.stream);
    c.kernels++;
    CK(cudaMemcpyAsync(y, k.io + 16, 8, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    const double r0 = std::max(-2.0, std::min(2.0, (double)y[0]));
    const double r1 = std::max(-2.0, std::min(2.0, (double)y[1]));
    u = rate * std::pow(10.0, r0);
    churn = std::max(0.0, (churn_base + 1e-4) * std::pow(10.0, r1) - 1e-4);
  }
  if (!(u > 0.0) || !std::isfinite(u)) u = std::max(rate, 1e-30);
  k.pred_rate = u;
  // skin and interval minimising the predicted cost per step.  Entries grow
  // faster than the skin (more sub-element pairs come within reach): the
  // non-active entries are scaled by (skin ratio)^alpha, alpha learnt from
  // the rebuilds that changed the skin (1.6, the power measured on hull-grain
  // piles, to start).  The step time is measured over the last window,
  // with the narrow phase (timed by events, proportional to the list) apart;
  // the last full rebuild is timed in two parts, the broad phase (70 %
  // fixed) and the candidates-to-index part (proportional to the list); the
  // partial refreshes of the window are counted and timed.  The interval is
  // the number of steps the predicted displacement rate takes to use half
  // the skin (with a margin), which is also when the guard would force it.
  const double margin = 1.3, alpha = k.alpha;
  const double skin_before = k.skin;
  const double C = (double)std::max<int64_t>(1, ne0), A = std::min(active, C);
  // partial refreshes of the window: their rate grows as the skin shrinks
  // (the fast bodies use it up sooner); their time is part of the window's
  // step time and is taken out of it
  const double P = (double)k.partial_in_window / (double)std::max<int64_t>(1, k.since);
  const double Rp = k.partial_ms;
  const double T = std::max(0.0, (k.step_ms > 0 ? k.step_ms : 0.2) - P * Rp);
  const double Tn = k.narrow_cnt > 0 ? std::min(T, k.narrow_acc / (double)k.narrow_cnt) : 0.4 * T;
  const double Rbp = k.rebuild_bp_ms > 0 ? k.rebuild_bp_ms : 2.0;
  const double Rvar = k.rebuild_var_ms > 0 ? k.rebuild_var_ms : 2.0;
  double best = 1e300, best_s = k.skin;
  int64_t best_k = k.interval;
  for (int m = -4; m <= 4; m++) {
    double sk = std::min(k.cfg.skin_max, std::max(k.cfg.skin_min, k.skin * std::pow(2.0, 0.25 * m)));
    double kk = std::floor(0.5 * sk / std::max(u * margin * (1.0 + churn), 1e-30));
    int64_t ki = (int64_t)std::max<double>(k.cfg.interval_min, std::min<double>(k.cfg.interval_max, kk));
    double ratio = (A + (C - A) * std::pow(sk / std::max(k.skin, 1e-30), alpha)) / C;
    double J = (T - Tn) + Tn * ratio + (Rbp * (0.7 + 0.3 * ratio) + Rvar * ratio) / (double)ki +
               P * (k.skin / sk) * Rp;
    if (J < best) { best = J; best_s = sk; best_k = ki; }
  }
  k.skin = best_s;
  k.interval = best_k;
  s.dVerlet = k.skin;
  s.DVerlet = k.cfg.dverlet_ratio * k.skin;
  s.sk_flag_at = (float)(0.25 * k.skin);
  settle_before_update(c);
  // the rebuild itself, timed
  float rms = 0.f, rbp = 0.f;
  if (!c.w.split) CK(cudaEventCreate(&c.w.split));
  CK(cudaEventRecord(k.ea, c.stream));
  c.w.timing_split = true;
  int rc = rebuild_nl(c);
  c.w.timing_split = false;
  if (rc) return rc;
  CK(cudaEventRecord(k.eb, c.stream));
  CK(cudaEventSynchronize(k.eb));
  CK(cudaEventElapsedTime(&rms, k.ea, k.eb));
  CK(cudaEventElapsedTime(&rbp, k.ea, c.w.split));
  k.rebuild_bp_ms = rbp;
  k.rebuild_var_ms = std::max(0.0, (double)rms - (double)rbp);
  k.rebuild_ms = k.rebuild_ms > 0 ? 0.7 * k.rebuild_ms + 0.3 * rms : rms;
  c.nl_updates++;
  k.rebuilds++;
  if (forced) k.forced++;
  else k.scheduled++;
  const double churn_obs = std::fabs((double)s.ne - (double)ne0) / std::max(1.0, (double)ne0);
  // growth exponent of the non-active entries with the skin, from this
  // rebuild when the skin changed (exponential average, starts at 1.6)
  if (std::fabs(std::log(k.skin / skin_before)) > 0.05 && (double)ne0 > 1.05 * A && (double)s.ne > 1.05 * A) {
    const double obs = std::log(((double)s.ne - A) / ((double)ne0 - A)) / std::log(k.skin / skin_before);
    k.alpha = 0.7 * k.alpha + 0.3 * std::max(0.3, std::min(3.0, obs));
  }
  k.pred_churn = churn_obs;
  // training sample: the previous window's features -> this window's outcome
  if (k.have_prev) {
    std::array<float, 2> y{lg(rate / ref) - k.feat_prev[0], lg(churn_obs + 1e-4) - lg(k.churn_base_prev + 1e-4)};
    if (k.rx.size() < (size_t)mlp_max_batch()) {
      k.rx.push_back(k.feat_prev);
      k.ry.push_back(y);
    } else {
      k.rx[k.rhead] = k.feat_prev;
      k.ry[k.rhead] = y;
      k.rhead = (k.rhead + 1) % k.rx.size();
    }
  }
  k.feat_prev = f;
  k.churn_base_prev = churn_base;
  k.have_prev = true;
  if (k.cfg.use_mlp && (rc = skin_train(c))) return rc;
  c.kernels += launch_skin_reset(s, nullptr, k.ref_pos, k.ref_q, k.maxd, k.path, c.stream);
  CK(cudaMemsetAsync(s.flags + FLAG_NEED_UPDATE, 0, sizeof(unsigned long long), c.stream));
  k.since = 0;
  k.partial_since_global = 0;
  k.narrow_acc = 0.0;
  k.narrow_cnt = 0;
  k.partial_in_window = 0;
  CK(cudaEventRecord(k.ea, c.stream));
  return 0;
}

// The launches of one step body (flag reset, controls, drift, global
// vertices, narrow phase + law, resultants + accelerations, breakage) as one
// CUDA graph: captured on the context stream the first time and whenever the
// scene description the kernels receive by value has changed since (a
// rebuild swaps the entry buffers, a parameter call changes scalars), then
// replayed.  Same kernels, same arguments, same order as the launch-by-launch
// path, so the results are identical.
static int step_launches(Ctx& c, bool time_narrow = true) {
  Scene& s = c.s;
  int n = 0;
  n += launch_controls_pre(s, c.stream);
  n += launch_drift(s, c.stream);
  n += launch_glob_vertices(s, c.stream);
  // the skin's cost model wants the narrow-phase time
  const bool timed = time_narrow && c.skin.on && c.skin.nev[0];
  if (timed) cudaEventRecord(c.skin.nev[0], c.stream);
  n += c.form == RK_FORM_MIXED ? launch_narrow_force_mixed(s, c.stream) : launch_narrow_force(s, c.stream);
  if (timed) cudaEventRecord(c.skin.nev[1], c.stream);
  n += launch_gather_heavy(s, c.stream) + launch_gather_accel(s, 1, c.stream);
  n += launch_breakage(s, c.stream);
  return n;
}

// Online block-size tuning: during the first steps after rk_set_autotune,
// step k launches the four tuned kernels (narrow phase, resultants, global
// vertices, drift) with candidate block size k mod 5, timed with events;
// then each kernel keeps its fastest size.  Every thread of these kernels
// works on its own entry, body or vertex (ordered sums included), so the
// block size changes no result and the tuning steps are ordinary steps.
static const int kTuneCand[5] = {32, 64, 128, 256, 512};
constexpr int kNumCand = 5;

static int tune_step(Ctx& c) {
  Scene& s = c.s;
  const int64_t done = c.tune_total - c.tune_left;
  const int ci = (int)(done % kNumCand);
  for (int k = 0; k < 4; k++) s.tpb[k] = std::min(kTuneCand[ci], max_tpb(k, c.form == RK_FORM_MIXED));
  cudaStream_t st = c.stream;
  int n = launch_controls_pre(s, st);
  CK(cudaEventRecord(c.tev[0], st));
  n += launch_drift(s, st);
  CK(cudaEventRecord(c.tev[1], st));
  n += launch_glob_vertices(s, st);
  CK(cudaEventRecord(c.tev[2], st));
  n += c.form == RK_FORM_MIXED ? launch_narrow_force_mixed(s, st) : launch_narrow_force(s, st);
  CK(cudaEventRecord(c.tev[3], st));
  n += launch_gather_heavy(s, st);
  CK(cudaEventRecord(c.tev[4], st));
  n += launch_gather_accel(s, 1, st);
  CK(cudaEventRecord(c.tev[5], st));
  n += launch_breakage(s, st);
  c.kernels += n;
  CK(cudaEventSynchronize(c.tev[5]));
  float ms[4] = {0, 0, 0, 0};
  cudaEventElapsedTime(&ms[3], c.tev[0], c.tev[1]);  // drift
  cudaEventElapsedTime(&ms[2], c.tev[1], c.tev[2]);  // global vertices
  cudaEventElapsedTime(&ms[0], c.tev[2], c.tev[3]);  // narrow phase
  cudaEventElapsedTime(&ms[1], c.tev[4], c.tev[5]);  // resultants
  for (int k = 0; k < 4; k++) c.tune_ms[k][ci] += ms[k];
  if (--c.tune_left == 0) {
    for (int k = 0; k < 4; k++) {
      int best = 2;
      for (int q = 0; q < kNumCand; q++)
        if (c.tune_ms[k][q] < c.tune_ms[k][best]) best = q;
      s.tpb[k] = std::min(kTuneCand[best], max_tpb(k, c.form == RK_FORM_MIXED));
    }
  }
  return RK_OK;
}

// Instantiates captured graph g into *ex (updating it in place when the
// topology allows); g is destroyed.
static int graph_install(Ctx& c, cudaGraph_t g, cudaGraphExec_t* ex, const char* what) {
  bool updated = false;
  if (*ex) {
    cudaGraphExecUpdateResultInfo info;
    updated = cudaGraphExecUpdate(*ex, g, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();
      cudaGraphExecDestroy(*ex);
      *ex = nullptr;
    }
  }
  if (!updated) {
    const cudaError_t e = cudaGraphInstantiate(ex, g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      *ex = nullptr;
      c.err = std::string(what) + " instantiation: " + cudaGetErrorString(e);
      return RK_ERR_CUDA;
    }
  }
  cudaGraphDestroy(g);
  return RK_OK;
}

static int step_graph(Ctx& c) {
  Scene& s = c.s;
  const bool stale = !c.gexec || c.gform != c.form || std::memcmp(&c.gscene, &s, sizeof(Scene)) != 0;
  if (stale) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(s.flags + FLAG_NACTIVE, 0, sizeof(unsigned long long), c.stream);
    int n = step_launches(c);
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      c.err = std::string("step graph capture: ") + cudaGetErrorString(e);
      return RK_ERR_CUDA;
    }
    const int rc = graph_install(c, g, &c.gexec, "step graph");
    if (rc) return rc;
    std::memcpy(&c.gscene, &s, sizeof(Scene));  // byte copy: the comparison above is bytewise
    c.gform = c.form;
    c.glaunched = n;
    c.graph_captures++;
  }
  CK(cudaGraphLaunch(c.gexec, c.stream));
  c.skin.narrow_timed = c.skin.on && c.skin.nev[0];
  c.graph_replays++;
  c.kernels += c.glaunched;
  return RK_OK;
}

// Largest batch of the device-decided skin mode (skin_batch): long enough to
// take the host round trip out of almost every step, short enough that the
// steps skipped after a trigger (each a handful of launches that return at
// once) stay cheap.  A call for fewer steps runs the largest power-of-two
// batch that fits, so that no step is skipped for want of work.
constexpr int kSkinBatch = 16;

// The graph of a batch of 2^lg steps, opened by k_skin_begin; each step's
// resultant kernel closes it (skin_batch_step_end); the narrow phase of the
// first step is timed for the skin's cost model.  Captured with s.sk_ctl set,
// like the launches it holds.
static int batch_graph(Ctx& c, int lg) {
  Scene& s = c.s;
  const bool stale =
      !c.bexec[lg] || c.bform[lg] != c.form || std::memcmp(&c.bscene[lg], &s, sizeof(Scene)) != 0;
  if (stale) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    int n = 0;
    n += launch_skin_begin(s, c.stream);
    for (int q = 0; q < (1 << lg); q++) n += step_launches(c, q == 0);
    const cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      c.err = std::string("skin batch graph capture: ") + cudaGetErrorString(e);
      return RK_ERR_CUDA;
    }
    const int rc = graph_install(c, g, &c.bexec[lg], "skin batch graph");
    if (rc) return rc;
    std::memcpy(&c.bscene[lg], &s, sizeof(Scene));
    c.bform[lg] = c.form;
    c.blaunched[lg] = n;
    c.graph_captures++;
  }
  CK(cudaGraphLaunch(c.bexec[lg], c.stream));
  c.graph_replays++;
  c.kernels += c.blaunched[lg];
  return RK_OK;
}

static int skin_partial(Ctx& c, int64_t nflag);

// Up to `left` steps of the skin mode as one batch: the device checks the
// exact guard after every step and halts the batch when a refresh is due, so
// the host syncs once per batch; it then takes the same decision as
// skin_after_step from the halting step's guard words.  *done = steps run.
static int skin_batch(Ctx& c, int64_t left, int64_t* done) {
  Skin& k = c.skin;
  Scene& s = c.s;
  int lg = 0;
  while (lg < 4 && (int64_t)2 << lg <= left) lg++;
  const int64_t want = (int64_t)1 << lg;
  unsigned int* in = k.h_ctl;
  unsigned int* out = k.h_ctl + 16;
  float trig = (float)(0.5 * k.skin);
  if ((double)trig < 0.5 * k.skin) trig = std::nextafter(trig, INFINITY);
  in[0] = 0u;
  in[1] = 0u;
  in[2] = (unsigned)std::min<int64_t>(k.since, 0x7fffffff);
  in[3] = (unsigned)want;
  in[4] = (unsigned)std::min<int64_t>(std::max<int64_t>(k.interval, 1), 0x7fffffff);
  std::memcpy(&in[5], &trig, 4);
  in[6] = k.partial_since_global > 0 ? 1u : 0u;
  in[7] = 0u;
  CK(cudaMemcpyAsync(k.d_ctl, in, 8 * sizeof(unsigned int), cudaMemcpyHostToDevice, c.stream));
  s.sk_ctl = k.d_ctl;
  int rc = batch_graph(c, lg);
  s.sk_ctl = nullptr;
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, k.d_ctl, 16 * sizeof(unsigned int), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaEventRecord(k.bev, c.stream));
  CK(cudaEventSynchronize(k.bev));
  const int64_t ex = out[1];
  if (ex < 1 || ex > want) {
    c.err = "skin batch: step count out of range";
    return RK_ERR_STATE;
  }
  for (int64_t q = 0; q < ex; q++) {
    c.t += s.dt;
    c.interVerletC += s.dt;
  }
  c.steps += ex;
  *done = ex;
  c.more_steps_follow = ex < left;
  c.forces_stale = s.nheavy_lazy > 0;
  k.since = out[2];
  if (k.nev[0]) {  // the first step of the batch ran its narrow phase between these events
    float nms = 0.f;
    if (cudaEventElapsedTime(&nms, k.nev[0], k.nev[1]) == cudaSuccess) {
      k.narrow_acc += nms;
      k.narrow_cnt++;
    } else {
      cudaGetLastError();
    }
  }
  k.narrow_timed = false;
  k.have_pred = false;
  const unsigned int* hg = out + 8;
  const double dmax = to_f(hg[0]), vmax = to_f(hg[1]), gmax = to_f(hg[2]);
  const int64_t nflag = (int64_t)hg[3];
  const double crit = k.partial_since_global > 0 ? gmax : dmax;
  if (k.since >= k.interval) return skin_rebuild(c, dmax, vmax, false);
  if (crit >= 0.5 * k.skin) {
    if (k.cfg.partial_fraction > 0.0 && nflag > 0 && (double)nflag <= k.cfg.partial_fraction * (double)s.n)
      return skin_partial(c, nflag);
    return skin_rebuild(c, dmax, vmax, true);
  }
  return 0;
}

// Partial refresh of the flagged bodies (see rk_skin.cu): the neighbour
// list restricted to their pairs, and their snapshots reset.
static int skin_partial(Ctx& c, int64_t nflag) {
  Skin& k = c.skin;
  Scene& s = c.s;
  settle_before_update(c);
  CK(cudaEventRecord(k.pa, c.stream));
  int rc = rebuild_nl(c, k.flag);
  if (rc) return rc;
  c.kernels += launch_skin_reset(s, k.flag, k.ref_pos, k.ref_q, k.maxd, k.path, c.stream);
  CK(cudaEventRecord(k.pb, c.stream));
  CK(cudaEventSynchronize(k.pb));
  float pms = 0.f;
  CK(cudaEventElapsedTime(&pms, k.pa, k.pb));
  k.partial_ms = k.partial_ms > 0 ? 0.7 * k.partial_ms + 0.3 * pms : pms;
  k.partial_in_window++;
  c.nl_updates++;
  k.partial++;
  k.partial_bodies += nflag;
  k.partial_since_global++;
  return 0;
}

// The guard's read-back is pipelined when the prediction it makes is exact
// for the scene: no control moves a driven body between steps, and neither
// interfaces nor the reference guard can request an update.  Then the host
// reads the previous step's bound of this state while the GPU already runs
// this step, and waits for this step's own (exact) guard values only when
// the bound comes within 2 % of the trigger.
static bool guard_pipelined(const Ctx& c) {
  const Scene& s = c.s;
  return s.ncontrols == 0 && s.servo_kind == 0 && s.nif == 0 && s.dynamic_nl == 0;
}

int skin_after_step(Ctx& c) {
  Skin& k = c.skin;
  Scene& s = c.s;
  // the step's resultant kernel evaluated the guard into d_guard
  const int slot = k.gslot;
  unsigned int* hg = k.h_guard + 8 * slot;
  CK(cudaMemcpyAsync(hg, k.d_guard, 32, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaEventRecord(k.gev[slot], c.stream));
  k.gslot ^= 1;
  k.since++;
  const bool pipe = guard_pipelined(c);
  if (pipe && k.have_pred) {
    // the previous step's guard predicted this state
    const unsigned int* hp = k.h_guard + 8 * (slot ^ 1);
    CK(cudaEventSynchronize(k.gev[slot ^ 1]));
    const double pcrit = to_f(k.partial_since_global > 0 ? hp[7] : hp[6]);
    const bool due = pcrit >= 0.5 * k.skin * 0.98 || k.since >= k.interval;
    if (!due) {
      k.narrow_timed = false;  // this step's events may still be running
      return 0;
    }
  }
  // this step's guard: the exact values of this state
  CK(cudaEventSynchronize(k.gev[slot]));
  int rc;
  if (!pipe && (rc = read_flags(c))) return rc;
  if (k.narrow_timed) {
    float nms = 0.f;
    if (cudaEventElapsedTime(&nms, k.nev[0], k.nev[1]) == cudaSuccess) {
      k.narrow_acc += nms;
      k.narrow_cnt++;
    } else {
      cudaGetLastError();  // not timed this step: the model falls back to its default share
    }
    k.narrow_timed = false;
  }
  k.have_pred = pipe;  // holds until a refresh moves the snapshots
  const double dmax = to_f(hg[0]), vmax = to_f(hg[1]), gmax = to_f(hg[2]);
  const int64_t nflag = (int64_t)hg[3];
  const double crit = k.partial_since_global > 0 ? gmax : dmax;
  const bool forced = crit >= 0.5 * k.skin;
  const bool need = !pipe && c.h_flags[FLAG_NEED_UPDATE] != 0ull;
  if (need || k.since >= k.interval) {
    k.have_pred = false;
    return skin_rebuild(c, dmax, vmax, false);
  }
  if (forced) {
    k.have_pred = false;
    if (k.cfg.partial_fraction > 0.0 && nflag > 0 && (double)nflag <= k.cfg.partial_fraction * (double)s.n)
      return skin_partial(c, nflag);
    return skin_rebuild(c, dmax, vmax, true);
  }
  return 0;
}

extern "C" {

int rk_abi_version(void) { return RK_ABI_VERSION; }

int rk_create(rk_ctx** out, const rk_config* cfg) {
  if (!out) return RK_ERR_ARG;
  *out = nullptr;
  rk_ctx* x = new (std::nothrow) rk_ctx();
  if (!x) return RK_ERR_CAPACITY;
  Ctx& c = x->c;
  c.device = cfg ? cfg->device : 0;
  c.form = cfg ? cfg->form : RK_FORM_FP64;
  c.s.fast_body = c.form == RK_FORM_MIXED ? 1 : 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || c.device < 0 || c.device >= ndev) {
    delete x;
    return RK_ERR_CUDA;
  }
  if (c.form != RK_FORM_FP64 && c.form != RK_FORM_MIXED) {
    delete x;
    return RK_ERR_UNSUPPORTED;
  }
  if (cudaSetDevice(c.device) != cudaSuccess || cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c.ev0) != cudaSuccess || cudaEventCreate(&c.ev1) != cudaSuccess ||
      cudaMallocHost(&c.h_flags, FLAG_COUNT * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&c.s.flags, FLAG_COUNT * sizeof(unsigned long long)) != cudaSuccess) {
    delete x;
    return RK_ERR_CUDA;
  }
  cudaMemsetAsync(c.s.flags, 0, FLAG_COUNT * sizeof(unsigned long long), c.stream);
  c.s.n = 0;
  c.s.ne = 0;
  c.s.nif = 0;
  int64_t cap0 = cfg && cfg->entry_capacity > 0 ? cfg->entry_capacity : 1024;
  if (ensure_entry_capacity(c, 0, cap0) || ensure_entry_capacity(c, 1, cap0)) {
    rk_destroy(x);
    return RK_ERR_CUDA;
  }
  bind_entries(c);
  // empty interface table
  dupload(c, c.s.if_i, (const int*)nullptr, 0);
  *out = x;
  return RK_OK;
}

void rk_destroy(rk_ctx* x) {
  if (!x) return;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.gexec) cudaGraphExecDestroy(c.gexec);
  for (cudaGraphExec_t e : c.bexec)
    if (e) cudaGraphExecDestroy(e);
  for (int k = 0; k < 8; k++)
    if (c.tev[k]) cudaEventDestroy(c.tev[k]);
  Scene& s = c.s;
  dfree(s.vert_ofs); dfree(s.edge_ofs); dfree(s.edges); dfree(s.face_ofs); dfree(s.face_vofs); dfree(s.face_verts);
  dfree(s.svert); dfree(s.sradius); dfree(s.sobb); dfree(s.sbox); dfree(s.bbox);
  dfree(s.pos); dfree(s.vel); dfree(s.acc); dfree(s.Q); dfree(s.vrot); dfree(s.arot); dfree(s.force); dfree(s.moment);
  dfree(s.hom); dfree(s.mass); dfree(s.inertia); dfree(s.rad); dfree(s.inv_mi); dfree(s.shape); dfree(s.group); dfree(s.cluster);
  dfree(s.gv_ofs); dfree(s.gv_body); dfree(s.lv); dfree(s.gv); dfree(s.gvr); dfree(s.posf); dfree(s.rotm); dfree(s.gsum); dfree(s.uv64); dfree(s.uvf); dfree(s.bobb); dfree(s.bobbf); dfree(s.baabb); dfree(s.dpos); dfree(s.dq);
  dfree(s.table); dfree(s.controls);
  dfree(s.act); dfree(s.cf); dfree(s.cmi); dfree(s.cmj); dfree(s.iofs); dfree(s.jofs); dfree(s.jsplit); dfree(s.jlist); dfree(s.nperm); dfree(s.egv); dfree(s.slow);
  dfree(s.heavy); dfree(s.is_heavy); dfree(s.sph); dfree(s.sph_ofs); dfree(s.sph_body); dfree(s.heavy_lazy); dfree(s.bnd);
  dfree(s.needres); dfree(s.scene_of); dfree(s.bf_surf);
  dfree(c.name_chars); dfree(c.name_ofs);
  dfree(s.if_i); dfree(s.if_j); dfree(s.if_dn0); dfree(s.if_par); dfree(s.if_inner); dfree(s.if_broken);
  dfree(s.if_break); dfree(s.if_ofs); dfree(s.flags);
  free_entrybuf(c.eb[0]);
  free_entrybuf(c.eb[1]);
  NLWork& w = c.w;
  dfree(w.pairs); dfree(w.hp); dfree(w.hp_tmp); dfree(w.hp_mask); dfree(w.cand); dfree(w.cand_tmp);
  dfree(w.flag); dfree(w.stale); dfree(w.stale_src); dfree(w.fkey); dfree(w.fsrc); dfree(w.jkeys); dfree(w.jtmp);
  dfree(w.tmp); dfree(w.counter); dfree(w.gkeys); dfree(w.gtmp); dfree(w.gover); dfree(w.gis_over); dfree(w.gmark);
  if (w.gstat) cudaFree(w.gstat);
  if (w.split) cudaEventDestroy(w.split);
  dfree(c.kin_stage);
  dfree(c.ext_part);
  dfree(c.ext_u);
  dfree(c.d_ke);
  {
    Skin& k = c.skin;
    dfree(k.ref_pos); dfree(k.ref_q); dfree(k.rsw); dfree(k.d_guard); dfree(k.master); dfree(k.m); dfree(k.v);
    dfree(k.maxd); dfree(k.path); dfree(k.flag); dfree(k.d_hist);
    dfree(k.grad); dfree(k.loss); dfree(k.X); dfree(k.T); dfree(k.io);
    if (k.w) cudaFree(k.w);
    if (k.h_guard) cudaFreeHost(k.h_guard);
    if (k.d_ctl) cudaFree(k.d_ctl);
    if (k.h_ctl) cudaFreeHost(k.h_ctl);
    if (k.bev) cudaEventDestroy(k.bev);
    if (k.ea) cudaEventDestroy(k.ea);
    for (cudaEvent_t e : {k.nev[0], k.nev[1], k.pa, k.pb, k.gev[0], k.gev[1]})
      if (e) cudaEventDestroy(e);
    if (k.eb) cudaEventDestroy(k.eb);
  }
  for (int k = 0; k < 2 * RK_NPHASE; k++)
    if (c.pev[k]) cudaEventDestroy(c.pev[k]);
  if (c.h_flags) cudaFreeHost(c.h_flags);
  if (c.ev0) cudaEventDestroy(c.ev0);
  if (c.ev1) cudaEventDestroy(c.ev1);
  if (c.stream) cudaStreamDestroy(c.stream);
  delete x;
}

const char* rk_last_error(const rk_ctx* x) { return x ? x->c.err.c_str() : "null context"; }

int rk_upload_shapes(rk_ctx* x, const rk_shapes* sh) {
  if (!x || !sh || sh->nshapes <= 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const int ns = sh->nshapes;
  const int nv = sh->vert_ofs[ns], ne = sh->edge_ofs[ns], nf = sh->face_ofs[ns], nfv = sh->face_vofs[nf];
  const std::vector<int> nv_before = c.shape_nv, ne_before = c.shape_ne, nf_before = c.shape_nf;
  c.shape_nv.assign(ns, 0);
  c.shape_ne.assign(ns, 0);
  c.shape_nf.assign(ns, 0);
  for (int k = 0; k < ns; k++) {
    int v = sh->vert_ofs[k + 1] - sh->vert_ofs[k];
    int e = sh->edge_ofs[k + 1] - sh->edge_ofs[k];
    int f = sh->face_ofs[k + 1] - sh->face_ofs[k];
    if (v <= 0 || v > 64) return fail(c, RK_ERR_CAPACITY, "a shape has no vertex or more than 64 vertices");
    if (e >= kMaxSub || f >= kMaxSub) return fail(c, RK_ERR_CAPACITY, "a shape has more than 1023 edges or faces");
    c.shape_nv[k] = v;
    c.shape_ne[k] = e;
    c.shape_nf[k] = f;
  }
  c.shape_vmax.assign(ns, 0.0);
  for (int k = 0; k < ns; k++)
    for (int v = sh->vert_ofs[k]; v < sh->vert_ofs[k + 1]; v++) {
      const double* p = sh->vertices + 3 * (int64_t)v;
      c.shape_vmax[k] = std::max(c.shape_vmax[k], std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
    }
  for (int f = 0; f < nf; f++)
    if (sh->face_vofs[f + 1] - sh->face_vofs[f] < 3) return fail(c, RK_ERR_ARG, "a face has fewer than 3 vertices");
  // the box of each shape's vertices in its own frame (centre, half extents)
  std::vector<double> sbox(6 * (size_t)ns);
  for (int k = 0; k < ns; k++) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v = sh->vert_ofs[k]; v < sh->vert_ofs[k + 1]; v++)
      for (int d = 0; d < 3; d++) {
        lo[d] = std::min(lo[d], sh->vertices[3 * (int64_t)v + d]);
        hi[d] = std::max(hi[d], sh->vertices[3 * (int64_t)v + d]);
      }
    for (int d = 0; d < 3; d++) {
      sbox[6 * k + d] = 0.5 * (lo[d] + hi[d]);
      sbox[6 * k + 3 + d] = 0.5 * (hi[d] - lo[d]);
    }
  }
  Scene& s = c.s;
  int rc;
  if ((rc = dupload(c, s.vert_ofs, sh->vert_ofs, ns + 1)) || (rc = dupload(c, s.edge_ofs, sh->edge_ofs, ns + 1)) ||
      (rc = dupload(c, s.edges, sh->edges, 2 * (int64_t)ne)) || (rc = dupload(c, s.face_ofs, sh->face_ofs, ns + 1)) ||
      (rc = dupload(c, s.face_vofs, sh->face_vofs, nf + 1)) ||
      (rc = dupload(c, s.face_verts, sh->face_verts, nfv)) || (rc = dupload(c, s.svert, sh->vertices, 3 * (int64_t)nv)) ||
      (rc = dupload(c, s.sradius, sh->radius, ns)) || (rc = dupload(c, s.sobb, sh->obb, 15 * (int64_t)ns)) ||
      (rc = dupload(c, s.sbox, sbox.data(), 6 * (int64_t)ns)))
    return rc;
  s.nshapes = ns;
  c.shape_radius.assign(sh->radius, sh->radius + ns);
  c.have_shapes = true;
  if (c.have_bodies && c.s.n > 0) {  // bodies placed on the new shape tables: same element counts only
    bool same = true;
    for (int64_t b = 0; b < c.s.n && b < (int64_t)c.body_shape.size() && same; b++) {
      const int q = c.body_shape[b];
      same = q < ns && q < (int)nv_before.size() && c.shape_nv[q] == nv_before[q] && c.shape_ne[q] == ne_before[q] &&
             c.shape_nf[q] == nf_before[q];
    }
    if (!same) {
      c.have_bodies = false;
      c.s.n = 0;
      c.s.ne = 0;
      return fail(c, RK_ERR_STATE, "new shape tables change the bodies' vertex, edge or face counts: upload the bodies again");
    }
    c.kernels += launch_body_verts(c.s, c.stream);
    CK(cudaGetLastError());
  }
  return RK_OK;
}

int rk_upload_bodies(rk_ctx* x, const rk_bodies* b) {
  if (!x || !b || b->n <= 0 || b->n_driven < 0 || b->n_driven > b->n) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_shapes) return fail(c, RK_ERR_STATE, "upload the shapes before the bodies");
  if (b->n >= kMaxBody) return fail(c, RK_ERR_CAPACITY, "more than 2^21 - 1 bodies");
  const int64_t n = b->n;
  // new bodies: the learned skin (per-body guard state) starts again with rk_set_skin
  c.skin.on = false;
  skin_bind(c, false);
  c.s.near_geometric = 0;
  std::vector<int64_t> gv_ofs(n + 1, 0);
  std::vector<double> rad(n);
  std::vector<float> inv_mi(4 * n);  // the mixed form's 1/m, 1/Ix, 1/Iy, 1/Iz
  for (int64_t i = 0; i < n; i++) {
    int sh = b->shape[i];
    if (sh < 0 || sh >= c.s.nshapes) return fail(c, RK_ERR_ARG, "body shape index out of range");
    gv_ofs[i + 1] = gv_ofs[i] + c.shape_nv[sh];
    rad[i] = b->homothety[i] * c.shape_radius[sh];  // Particle::MinkowskiRadius (Particle.cpp:71)
    inv_mi[4 * i] = (float)(1.0 / b->mass[i]);
    for (int d = 0; d < 3; d++) inv_mi[4 * i + 1 + d] = (float)(1.0 / b->inertia[3 * i + d]);
  }
  const int64_t nv = gv_ofs[n];
  std::vector<int64_t> sph_ofs(n + 1, 0);
  for (int64_t i = 0; i < n; i++) {
    int sh = b->shape[i];
    sph_ofs[i + 1] = sph_ofs[i] + c.shape_nv[sh] + c.shape_ne[sh] + c.shape_nf[sh];
  }
  c.nsph = sph_ofs[n];
  std::vector<int> sph_body(std::max<int64_t>(sph_ofs[n], 1));
  for (int64_t i = 0; i < n; i++)
    for (int64_t k = sph_ofs[i]; k < sph_ofs[i + 1]; k++) sph_body[k] = (int)i;
  std::vector<int> gv_body(nv);
  for (int64_t i = 0; i < n; i++)
    for (int64_t k = gv_ofs[i]; k < gv_ofs[i + 1]; k++) gv_body[k] = (int)i;
  Scene& s = c.s;
  int rc;
  if ((rc = dupload(c, s.pos, b->pos, 3 * n)) || (rc = dupload(c, s.vel, b->vel, 3 * n)) ||
      (rc = dupload(c, s.acc, b->acc, 3 * n)) || (rc = dupload(c, s.Q, b->Q, 4 * n)) ||
      (rc = dupload(c, s.vrot, b->vrot, 3 * n)) || (rc = dupload(c, s.arot, b->arot, 3 * n)) ||
      (rc = dupload(c, s.force, (const double*)nullptr, 3 * n)) ||
      (rc = dupload(c, s.moment, (const double*)nullptr, 3 * n)) || (rc = dupload(c, s.hom, b->homothety, n)) ||
      (rc = dupload(c, s.mass, b->mass, n)) || (rc = dupload(c, s.inertia, b->inertia, 3 * n)) ||
      (rc = dupload(c, s.rad, rad.data(), n)) || (rc = dupload(c, s.inv_mi, inv_mi.data(), 4 * n)) || (rc = dupload(c, s.shape, b->shape, n)) ||
      (rc = dupload(c, s.group, b->group, n)) || (rc = dupload(c, s.cluster, b->cluster, n)) ||
      (rc = dupload(c, s.gv_ofs, gv_ofs.data(), n + 1)) || (rc = dupload(c, s.gv_body, gv_body.data(), nv)) ||
      (rc = dalloc(c, s.lv, std::max<int64_t>(nv, 1))) ||
      (rc = dupload(c, s.gv, (const double*)nullptr, 3 * nv)) || (rc = dupload(c, s.gvr, (const float*)nullptr, 3 * nv)) ||
      (rc = dupload(c, s.bobb, (const double*)nullptr, 15 * n)) ||
      (rc = dupload(c, s.bobbf, (const float*)nullptr, 15 * n)) ||
      (rc = dupload(c, s.bbox, (const float*)nullptr, 15 * n)) ||
      (rc = dalloc(c, s.posf, n)) || (rc = dalloc(c, s.rotm, 9 * n)) || (rc = dalloc(c, s.gsum, 6 * n)) ||
      (rc = dalloc(c, s.uv64, 3 * std::max<int64_t>(nv, 1))) || (rc = dalloc(c, s.uvf, std::max<int64_t>(nv, 1))) ||
      (rc = dupload(c, s.baabb, (const float*)nullptr, 6 * n)) ||
      (rc = dupload(c, s.dpos, (const double*)nullptr, 3 * n)) || (rc = dupload(c, s.dq, (const double*)nullptr, 4 * n)) ||
      (rc = dupload(c, s.iofs, (const int64_t*)nullptr, n + 1)) ||
      (rc = dupload(c, s.jofs, (const int64_t*)nullptr, n + 1)) ||
      (rc = dupload(c, s.jsplit, (const int64_t*)nullptr, n)) ||
      (rc = dupload(c, s.if_ofs, (const int64_t*)nullptr, n + 1)) ||
      (rc = dupload(c, s.sph_ofs, sph_ofs.data(), n + 1)) || (rc = dalloc(c, s.sph, sph_ofs[n])) ||
      (rc = dupload(c, s.sph_body, sph_body.data(), std::max<int64_t>(sph_ofs[n], 1))) ||
      (rc = dupload(c, s.is_heavy, (const uint8_t*)nullptr, n)) || (rc = dalloc(c, s.heavy, n)) ||
      (rc = dalloc(c, s.heavy_lazy, n)) || (rc = dalloc(c, s.bnd, n)) || (rc = dalloc(c, s.needres, n)))
    return rc;
  s.nlv = 0;
  s.nheavy = 0;
  s.nheavy_lazy = 0;
  dfree(s.scene_of);
  c.needres_host.assign(n, 1);
  for (int64_t i = 0; i < b->n_driven; i++) c.needres_host[i] = 0;
  CK(cudaMemcpyAsync(s.needres, c.needres_host.data(), n, cudaMemcpyHostToDevice, c.stream));
  if (!c.w.counter) CK(cudaMalloc(&c.w.counter, 64));
  // deltaQ starts as the identity quaternion
  std::vector<double> dq(4 * n, 0.0);
  for (int64_t i = 0; i < n; i++) dq[4 * i] = 1.0;
  CK(cudaMemcpyAsync(s.dq, dq.data(), dq.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (s.bf_kind == RK_BF_VISCOUS_FLUID && c.bf_n != n) {  // its per-body volumes no longer match
    dfree(s.bf_surf);
    s.bf_kind = RK_BF_NONE;
  }
  s.n = n;
  s.n_driven = b->n_driven;
  s.nvert = nv;
  launch_body_verts(s, c.stream);
  c.kernels++;
  CK(cudaGetLastError());
  c.body_shape.assign(b->shape, b->shape + n);
  c.body_hom.assign(b->homothety, b->homothety + n);
  s.ne = 0;
  s.nif = 0;
  c.have_bodies = true;
  return RK_OK;
}

int rk_set_params(rk_ctx* x, const rk_params* p) {
  if (!x || !p || p->ngroup <= 0 || !p->table || !(p->dt > 0.0)) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (p->law < 0 || p->law > 2) return fail(c, RK_ERR_UNSUPPORTED, "unknown force law");
  const int G = p->ngroup;
  std::vector<LawParams> tab((size_t)G * G);
  const double kPi = 3.14159265358979323846;
  for (int g1 = 0; g1 < G; g1++)
    for (int g2 = 0; g2 < G; g2++) {
      LawParams& L = tab[(size_t)g1 * G + g2];
      for (int k = 0; k < 24; k++) L.p[k] = 0.0;
      for (int k = 0; k < RK_NPARAM; k++) L.p[k] = p->table[((size_t)k * G + g1) * G + g2];
      // damping rate of Rockable.cpp:1368-1376, evaluated with the host libm
      double en2 = L.p[RK_P_EN2];
      if (en2 > 0.0 && en2 < 1.0) {
        double logen = 0.5 * log(en2);
        L.p[22] = -logen / sqrt(logen * logen + kPi * kPi);
      } else if (en2 <= 0.0) {
        L.p[22] = 1.0;
      } else {
        L.p[22] = 0.0;
      }
    }
  Scene& s = c.s;
  int rc;
  if ((rc = dupload(c, s.table, tab.data(), (int64_t)tab.size()))) return rc;
  s.ngroup = G;
  s.law = p->law;
  s.params_in_interfaces = p->params_in_interfaces;
  s.dt = p->dt;
  s.dt_2 = 0.5 * p->dt;
  s.dt2_2 = s.dt_2 * p->dt;  // Rockable.cpp:2559-2560
  for (int k = 0; k < 3; k++) s.gravity[k] = p->gravity[k];
  s.DVerlet = p->DVerlet;
  s.dVerlet = p->dVerlet;
  s.num_damp = p->numerical_damping;
  s.dynamic_nl = p->dynamic_update_nl;
  s.disp_update = p->disp_update_nl;
  s.angle_update = p->angle_update_nl;
  c.t = p->t;
  c.interVerlet = p->interVerlet;
  c.interVerletC = p->interVerletC;
  c.have_params = true;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_upload_entries(rk_ctx* x, const rk_entries* e) {
  if (!x || !e || e->n < 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies before the entries");
  const int64_t n = e->n;
  int rc;
  if ((rc = ensure_entry_capacity(c, c.cur, n))) return rc;
  bind_entries(c);
  Scene& s = c.s;
  s.ne = n;
  if (n > 0) {
    int* d_t = nullptr;
    int* d_is = nullptr;
    int* d_js = nullptr;
    int* d_bad = nullptr;
    if ((rc = dupload(c, d_t, e->type, n)) || (rc = dupload(c, d_is, e->isub, n)) ||
        (rc = dupload(c, d_js, e->jsub, n)) || (rc = dupload(c, d_bad, (const int*)nullptr, 1)))
      return rc;
    CK(cudaMemcpyAsync(s.ei, e->i, n * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.ej, e->j, n * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.dn, e->dn, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.fn, e->fn, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.ft, e->ft, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.mom, e->mom, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.damp, e->damp, n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    if (e->bond) CK(cudaMemcpyAsync(s.bond, e->bond, n * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    else CK(cudaMemsetAsync(s.bond, 0xff, n * sizeof(int), c.stream));
    CK(cudaMemsetAsync(s.gn, 0, 3 * n * sizeof(double), c.stream));
    CK(cudaMemsetAsync(s.gpos, 0, 3 * n * sizeof(double), c.stream));
    CK(cudaMemsetAsync(s.gvel, 0, 3 * n * sizeof(double), c.stream));
    k_upload_keys<<<nblk(n, 256), 256, 0, c.stream>>>(s, n, d_t, d_is, d_js, d_bad);
    k_check_sorted<<<nblk(n, 256), 256, 0, c.stream>>>(s.ekey, n, d_bad);
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    dfree(d_t); dfree(d_is); dfree(d_js); dfree(d_bad);
    if (bad == 1) { s.ne = 0; return fail(c, RK_ERR_ARG, "entry index out of range"); }
    if (bad == 2) { s.ne = 0; return fail(c, RK_ERR_ARG, "entries must be sorted by key and unique"); }
  }
  return build_index(c);
}

int rk_upload_interfaces(rk_ctx* x, const rk_interfaces* f) {
  if (!x || !f || f->n < 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies before the interfaces");
  const int64_t n = f->n, N = c.s.n;
  std::vector<int64_t> ofs(N + 1, 0);
  for (int64_t k = 0; k < n; k++) {
    if (f->i[k] < 0 || f->i[k] >= N || f->j[k] < 0 || f->j[k] >= N) return fail(c, RK_ERR_ARG, "interface body out of range");
    if (k > 0 && (f->i[k] < f->i[k - 1] || (f->i[k] == f->i[k - 1] && f->j[k] <= f->j[k - 1])))
      return fail(c, RK_ERR_ARG, "interfaces must be sorted by (i, j) and unique");
    ofs[f->i[k] + 1]++;
  }
  for (int64_t b = 0; b < N; b++) ofs[b + 1] += ofs[b];
  Scene& s = c.s;
  int rc;
  if ((rc = dupload(c, s.if_i, f->i, n)) || (rc = dupload(c, s.if_j, f->j, n)) ||
      (rc = dupload(c, s.if_dn0, f->dn0, n)) || (rc = dupload(c, s.if_par, f->params, 8 * n)) ||
      (rc = dupload(c, s.if_inner, f->is_inner, n)) || (rc = dupload(c, s.if_broken, (const uint8_t*)nullptr, n)) ||
      (rc = dupload(c, s.if_break, (const uint8_t*)nullptr, n)) || (rc = dupload(c, s.if_ofs, ofs.data(), N + 1)))
    return rc;
  s.nif = n;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_set_controls(rk_ctx* x, const rk_control* cs, int32_t n, const rk_servo* servo) {
  if (!x || n < 0 || (n > 0 && !cs)) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies before the controls");
  std::vector<Control> v(n);
  for (int k = 0; k < n; k++) {
    if (cs[k].body < 0 || cs[k].body >= c.s.n) return fail(c, RK_ERR_ARG, "control body out of range");
    v[k].type = cs[k].type;
    v[k].body = cs[k].body;
    v[k].value = cs[k].value;
    for (int d = 0; d < 3; d++) v[k].vec[d] = cs[k].vec[d];
  }
  Scene& s = c.s;
  int rc;
  if ((rc = dupload(c, s.controls, v.data(), n))) return rc;
  s.ncontrols = n;
  for (int64_t i = 0; i < s.n; i++) c.needres_host[i] = i >= s.n_driven ? 1 : 0;
  for (auto& q : v)
    if (q.type >= RK_X_FOR && q.type != RK_XYZROT_VEL) c.needres_host[q.body] = 1;
  CK(cudaMemcpyAsync(s.needres, c.needres_host.data(), s.n, cudaMemcpyHostToDevice, c.stream));
  if (s.ne > 0 && (rc = heavy_list(c))) return rc;
  s.servo_kind = 0;
  if (servo && servo->kind == 1) {
    if (servo->icontr < 0 || servo->icontr + 5 >= n) return fail(c, RK_ERR_ARG, "servo control index out of range");
    for (int k = 0; k < 6; k++) {
      if (servo->walls[k] < 0 || servo->walls[k] >= c.s.n) return fail(c, RK_ERR_ARG, "servo wall out of range");
      s.servo_walls[k] = servo->walls[k];
    }
    s.servo_kind = 1;
    s.servo_icontr = servo->icontr;
    s.servo_p = servo->pressure;
  } else if (servo && servo->kind != 0) {
    return fail(c, RK_ERR_UNSUPPORTED, "only the tritriIsostaticCompression servo is supported");
  }
  c.controls = v;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}


int rk_set_body_force(rk_ctx* x, int kind, const double* p, int32_t np, const double* body_volume) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies before the body force");
  static const int want[4] = {0, 4, 7, 1};
  if (kind < RK_BF_NONE || kind > RK_BF_VISCOUS_FLUID) return fail(c, RK_ERR_ARG, "unknown body force kind");
  if (np != want[kind] || (np > 0 && !p)) return fail(c, RK_ERR_ARG, "wrong number of body force parameters");
  if (kind == RK_BF_VISCOUS_FLUID && !body_volume) return fail(c, RK_ERR_ARG, "the viscous fluid needs body volumes");
  Scene& s = c.s;
  double bf[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (kind == RK_BF_ATTRACTING_POINT) {
    for (int k = 0; k < 4; k++) bf[k] = p[k];
  } else if (kind == RK_BF_PREFERRED_DIRECTION) {  // read(): both axes normalised, Kr = 2 momentMax / pi
    V3 a = v3(p[0], p[1], p[2]), b = v3(p[3], p[4], p[5]);
    normalize(a);
    normalize(b);
    bf[0] = a.x; bf[1] = a.y; bf[2] = a.z;
    bf[3] = b.x; bf[4] = b.y; bf[5] = b.z;
    bf[6] = 2.0 * p[6] / M_PI;
    bf[7] = M_PI;
  } else if (kind == RK_BF_VISCOUS_FLUID) {  // the drag coefficient 0.47 of a sphere, halved
    bf[0] = 0.5 * 0.47;
    bf[1] = p[0];
    std::vector<double> surf(s.n);
    for (int64_t b = 0; b < s.n; b++) surf[b] = std::pow(body_volume[b], 2.0 / 3.0);
    int rc;
    dfree(s.bf_surf);
    if ((rc = dupload(c, s.bf_surf, surf.data(), s.n))) return rc;
    CK(cudaStreamSynchronize(c.stream));
  }
  if (kind != RK_BF_VISCOUS_FLUID) dfree(s.bf_surf);
  for (int k = 0; k < 8; k++) s.bf[k] = bf[k];
  s.bf_kind = kind;
  c.bf_n = s.n;
  return RK_OK;
}

static int ready(Ctx& c) {
  if (!c.have_shapes || !c.have_bodies || !c.have_params)
    return fail(c, RK_ERR_STATE, "shapes, bodies and parameters must be uploaded first");
  return 0;
}

static int skin_alloc(Ctx& c) {
  Skin& k = c.skin;
  Scene& s = c.s;
  const int np = mlp_num_params();
  int rc;
  if (k.ref_pos && k.nalloc < s.n) {  // bodies re-uploaded with a larger count
    dfree(k.ref_pos); dfree(k.ref_q); dfree(k.rsw); dfree(k.maxd); dfree(k.path); dfree(k.flag);
    k.ref_pos = nullptr;
    if ((rc = dalloc(c, k.ref_pos, 3 * s.n)) || (rc = dalloc(c, k.ref_q, 4 * s.n)) || (rc = dalloc(c, k.rsw, s.n)) ||
        (rc = dalloc(c, k.maxd, s.n)) || (rc = dalloc(c, k.path, s.n)) || (rc = dalloc(c, k.flag, s.n)))
      return rc;
    k.nalloc = s.n;
  }
  if (!k.ref_pos) {
    k.nalloc = s.n;
    if ((rc = dalloc(c, k.ref_pos, 3 * s.n)) || (rc = dalloc(c, k.ref_q, 4 * s.n)) || (rc = dalloc(c, k.rsw, s.n)) ||
        (rc = dalloc(c, k.d_guard, 16)) || (rc = dalloc(c, k.d_hist, 64)) || (rc = dalloc(c, k.maxd, s.n)) ||
        (rc = dalloc(c, k.path, s.n)) ||
        (rc = dalloc(c, k.flag, s.n)) || (rc = dalloc(c, k.master, np)) || (rc = dalloc(c, k.m, np)) ||
        (rc = dalloc(c, k.v, np)) || (rc = dalloc(c, k.grad, np)) || (rc = dalloc(c, k.loss, 1)) ||
        (rc = dalloc(c, k.X, 16 * mlp_max_batch())) || (rc = dalloc(c, k.T, 2 * mlp_max_batch())) ||
        (rc = dalloc(c, k.io, 32)))
      return rc;
    char* wbuf = nullptr;
    CK(cudaMalloc(&wbuf, 2 * (size_t)np));
    k.w = wbuf;
    CK(cudaMallocHost(&k.h_guard, 64));
    CK(cudaMalloc(&k.d_ctl, 32 * sizeof(unsigned int)));
    CK(cudaMallocHost(&k.h_ctl, 32 * sizeof(unsigned int)));
    CK(cudaEventCreateWithFlags(&k.bev, cudaEventDisableTiming));
    CK(cudaEventCreate(&k.ea));
    CK(cudaEventCreate(&k.eb));
  }
  return 0;
}

int rk_mlp_num_params(void) { return mlp_num_params(); }

int rk_mlp_set_params(rk_ctx* x, const float* p) {
  if (!x || !p) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies first");
  int rc;
  if ((rc = skin_alloc(c))) return rc;
  Skin& k = c.skin;
  CK(cudaMemcpyAsync(k.master, p, 4 * (size_t)mlp_num_params(), cudaMemcpyHostToDevice, c.stream));
  launch_mlp_to_half(k.master, k.w, c.stream);
  CK(cudaMemsetAsync(k.m, 0, 4 * (size_t)mlp_num_params(), c.stream));
  CK(cudaMemsetAsync(k.v, 0, 4 * (size_t)mlp_num_params(), c.stream));
  k.adam_step = 0;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_mlp_get_params(rk_ctx* x, float* p) {
  if (!x || !p) return RK_ERR_ARG;
  Ctx& c = x->c;
  if (!c.skin.master) return fail(c, RK_ERR_STATE, "no network");
  CK(cudaMemcpyAsync(p, c.skin.master, 4 * (size_t)mlp_num_params(), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_mlp_forward(rk_ctx* x, const float* in, float* out) {
  if (!x || !in || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  if (!c.skin.master) return fail(c, RK_ERR_STATE, "no network");
  Skin& k = c.skin;
  CK(cudaMemcpyAsync(k.io, in, 64, cudaMemcpyHostToDevice, c.stream));
  launch_mlp_infer(k.w, k.io, k.io + 16, c.stream);
  CK(cudaMemcpyAsync(out, k.io + 16, 8, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_mlp_gradient(rk_ctx* x, const float* X, const float* T, int32_t nb, float* grad, float* loss) {
  if (!x || !X || !T || nb <= 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  if (!c.skin.master) return fail(c, RK_ERR_STATE, "no network");
  if (nb > mlp_max_batch()) return fail(c, RK_ERR_CAPACITY, "batch larger than 128");
  Skin& k = c.skin;
  CK(cudaMemcpyAsync(k.X, X, 64 * (size_t)nb, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(k.T, T, 8 * (size_t)nb, cudaMemcpyHostToDevice, c.stream));
  launch_mlp_grad(k.w, k.X, k.T, nb, k.grad, k.loss, c.stream);
  if (grad) CK(cudaMemcpyAsync(grad, k.grad, 4 * (size_t)mlp_num_params(), cudaMemcpyDeviceToHost, c.stream));
  if (loss) CK(cudaMemcpyAsync(loss, k.loss, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  CK(cudaGetLastError());
  return RK_OK;
}

int rk_set_skin(rk_ctx* x, const rk_skin_config* cfg) {
  if (!x || !cfg) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  int rc;
  if ((rc = ready(c))) return rc;
  Skin& k = c.skin;
  if (!cfg->enabled) {
    k.on = false;
    skin_bind(c, false);
    c.s.near_geometric = 0;
    return RK_OK;
  }
  if (!(cfg->skin_min > 0.0) || cfg->skin_max < cfg->skin_min || cfg->interval_min < 1 ||
      cfg->interval_max < cfg->interval_min || !(cfg->dverlet_ratio >= 1.0) || !(cfg->partial_fraction >= 0.0) ||
      cfg->partial_fraction > 1.0)
    return fail(c, RK_ERR_ARG, "invalid skin configuration");
  if ((rc = skin_alloc(c))) return rc;
  Scene& s = c.s;
  k.cfg = *cfg;
  // swing radius of every body (largest vertex distance, scaled)
  std::vector<float> rsw(s.n);
  for (int64_t b = 0; b < s.n; b++) rsw[b] = (float)(c.body_hom[b] * c.shape_vmax[c.body_shape[b]] * (1.0 + 1e-6));
  CK(cudaMemcpyAsync(k.rsw, rsw.data(), rsw.size() * 4, cudaMemcpyHostToDevice, c.stream));
  // network: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) from the seed, zero biases
  const int np = mlp_num_params();
  std::vector<float> p(np, 0.f);
  uint64_t st = cfg->seed ? cfg->seed : 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  // (the output layer starts at zero: see the prediction in skin_rebuild)
  const int layers[3][3] = {{0, 64, 16}, {64 * 16 + 64, 64, 64}, {64 * 16 + 64 + 64 * 64 + 64, 2, 64}};
  for (auto& L : layers) {
    double a = L[1] == 2 ? 0.0 : 1.0 / std::sqrt((double)L[2]);
    for (int q = 0; q < L[1] * L[2]; q++) p[L[0] + q] = (float)((2.0 * rnd() - 1.0) * a);
  }
  CK(cudaMemcpyAsync(k.master, p.data(), 4 * (size_t)np, cudaMemcpyHostToDevice, c.stream));
  launch_mlp_to_half(k.master, k.w, c.stream);
  CK(cudaMemsetAsync(k.m, 0, 4 * (size_t)np, c.stream));
  CK(cudaMemsetAsync(k.v, 0, 4 * (size_t)np, c.stream));
  k.adam_step = 0;
  k.rx.clear();
  k.ry.clear();
  k.rhead = 0;
  k.have_prev = false;
  k.skin = std::min(cfg->skin_max, std::max(cfg->skin_min, s.dVerlet));
  k.interval = cfg->interval_min;
  k.since = 0;
  k.rebuilds = k.forced = k.scheduled = 0;
  k.partial = k.partial_bodies = k.partial_since_global = 0;
  k.rebuild_bp_ms = k.rebuild_var_ms = 0.0;
  k.alpha = 1.6;
  k.step_ms = k.rebuild_ms = 0.0;
  for (double& r : k.rates) r = 0.0;
  s.dVerlet = k.skin;
  s.DVerlet = cfg->dverlet_ratio * k.skin;
  for (cudaEvent_t* e : {&k.nev[0], &k.nev[1], &k.pa, &k.pb, &k.gev[0], &k.gev[1]})
    if (!*e) CK(cudaEventCreate(e));
  k.gslot = 0;
  k.have_pred = false;
  k.narrow_acc = k.partial_ms = 0.0;
  k.narrow_cnt = k.partial_in_window = 0;
  k.on = true;
  skin_bind(c, true);
  s.near_geometric = cfg->exact_contacts ? 1 : 0;
  // start from a fresh list built with the initial skin
  launch_glob_vertices(s, c.stream, true);
  if ((rc = rebuild_nl(c))) return rc;
  launch_skin_reset(s, nullptr, k.ref_pos, k.ref_q, k.maxd, k.path, c.stream);
  CK(cudaEventRecord(k.ea, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_get_skin_stats(rk_ctx* x, rk_skin_stats* o) {
  if (!x || !o) return RK_ERR_ARG;
  Skin& k = x->c.skin;
  o->rebuilds = k.rebuilds;
  o->forced = k.forced;
  o->scheduled = k.scheduled;
  o->skin = k.skin;
  o->interval = k.interval;
  o->last_rate = k.last_rate;
  o->predicted_rate = k.pred_rate;
  o->loss = k.last_loss;
  o->partial = k.partial;
  o->partial_bodies = k.partial_bodies;
  o->train_steps = (int64_t)k.adam_step;
  o->windows = (int64_t)k.rx.size();
  o->rebuild_ms = k.rebuild_ms;
  o->partial_ms = k.partial_ms;
  return RK_OK;
}

int rk_set_broadphase(rk_ctx* x, int mode) {
  if (!x || mode < 0 || mode > 2) return RK_ERR_ARG;
  x->c.broadphase = mode;
  return RK_OK;
}

int rk_set_scenes(rk_ctx* x, const int32_t* scene_of) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies first");
  Scene& s = c.s;
  if (!scene_of) {
    dfree(s.scene_of);
    return RK_OK;
  }
  int rc;
  if ((rc = dupload(c, s.scene_of, scene_of, s.n))) return rc;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_set_autotune(rk_ctx* x, int rounds) {
  if (!x || rounds < 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  for (int k = 0; k < 8; k++)
    if (!c.tev[k]) CK(cudaEventCreate(&c.tev[k]));
  for (auto& row : c.tune_ms)
    for (double& v : row) v = 0.0;
  c.tune_total = c.tune_left = kNumCand * (int64_t)rounds;
  return RK_OK;
}

int rk_get_block_sizes(const rk_ctx* x, int32_t* tpb) {
  if (!x || !tpb) return RK_ERR_ARG;
  const int def[4] = {128, 128, 256, 128};
  for (int k = 0; k < 4; k++) tpb[k] = x->c.s.tpb[k] > 0 ? x->c.s.tpb[k] : def[k];
  return RK_OK;
}

int rk_set_graphs(rk_ctx* x, int on) {
  if (!x) return RK_ERR_ARG;
  x->c.use_graphs = on ? 1 : 0;
  return RK_OK;
}

int rk_get_graph_stats(const rk_ctx* x, int64_t* captures, int64_t* replays) {
  if (!x) return RK_ERR_ARG;
  if (captures) *captures = x->c.graph_captures;
  if (replays) *replays = x->c.graph_replays;
  return RK_OK;
}

int rk_set_form(rk_ctx* x, int form) {
  if (!x) return RK_ERR_ARG;
  if (form != RK_FORM_FP64 && form != RK_FORM_MIXED) return fail(x->c, RK_ERR_UNSUPPORTED, "unknown form");
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const int fb = form == RK_FORM_MIXED ? 1 : 0;
  c.form = form;
  if (c.s.fast_body != fb) {
    c.s.fast_body = fb;
    // the resultant kernels split the heavy bodies differently (is_heavy 3)
    if (c.s.ne > 0) {
      const int rc = heavy_list(c);
      if (rc) return rc;
    }
  }
  return RK_OK;
}

int rk_set_record_geometry(rk_ctx* x, int on) {
  if (!x) return RK_ERR_ARG;
  x->c.s.record_geom = on ? 1 : 0;
  return RK_OK;
}


// Rockable::accelerations without a time increment (the load-time step).
int rk_accelerations(rk_ctx* x) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  int rc;
  if ((rc = ready(c))) return rc;
  Scene& s = c.s;
  CK(cudaMemsetAsync(s.flags + FLAG_NACTIVE, 0, sizeof(unsigned long long), c.stream));
  launch_glob_vertices(s, c.stream, true);
  if (c.form == RK_FORM_MIXED) launch_narrow_force_mixed(s, c.stream);
  else launch_narrow_force(s, c.stream);
  launch_gather_heavy(s, c.stream);
  launch_gather_accel(s, 0, c.stream);
  launch_breakage(s, c.stream);
  c.forces_stale = s.nheavy_lazy > 0;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_update_nl(rk_ctx* x) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  int rc;
  if ((rc = ready(c))) return rc;
  settle_lazy_forces(c);
  launch_glob_vertices(c.s, c.stream, true);
  if ((rc = rebuild_nl(c))) return rc;
  c.nl_updates++;
  if (c.skin.on) {
    // the list now holds the current state (which the host may have moved):
    // the skin's guard restarts from it, as after a full skin rebuild
    Skin& k = c.skin;
    c.kernels += launch_skin_reset(c.s, nullptr, k.ref_pos, k.ref_q, k.maxd, k.path, c.stream);
    k.since = 0;
    k.partial_since_global = 0;
    k.have_pred = false;
  }
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

// nsteps passes of the loop body of Rockable::integrate (Rockable.cpp:2584-2736)
// without conf output: t += dt, velocity-Verlet step, NL update when the
// interVerlet counter elapsed or an update was requested, dynamic guard.
int rk_step(rk_ctx* x, int64_t nsteps, rk_step_report* rep) {
  if (!x || nsteps < 0) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  int rc;
  if ((rc = ready(c))) return rc;
  Scene& s = c.s;
  const bool need_flags = s.dynamic_nl != 0 || s.nif > 0;
  int64_t k0 = c.kernels, nl0 = c.nl_updates;
  c.skin.have_pred = false;  // the state may have been changed since the last call (uploads)
  CK(cudaEventRecord(c.ev0, c.stream));
  for (int64_t it = 0; it < nsteps; it++) {
    const bool tuning = c.tune_left > 0 && !c.profiling;
    const bool graphed = c.use_graphs && !c.profiling && !tuning;
    if (graphed && c.skin.on && c.skin.d_ctl && guard_pipelined(c)) {
      // the skin's decisions taken on the device, a batch of steps per round trip
      int64_t ex = 0;
      if ((rc = skin_batch(c, nsteps - it, &ex))) return rc;
      it += ex - 1;
      continue;
    }
    c.t += s.dt;
    c.interVerletC += s.dt;
    c.more_steps_follow = it + 1 < nsteps;
    if (graphed) {
      if ((rc = step_graph(c))) return rc;
    } else {
      CK(cudaMemsetAsync(s.flags + FLAG_NACTIVE, 0, sizeof(unsigned long long), c.stream));
    }
    int ph = 0;
    auto mark = [&](int phase, bool end) {
      if (c.profiling) cudaEventRecord(c.pev[2 * phase + (end ? 1 : 0)], c.stream);
    };
    auto phase = [&](int p, int launched) {
      (void)ph;
      c.kernels += launched;
      if (c.profiling && launched) {
        mark(p, true);
        cudaEventSynchronize(c.pev[2 * p + 1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c.pev[2 * p], c.pev[2 * p + 1]);
        c.prof_ms[p] += ms;
        c.prof_n[p] += launched;
      }
    };
    if (tuning) {
      if ((rc = tune_step(c))) return rc;
    } else if (!graphed) {
      mark(0, false); phase(0, launch_controls_pre(s, c.stream));
      mark(1, false); phase(1, launch_drift(s, c.stream));
      mark(2, false); phase(2, launch_glob_vertices(s, c.stream));
      mark(3, false);
      const bool ntimed = c.skin.on && c.skin.nev[0];
      if (ntimed) cudaEventRecord(c.skin.nev[0], c.stream);
      phase(3, c.form == RK_FORM_MIXED ? launch_narrow_force_mixed(s, c.stream) : launch_narrow_force(s, c.stream));
      if (ntimed) cudaEventRecord(c.skin.nev[1], c.stream);
      c.skin.narrow_timed = ntimed;
      mark(4, false); phase(4, launch_gather_heavy(s, c.stream) + launch_gather_accel(s, 1, c.stream));
      mark(5, false); phase(5, launch_breakage(s, c.stream));
    }
    c.forces_stale = s.nheavy_lazy > 0;
    if (c.skin.on) {
      if ((rc = skin_after_step(c))) return rc;
      c.steps++;
      continue;
    }
    bool need = false;
    if (need_flags) {
      if ((rc = read_flags(c))) return rc;
      need = c.h_flags[FLAG_NEED_UPDATE] != 0ull;
    }
    if (need || c.interVerletC >= c.interVerlet - s.dt_2) {
      settle_before_update(c);
      mark(6, false);
      int64_t k1 = c.kernels;
      if ((rc = rebuild_nl(c))) return rc;
      int64_t launched = c.kernels - k1;
      c.kernels = k1;
      phase(6, (int)launched);
      c.nl_updates++;
      if (!need) c.interVerletC = 0.0;
      else CK(cudaMemsetAsync(s.flags + FLAG_NEED_UPDATE, 0, sizeof(unsigned long long), c.stream));
    }
    if (s.dynamic_nl) { mark(7, false); phase(7, launch_guard(s, c.stream)); }
    c.steps++;
  }
  c.more_steps_follow = false;
  CK(cudaEventRecord(c.ev1, c.stream));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(c.ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  c.last_ms = ms;
  c.last_kernels = c.kernels - k0;
  if (rep) {
    if ((rc = read_flags(c))) return rc;
    rep->steps_done = nsteps;
    rep->nl_updates = c.nl_updates - nl0;
    rep->n_entries = s.ne;
    rep->n_active = (int64_t)c.h_flags[FLAG_NACTIVE];
    rep->n_broken = (int64_t)c.h_flags[FLAG_NBROKEN];
    rep->t = c.t;
  }
  return RK_OK;
}

int rk_synchronize(rk_ctx* x) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int64_t rk_num_bodies(const rk_ctx* x) { return x ? x->c.s.n : -1; }
int64_t rk_num_entries(const rk_ctx* x) { return x ? x->c.s.ne : -1; }
int64_t rk_num_interfaces(const rk_ctx* x) { return x ? x->c.s.nif : -1; }

int rk_download_bodies(rk_ctx* x, double* pos, double* vel, double* acc, double* Q, double* vrot, double* arot,
                       double* force, double* moment) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  if (force || moment) settle_lazy_forces(c);
  const size_t n3 = 3 * (size_t)s.n * sizeof(double);
  if (pos) CK(cudaMemcpyAsync(pos, s.pos, n3, cudaMemcpyDeviceToHost, c.stream));
  if (vel) CK(cudaMemcpyAsync(vel, s.vel, n3, cudaMemcpyDeviceToHost, c.stream));
  if (acc) CK(cudaMemcpyAsync(acc, s.acc, n3, cudaMemcpyDeviceToHost, c.stream));
  if (Q) CK(cudaMemcpyAsync(Q, s.Q, 4 * (size_t)s.n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  if (vrot) CK(cudaMemcpyAsync(vrot, s.vrot, n3, cudaMemcpyDeviceToHost, c.stream));
  if (arot) CK(cudaMemcpyAsync(arot, s.arot, n3, cudaMemcpyDeviceToHost, c.stream));
  if (force) CK(cudaMemcpyAsync(force, s.force, n3, cudaMemcpyDeviceToHost, c.stream));
  if (moment) CK(cudaMemcpyAsync(moment, s.moment, n3, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

__global__ void k_unpack_tsub(const uint32_t* ts, int64_t n, int* t, int* isub, int* jsub) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  t[e] = tsub_type(ts[e]);
  isub[e] = tsub_isub(ts[e]);
  jsub[e] = tsub_jsub(ts[e]);
}

int rk_set_shape_names(rk_ctx* x, const char* const* names, int32_t n) {
  if (!x || n < 0 || (n > 0 && !names)) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_shapes || n != c.s.nshapes) return fail(c, RK_ERR_ARG, "one name per uploaded shape");
  std::vector<int> ofs(n + 1, 0);
  std::string all;
  for (int k = 0; k < n; k++) {
    if (!names[k]) return fail(c, RK_ERR_ARG, "a shape name is missing");
    all += names[k];
    ofs[k + 1] = (int)all.size();
  }
  int rc;
  if ((rc = dupload(c, c.name_chars, all.data(), std::max<int64_t>((int64_t)all.size(), 1))) ||
      (rc = dupload(c, c.name_ofs, ofs.data(), n + 1)))
    return rc;
  CK(cudaStreamSynchronize(c.stream));
  c.have_names = true;
  return RK_OK;
}

int rk_format_conf(rk_ctx* x, int32_t prec, char* buf, int64_t cap, int64_t* particles_len,
                   int64_t* interactions_len, int64_t* n_active) {
  if (!x || prec < 0 || prec > 17) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies || !c.have_names) return fail(c, RK_ERR_STATE, "upload the bodies and the shape names first");
  Scene& s = c.s;
  cudaStream_t st = c.stream;
  const int64_t nb = s.n, ne = s.ne;
  // bodies: one slot each, then the active entries: flags, their positions
  char* slots = nullptr;
  int64_t *lens = nullptr, *ofs = nullptr, *flag = nullptr;
  void* tmp = nullptr;
  char* out = nullptr;
  int rc = RK_OK;
  int64_t lp = 0, li = 0, na = 0;
  auto cleanup = [&]() {
    dfree(slots); dfree(lens); dfree(ofs); dfree(flag); dfree(out);
    if (tmp) cudaFree(tmp);
  };
  const int64_t nmax = std::max<int64_t>(nb, ne) + 1;
  if ((rc = dalloc(c, lens, nmax)) || (rc = dalloc(c, ofs, nmax)) || (rc = dalloc(c, flag, ne + 1))) {
    cleanup();
    return rc;
  }
  if (cudaMalloc(&tmp, scan_temp_bytes(nmax)) != cudaSuccess) {
    cleanup();
    return fail(c, RK_ERR_CUDA, "no device memory for the conf text");
  }
  if (ne > 0) {
    k_conf_active<<<nblk(ne, 256), 256, 0, st>>>(s, flag);
    cudaMemsetAsync(flag + ne, 0, sizeof(int64_t), st);
    exclusive_scan_i64(flag, flag, ne + 1, tmp, st);
    cudaMemcpyAsync(&na, flag + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      cleanup();
      return fail(c, RK_ERR_CUDA, "conf text: active entries");
    }
  }
  // the two sections, one after the other
  for (int part = 0; part < 2; part++) {
    const int64_t nl = part == 0 ? nb : na;
    const int slot = part == 0 ? kConfBodySlot : kConfEntrySlot;
    int64_t& len = part == 0 ? lp : li;
    if (nl == 0) continue;
    dfree(slots);
    if ((rc = dalloc(c, slots, nl * (int64_t)slot))) break;
    if (part == 0) k_conf_bodies<<<nblk(nb, 128), 128, 0, st>>>(s, c.name_chars, c.name_ofs, prec, slots, lens);
    else k_conf_entries<<<nblk(ne, 128), 128, 0, st>>>(s, flag, prec, slots, lens);
    cudaMemsetAsync(lens + nl, 0, sizeof(int64_t), st);
    exclusive_scan_i64(lens, ofs, nl + 1, tmp, st);
    cudaMemcpyAsync(&len, ofs + nl, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) { rc = fail(c, RK_ERR_CUDA, "conf text: formatting"); break; }
    const int64_t at = part == 0 ? 0 : lp;
    if (buf && at + len <= cap) {
      dfree(out);
      if ((rc = dalloc(c, out, std::max<int64_t>(len, 1)))) break;
      k_conf_pack<<<nblk(nl * 32, 256), 256, 0, st>>>(slots, slot, ofs, lens, nl, out);
      if (cudaMemcpyAsync(buf + at, out, (size_t)len, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        rc = fail(c, RK_ERR_CUDA, "conf text: copy");
        break;
      }
    }
  }
  cleanup();
  if (rc) return rc;
  if (particles_len) *particles_len = lp;
  if (interactions_len) *interactions_len = li;
  if (n_active) *n_active = na;
  if (buf && lp + li > cap) return fail(c, RK_ERR_CAPACITY, "the conf text needs a larger buffer");
  return RK_OK;
}

// ------------------------------------------------------- data extractors ----
static int ext_scratch(Ctx& c) {
  int rc;
  if (!c.ext_part && (rc = dalloc(c, c.ext_part, 8 * kExtBlocks))) return rc;
  if (!c.ext_u && (rc = dalloc(c, c.ext_u, 8))) return rc;
  return 0;
}

int rk_extract_mean_velocity(rk_ctx* x, double* mean) {
  if (!x || !mean) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const Scene& s = c.s;
  if (s.n <= 0) return fail(c, RK_ERR_STATE, "no bodies");
  int rc;
  if ((rc = ext_scratch(c))) return rc;
  k_ext_speed<<<kExtBlocks, kExtThreads, 0, c.stream>>>(s, c.ext_part);
  c.kernels++;
  double part[kExtBlocks];
  CK(cudaMemcpyAsync(part, c.ext_part, sizeof part, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  double m = 0.0;
  for (int k = 0; k < kExtBlocks; k++) m += part[k];
  *mean = m / (double)s.n;
  return RK_OK;
}

int rk_extract_dn_stat(rk_ctx* x, double* out) {
  if (!x || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const Scene& s = c.s;
  double mn = 1e20, mx = -1e20, sum = 0.0, sneg = 0.0, nneg = 0.0, spos = 0.0, npos = 0.0;
  double pmin[3] = {0.0, 0.0, 0.0};
  if (s.ne > 0) {
    int rc;
    if ((rc = ext_scratch(c))) return rc;
    k_ext_dn<<<kExtBlocks, kExtThreads, 0, c.stream>>>(s, c.ext_part);
    c.kernels++;
    double part[8 * kExtBlocks];
    CK(cudaMemcpyAsync(part, c.ext_part, sizeof part, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    int64_t imn = INT64_MAX;
    for (int k = 0; k < kExtBlocks; k++) {
      const double* p = part + 8 * k;
      sum += p[0];
      sneg += p[1];
      nneg += p[2];
      spos += p[3];
      npos += p[4];
      const int64_t ik = p[6] >= 9.2e18 ? INT64_MAX : (int64_t)p[6];
      if (ik != INT64_MAX && (p[5] < mn || (!(mn < p[5]) && ik < imn))) {
        mn = p[5];
        imn = ik;
      }
      if (p[7] > mx) mx = p[7];
    }
    if (imn != INT64_MAX) {
      CK(cudaMemcpyAsync(pmin, s.gpos + 3 * imn, sizeof pmin, cudaMemcpyDeviceToHost, c.stream));
      CK(cudaStreamSynchronize(c.stream));
    }
  }
  if (nneg > 0.0) sneg /= nneg;
  if (npos > 0.0) spos /= npos;
  if (nneg > 0.0 || npos > 0.0) sum /= (nneg + npos);
  const double o[10] = {mn, mx, sum, sneg, spos, nneg, npos, pmin[0], pmin[1], pmin[2]};
  for (int k = 0; k < 10; k++) out[k] = o[k];
  return RK_OK;
}

int rk_extract_cluster_aabb(rk_ctx* x, int32_t cluster, double* out) {
  if (!x || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const Scene& s = c.s;
  for (int k = 0; k < 7; k++) out[k] = 0.0;
  if (s.nvert <= 0) return RK_OK;
  int rc;
  if ((rc = ext_scratch(c))) return rc;
  const unsigned long long init[7] = {~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull, 0ull};
  CK(cudaMemcpyAsync(c.ext_u, init, sizeof init, cudaMemcpyHostToDevice, c.stream));
  k_ext_cluster_box<<<nblk(s.nvert, 256), 256, 0, c.stream>>>(s, cluster, c.ext_u);
  c.kernels++;
  unsigned long long r[7];
  CK(cudaMemcpyAsync(r, c.ext_u, sizeof r, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (r[6]) {  // else the zero box of an empty cluster, as the reference prints it
    out[0] = 1.0;
    for (int k = 0; k < 6; k++) out[1 + k] = ext_unord(r[k]);
  }
  return RK_OK;
}

int rk_extract_duo_balance(rk_ctx* x, int32_t i, int32_t j, int64_t* out) {
  if (!x || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  const Scene& s = c.s;
  for (int k = 0; k < 4; k++) out[k] = 0;
  if (s.ne <= 0) return RK_OK;
  int rc;
  if ((rc = ext_scratch(c))) return rc;
  CK(cudaMemsetAsync(c.ext_u, 0, 4 * sizeof(unsigned long long), c.stream));
  k_ext_duo<<<nblk(s.ne, 256), 256, 0, c.stream>>>(s, i, j, c.ext_u);
  c.kernels++;
  unsigned long long r[4];
  CK(cudaMemcpyAsync(r, c.ext_u, sizeof r, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (int k = 0; k < 4; k++) out[k] = (int64_t)r[k];
  return RK_OK;
}

int rk_download_body(rk_ctx* x, int64_t b, double* out) {
  if (!x || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (b < 0 || b >= c.s.n) return fail(c, RK_ERR_ARG, "body index out of range");
  settle_lazy_forces(c);  // a driven body's resultant summed on demand
  int rc;
  if ((rc = ext_scratch(c))) return rc;
  k_ext_body<<<1, 32, 0, c.stream>>>(c.s, b, c.ext_part);
  c.kernels++;
  CK(cudaMemcpyAsync(out, c.ext_part, 25 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_download_contributions(rk_ctx* x, double* f, double* mi, double* mj) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  if (s.ne == 0) return RK_OK;
  const size_t d3 = 3 * (size_t)s.ne * sizeof(double);
  if (f) CK(cudaMemcpyAsync(f, s.cf, d3, cudaMemcpyDeviceToHost, c.stream));
  if (mi) CK(cudaMemcpyAsync(mi, s.cmi, d3, cudaMemcpyDeviceToHost, c.stream));
  if (mj) CK(cudaMemcpyAsync(mj, s.cmj, d3, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_download_entries(rk_ctx* x, int32_t* i, int32_t* j, int32_t* type, int32_t* isub, int32_t* jsub, double* dn,
                        double* fn, double* ft, double* mom, double* damp, int32_t* bond, uint8_t* active, double* n,
                        double* pos, double* vel) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  const int64_t ne = s.ne;
  if (ne == 0) return RK_OK;
  const size_t d1 = (size_t)ne * sizeof(double), d3 = 3 * d1, i1 = (size_t)ne * sizeof(int);
  if (i) CK(cudaMemcpyAsync(i, s.ei, i1, cudaMemcpyDeviceToHost, c.stream));
  if (j) CK(cudaMemcpyAsync(j, s.ej, i1, cudaMemcpyDeviceToHost, c.stream));
  if (type || isub || jsub) {
    int *dt = nullptr, *di = nullptr, *dj = nullptr;
    int rc;
    if ((rc = dalloc(c, dt, ne)) || (rc = dalloc(c, di, ne)) || (rc = dalloc(c, dj, ne))) return rc;
    k_unpack_tsub<<<nblk(ne, 256), 256, 0, c.stream>>>(s.etsub, ne, dt, di, dj);
    if (type) CK(cudaMemcpyAsync(type, dt, i1, cudaMemcpyDeviceToHost, c.stream));
    if (isub) CK(cudaMemcpyAsync(isub, di, i1, cudaMemcpyDeviceToHost, c.stream));
    if (jsub) CK(cudaMemcpyAsync(jsub, dj, i1, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    dfree(dt); dfree(di); dfree(dj);
  }
  if (dn) CK(cudaMemcpyAsync(dn, s.dn, d1, cudaMemcpyDeviceToHost, c.stream));
  if (fn) CK(cudaMemcpyAsync(fn, s.fn, d1, cudaMemcpyDeviceToHost, c.stream));
  if (ft) CK(cudaMemcpyAsync(ft, s.ft, d3, cudaMemcpyDeviceToHost, c.stream));
  if (mom) CK(cudaMemcpyAsync(mom, s.mom, d3, cudaMemcpyDeviceToHost, c.stream));
  if (damp) CK(cudaMemcpyAsync(damp, s.damp, d1, cudaMemcpyDeviceToHost, c.stream));
  if (bond) CK(cudaMemcpyAsync(bond, s.bond, i1, cudaMemcpyDeviceToHost, c.stream));
  std::vector<double> dn_h;
  std::vector<int32_t> bond_h;
  if (active) {  // active = dn < 0 or bonded (Rockable.cpp:3005-3029), from the stored history
    dn_h.resize(ne);
    bond_h.resize(ne);
    CK(cudaMemcpyAsync(dn_h.data(), s.dn, d1, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(bond_h.data(), s.bond, i1, cudaMemcpyDeviceToHost, c.stream));
  }
  if (n) CK(cudaMemcpyAsync(n, s.gn, d3, cudaMemcpyDeviceToHost, c.stream));
  if (pos) CK(cudaMemcpyAsync(pos, s.gpos, d3, cudaMemcpyDeviceToHost, c.stream));
  if (vel) CK(cudaMemcpyAsync(vel, s.gvel, d3, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (active)
    for (int64_t e = 0; e < ne; e++) active[e] = (dn_h[e] < 0.0 || bond_h[e] >= 0) ? 1 : 0;
  return RK_OK;
}

int rk_download_interfaces(rk_ctx* x, int32_t* i, int32_t* j, uint8_t* broken) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  if (s.nif == 0) return RK_OK;
  if (i) CK(cudaMemcpyAsync(i, s.if_i, s.nif * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  if (j) CK(cudaMemcpyAsync(j, s.if_j, s.nif * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  if (broken) CK(cudaMemcpyAsync(broken, s.if_broken, s.nif, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_get_stats(rk_ctx* x, rk_stats* out) {
  if (!x || !out) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  std::memset(out, 0, sizeof *out);
  if (s.n > 0) {
    int64_t nb = (s.n + 255) / 256;
    if (nb > c.ke_blocks) {
      dfree(c.d_ke);
      CK(cudaMalloc(&c.d_ke, 2 * nb * sizeof(double)));
      c.ke_blocks = nb;
    }
    launch_kinetic_energy(s, c.d_ke, c.stream);
    std::vector<double> h(2 * nb);
    CK(cudaMemcpyAsync(h.data(), c.d_ke, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    for (int64_t k = 0; k < nb; k++) {
      out->e_trans += h[2 * k];
      out->e_rot += h[2 * k + 1];
    }
    out->e_trans *= 0.5;
    out->e_rot *= 0.5;
  }
  int rc;
  if ((rc = read_flags(c))) return rc;
  out->n_entries = s.ne;
  out->n_active = (int64_t)c.h_flags[FLAG_NACTIVE];
  out->n_broken = (int64_t)c.h_flags[FLAG_NBROKEN];
  out->nl_updates = c.nl_updates;
  int64_t nfree = s.n - s.n_driven;
  out->coordination = nfree > 0 ? 2.0 * (double)out->n_active / (double)nfree : 0.0;
  return RK_OK;
}

int rk_upload_kinematics(rk_ctx* x, const double* pos, const double* vel, const double* acc, const double* Q,
                         const double* vrot, const double* arot) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  Scene& s = c.s;
  const size_t n3 = 3 * (size_t)s.n * sizeof(double);
  if (pos) CK(cudaMemcpyAsync(s.pos, pos, n3, cudaMemcpyHostToDevice, c.stream));
  if (vel) CK(cudaMemcpyAsync(s.vel, vel, n3, cudaMemcpyHostToDevice, c.stream));
  if (acc) CK(cudaMemcpyAsync(s.acc, acc, n3, cudaMemcpyHostToDevice, c.stream));
  if (Q) CK(cudaMemcpyAsync(s.Q, Q, 4 * (size_t)s.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  if (vrot) CK(cudaMemcpyAsync(s.vrot, vrot, n3, cudaMemcpyHostToDevice, c.stream));
  if (arot) CK(cudaMemcpyAsync(s.arot, arot, n3, cudaMemcpyHostToDevice, c.stream));
  return RK_OK;
}

int rk_upload_kinematics_packed(rk_ctx* x, const double* buf) {
  if (!x || !buf) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies first");
  int rc;
  if ((rc = ensure_kin_stage(c))) return rc;
  CK(cudaMemcpyAsync(c.kin_stage, buf, 19 * (size_t)c.s.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  c.kernels += launch_kin_pack(c.s, c.kin_stage, 0, c.stream);
  return RK_OK;
}

int rk_download_kinematics_packed(rk_ctx* x, double* buf) {
  if (!x || !buf) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (!c.have_bodies) return fail(c, RK_ERR_STATE, "upload the bodies first");
  int rc;
  if ((rc = ensure_kin_stage(c))) return rc;
  c.kernels += launch_kin_pack(c.s, c.kin_stage, 1, c.stream);
  CK(cudaMemcpyAsync(buf, c.kin_stage, 19 * (size_t)c.s.n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return RK_OK;
}

int rk_sort_keys(uint64_t* keys, int64_t n, int lo_bit, int hi_bit, void* stream) {
  if (n < 0 || (n > 0 && !keys) || lo_bit < 0 || hi_bit > 64 || lo_bit >= hi_bit) return RK_ERR_ARG;
  if (n <= 1) return RK_OK;
  cudaStream_t st = (cudaStream_t)stream;
  uint64_t* tmp = nullptr;
  void* temp = nullptr;
  if (cudaMalloc(&tmp, (size_t)n * sizeof(uint64_t)) != cudaSuccess) return RK_ERR_CUDA;
  if (cudaMalloc(&temp, sort_temp_bytes(n)) != cudaSuccess) {
    cudaFree(tmp);
    return RK_ERR_CUDA;
  }
  radix_sort_u64(keys, tmp, n, lo_bit, hi_bit, temp, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(tmp);
  cudaFree(temp);
  return e == cudaSuccess ? RK_OK : RK_ERR_CUDA;
}

int rk_set_profiling(rk_ctx* x, int on) {
  if (!x) return RK_ERR_ARG;
  Ctx& c = x->c;
  cudaSetDevice(c.device);
  if (on && !c.pev[0])
    for (int k = 0; k < 2 * RK_NPHASE; k++) CK(cudaEventCreate(&c.pev[k]));
  c.profiling = on ? 1 : 0;
  for (int k = 0; k < RK_NPHASE; k++) {
    c.prof_ms[k] = 0.0;
    c.prof_n[k] = 0;
  }
  return RK_OK;
}

int rk_get_profile(const rk_ctx* x, double* ms, int64_t* launches) {
  if (!x) return RK_ERR_ARG;
  for (int k = 0; k < RK_NPHASE; k++) {
    if (ms) ms[k] = x->c.prof_ms[k];
    if (launches) launches[k] = x->c.prof_n[k];
  }
  return RK_OK;
}

int rk_last_step_timing(const rk_ctx* x, double* ms, int64_t* kernels) {
  if (!x) return RK_ERR_ARG;
  if (ms) *ms = x->c.last_ms;
  if (kernels) *kernels = x->c.last_kernels;
  return RK_OK;
}

}  // extern "C"
