// rk_ctx.cuh -- host-side context of librk_gpu.so (one scene on one GPU).
#pragma once
#include <cstdint>
#include <array>
#include <string>
#include <vector>

#include "../../include/rk_gpu.h"
#include "rk_engine.cuh"

namespace rk {

// Per-entry arrays that survive a neighbour-list rebuild (double-buffered).
struct EntryBuf {
  int64_t cap = 0;
  int *ei = nullptr, *ej = nullptr;
  uint32_t* etsub = nullptr;
  uint64_t* ekey = nullptr;
  double *dn = nullptr, *fn = nullptr, *ft = nullptr, *mom = nullptr, *damp = nullptr;
  int* bond = nullptr;
  double *gn = nullptr, *gpos = nullptr, *gvel = nullptr;
};

// Scratch of the neighbour-list rebuild, grown on demand.
struct NLWork {
  cudaEvent_t split = nullptr;   // recorded after the pairs (when timing_split)
  bool timing_split = false;
  int64_t pair_cap = 0, hp_cap = 0, cand_cap = 0, old_cap = 0, fin_cap = 0, tmp_bytes = 0;
  uint64_t* pairs = nullptr;     // pair_cap
  uint64_t* hp = nullptr;        // hp_cap (half-pair keys owner<<21 | partner)
  uint64_t* hp_tmp = nullptr;    // hp_cap
  uint32_t* hp_mask = nullptr;   // kMaskWords * hp_cap
  uint64_t* cand = nullptr;      // cand_cap new entry keys
  uint64_t* cand_tmp = nullptr;  // cand_cap (sort)
  int64_t cand_hint = 0;         // candidates found by the previous rebuild
  int64_t* flag = nullptr;       // old_cap + 1
  uint64_t* stale = nullptr;     // old_cap
  int64_t* stale_src = nullptr;  // old_cap
  uint64_t* fkey = nullptr;      // fin_cap
  int64_t* fsrc = nullptr;       // fin_cap
  uint64_t* jkeys = nullptr;     // fin_cap
  uint64_t* jtmp = nullptr;      // fin_cap
  void* tmp = nullptr;           // scan / sort temp
  unsigned long long* counter = nullptr;
  // grid broad phase
  int64_t grid_cap = 0;
  uint64_t* gkeys = nullptr;
  uint64_t* gtmp = nullptr;
  int* gover = nullptr;
  uint8_t* gis_over = nullptr;
  uint8_t* gmark = nullptr;  // bodies of the pairs of a partial refresh
  int64_t mark_cap = 0;
  void* gstat = nullptr;
};

// Learned-skin state (rk_skin.cu kernels, policy in rk_api.cu).
struct Skin {
  rk_skin_config cfg{};
  bool on = false;
  double* ref_pos = nullptr;
  double* ref_q = nullptr;
  float* rsw = nullptr;
  int64_t nalloc = 0;               // bodies the per-body arrays hold
  float* maxd = nullptr;            // n: largest delta since the body's last refresh
  float* path = nullptr;            // n: path-length bound since the body's last refresh
  uint8_t* flag = nullptr;          // n: bodies due for a partial refresh
  unsigned int* d_guard = nullptr;  // guard reductions (see k_skin_guard)
  unsigned int* h_guard = nullptr;  // pinned
  // batched steps: control block (see rk_skin.cu) on the device, and its
  // pinned host copies (words 0-15 written before a batch, 16-31 read after)
  unsigned int* d_ctl = nullptr;
  unsigned int* h_ctl = nullptr;
  cudaEvent_t bev = nullptr;
  int64_t partial = 0, partial_bodies = 0, partial_since_global = 0, since_global = 0;
  // measured in the current window: narrow-phase time per step (events
  // around its launch, in the step graph too) and partial-refresh cost
  double narrow_acc = 0.0, partial_ms = 0.0;
  int64_t narrow_cnt = 0, partial_in_window = 0;
  cudaEvent_t nev[2] = {nullptr, nullptr}, pa = nullptr, pb = nullptr;
  bool narrow_timed = false;
  // double-buffered guard read-back (8 words per slot) and its events
  cudaEvent_t gev[2] = {nullptr, nullptr};
  int gslot = 0;
  bool have_pred = false;  // the last guard read holds a prediction for the next state
  // MLP
  float* master = nullptr;
  void* w = nullptr;
  float *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr, *X = nullptr, *T = nullptr, *io = nullptr;
  int adam_step = 0;
  std::vector<std::array<float, 16>> rx;
  std::vector<std::array<float, 2>> ry;
  size_t rhead = 0;
  std::array<float, 16> feat_prev{};
  double churn_base_prev = 0.0;  // churn the previous prediction was relative to
  bool have_prev = false;
  // window bookkeeping
  int64_t since = 0, interval = 100;
  double skin = 0.0;
  double rates[4] = {0, 0, 0, 0};
  double last_rate = 0.0, pred_rate = 0.0, pred_churn = 0.0, last_loss = 0.0;
  int64_t rebuilds = 0, forced = 0, scheduled = 0;
  double step_ms = 0.0, rebuild_ms = 0.0;  // measured costs (exponential averages)
  unsigned int* d_hist = nullptr;   // 64 bins (k_skin_hist)
  double rebuild_bp_ms = 0.0, rebuild_var_ms = 0.0;  // last full rebuild: broad phase, the rest
  double alpha = 1.6;  // entries ~ skin^alpha (non-active part), learnt
  cudaEvent_t ea = nullptr, eb = nullptr;
  double window_ms = 0.0;
};

struct Ctx {
  int device = 0;
  int form = RK_FORM_FP64;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  Scene s{};
  EntryBuf eb[2];
  int cur = 0;
  NLWork w;
  // host copies of small things
  std::vector<Control> controls;
  std::vector<int> shape_nv;  // vertices per shape
  std::vector<double> shape_radius;
  std::vector<int> shape_ne, shape_nf;
  std::vector<double> shape_vmax;      // largest vertex distance from the shape centre
  std::vector<int> body_shape;
  std::vector<double> body_hom;
  bool have_shapes = false, have_bodies = false, have_params = false;
  // loop bookkeeping (Rockable::integrate)
  double t = 0.0, interVerlet = 0.01, interVerletC = 0.0;
  int64_t nl_updates = 0, steps = 0;
  double last_ms = 0.0;
  int64_t last_kernels = 0;
  int64_t kernels = 0;
  unsigned long long* h_flags = nullptr;  // pinned mirror of the device flag block
  double* d_ke = nullptr;
  double* ext_part = nullptr;             // the extractors' per-block partial results
  unsigned long long* ext_u = nullptr;    // their atomic extremes and counts
  int64_t ke_blocks = 0;
  // contributions and per-step arrays (single-buffered)
  int64_t contrib_cap = 0;
  // per-phase profiling
  int profiling = 0;
  cudaEvent_t pev[2 * RK_NPHASE] = {};
  double prof_ms[RK_NPHASE] = {};
  int64_t prof_n[RK_NPHASE] = {};
  Skin skin;
  int broadphase = 0;  // 0 automatic, 1 all pairs, 2 grid
  float last_cell = 0.f;
  int64_t last_nover = 0;
  // grid of the last full build (cell size, range of the box centres): a
  // partial refresh reuses it -- any cell size finds every pair (bodies
  // larger than a cell are tested against all), and coordinates outside the
  // range are clamped, which only adds candidates -- and saves two reductions
  // and their host round trips
  float grid_lo[3] = {0.f, 0.f, 0.f}, grid_hi[3] = {0.f, 0.f, 0.f};
  int64_t grid_n = -1;  // bodies of that build (-1: none yet)
  bool forces_stale = false;
  bool more_steps_follow = false;  // inside rk_step, before its last step
  int64_t nsph = 0;                // sub-element spheres of all bodies
  double* kin_stage = nullptr;     // packed kinematics transfers (19 doubles per body)
  int64_t kin_stage_n = 0;
  std::vector<uint8_t> needres_host;
  int64_t bf_n = 0;  // body count the body force was set for
  // shape names for the device-formatted conf text (rk_set_shape_names)
  char* name_chars = nullptr;
  int* name_ofs = nullptr;
  bool have_names = false;
  // block-size autotuner of the step kernels (results do not depend on it)
  int64_t tune_left = 0, tune_total = 0;
  double tune_ms[4][5] = {};  // [kernel][candidate block size]
  cudaEvent_t tev[8] = {};
  // CUDA graph of one step's launches (re-captured when the scene changes)
  int use_graphs = 0;
  cudaGraphExec_t gexec = nullptr;
  Scene gscene{};       // the scene the graph was captured with
  int gform = -1;
  int glaunched = 0;    // kernels per replay
  int64_t graph_captures = 0, graph_replays = 0;
  // the graphs of batches of 1, 2, 4, 8, 16 skin steps (same rules as the step graph)
  cudaGraphExec_t bexec[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  Scene bscene[5]{};
  int bform[5] = {-1, -1, -1, -1, -1};
  int blaunched[5] = {0, 0, 0, 0, 0};
};

// Neighbour-list update; with `only` (device flags per body), only the pairs
// with at least one flagged body are visited (partial refresh).
int rebuild_nl(Ctx& c, const uint8_t* only = nullptr);
int heavy_list(Ctx& c);
int ensure_entry_capacity(Ctx& c, int which, int64_t n);
void bind_entries(Ctx& c);

}  // namespace rk
