// rk_engine.cuh -- device data layout of one scene and the kernel launchers
// shared by the translation units of librk_gpu.so.
//
// HBM layout (one context = one scene):
//   bodies    : SoA, 3 doubles per vector field (pos, vel, acc, vrot, arot,
//               force, moment), 4 per quaternion; coalesced for one thread
//               per body.
//   gvert     : global positions of every body's vertices, recomputed once
//               per step (3 doubles per vertex); body b's vertices start at
//               gv_ofs[b].  The narrow phase gathers these instead of
//               re-rotating shape vertices per sub-contact.
//   entries   : the neighbour list as SoA sorted by the 64-bit key
//               (i:21 | j:21 | type:2 | isub:10 | jsub:10), with history
//               (dn, fn, ft, mom, damp, bond) and per-step contributions
//               (force f, moment on i, moment on j) of active entries.
//   iofs/jofs : body -> first entry with key.i == b; body -> first slot of
//               jlist, the entry indices with key.j == b in entry order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "rk_math.cuh"

namespace rk {

// Lanes that sum one body's resultant in the mixed form's resultant kernel.
constexpr int kGatherLanes = 8;


constexpr int kMaxSub = 1024;       // sub-element index limit of the sort key
constexpr int kMaxBody = 1 << 21;   // body index limit of the sort key
constexpr int kMaskWords = 2;       // vertex cull mask words per half-pair (<= 64 vertices)
constexpr int kHeavy = 64;          // entries above which a body's resultant is summed by a block
constexpr int kHeavyWarp = 1024;    // mixed form: up to this many, by its warp inside the resultant kernel

__host__ __device__ __forceinline__ uint64_t entry_key(uint32_t i, uint32_t j, uint32_t t, uint32_t isub,
                                                       uint32_t jsub) {
  return ((uint64_t)i << 43) | ((uint64_t)j << 22) | ((uint64_t)t << 20) | ((uint64_t)isub << 10) | (uint64_t)jsub;
}
__host__ __device__ __forceinline__ uint32_t pack_tsub(uint32_t t, uint32_t isub, uint32_t jsub) {
  return (t << 30) | (isub << 15) | jsub;
}
__host__ __device__ __forceinline__ int tsub_type(uint32_t p) { return (int)(p >> 30); }
__host__ __device__ __forceinline__ int tsub_isub(uint32_t p) { return (int)((p >> 15) & 0x7fff); }
__host__ __device__ __forceinline__ int tsub_jsub(uint32_t p) { return (int)(p & 0x7fff); }

struct LawParams {  // one group pair
  double p[24];
};

struct Control {
  int type;
  int body;
  double value;
  double vec[3];
};

struct Scene {
  // ---- shapes
  int nshapes;
  int* vert_ofs;
  int* edge_ofs;
  int* edges;
  int* face_ofs;
  int* face_vofs;
  int* face_verts;
  double* svert;   // 3 per shape vertex
  double* sradius;
  double* sobb;    // 15 per shape
  double* sbox;    // 6 per shape: centre and half extents of the box of its vertices, in the shape frame
  // ---- bodies
  int64_t n;
  int64_t n_driven;
  double *pos, *vel, *acc, *Q, *vrot, *arot, *force, *moment;
  double *hom, *mass, *inertia, *rad;
  float* inv_mi;  // 4 per body: 1/m and the inverse principal moments, rounded to float (mixed form)
  int *shape, *group, *cluster;
  int64_t nvert;     // total global vertices
  int64_t* gv_ofs;   // n+1
  int* gv_body;      // nvert
  int* lv;           // nvert: vertices of the bodies that have neighbour-list entries (nlv of them)
  int64_t nlv;
  double* gv;        // 3*nvert
  float* gvr;        // 3*nvert: the same vertices relative to their body's centre, in FP32 (the
                     // mixed form's test of clearly separated entries)
  float4* posf;      // n: body centre rounded to FP32 and its Minkowski radius, written with the
                     // world vertices (the same test)
  double* uv64;      // 3*nvert: each body vertex scaled by the body's homothety, h v, in the shape
                     // frame (written at upload: what every placement of a vertex starts from)
  float4* uvf;       // nvert: the same rounded to FP32
  float* gsum;       // 6 per body: the mixed form's FP32 contact sums (force, moment) of the step
  double* rotm;      // 9 per body: the mixed form's FP64 rotation matrix of Q (row-major), written
                     // each step with gvr; its FP64 path places the few vertices it needs from it
  double* bobb;      // 15 per body (placed OBB, not enlarged)
  float* bobbf;      // float copy of bobb
  float* baabb;      // 6 per body: outward-rounded AABB of the OBB enlarged by DVerlet/2
  float* bbox;       // 15 per body: the shape's vertex box placed (centre, 3 axes, half extents), float:
                     // the root of the two-level pruning of the candidate sub-elements
  // dynamic guard
  double *dpos, *dq;  // 3n, 4n
  // ---- law
  int law;
  int params_in_interfaces;
  int ngroup;
  LawParams* table;  // ngroup*ngroup
  double dt, dt_2, dt2_2;
  double gravity[3];
  double DVerlet, dVerlet;
  double num_damp;
  // body force on the free bodies (rk_set_body_force): its parameters and,
  // for the viscous fluid, pow(h^3 V, 2/3) per body; the RK_BF_* kind below
  double bf[8];
  double* bf_surf;
  double disp_update, angle_update;
  int dynamic_nl;
  int bf_kind;
  // ---- controls
  int ncontrols;
  Control* controls;
  int servo_kind, servo_icontr, servo_walls[6];
  double servo_p;
  // ---- entries
  int64_t ne, cap;
  int *ei, *ej;
  uint32_t* etsub;
  uint64_t* ekey;
  double *dn, *fn, *ft, *mom, *damp;
  int* bond;
  uint8_t* act;
  double *cf, *cmi, *cmj;      // contributions (3 per entry each)
  double *gn, *gpos, *gvel;    // stored geometry (3 per entry each)
  int record_geom;
  int64_t* iofs;  // n+1
  int64_t* jofs;  // n+1
  int64_t* jsplit;  // n: first j-side slot of body b whose entry follows b's own block
  int* jlist;     // ne
  int* nperm;     // ne: entries grouped by sub-contact type (the narrow phase's thread order)
  int* slow;      // ne: the mixed narrow phase's entries for the full path, in the regions of
                  // nperm's type runs (type t from flags[FLAG_TOFS + t])
  // ne: global vertex indices of each entry's sub-elements (k_entry_gv, after every list change):
  // vertex-vertex (a, b), vertex-edge (a, p1, p2), vertex-triangle (a, A, B, C; w = -1 for
  // faces of more than 3 vertices), edge-edge (pi1, pi2, pj1, pj2)
  int4* egv;
  int egv_ok;     // egv holds the current list (global vertex indices fit in an int)
  int* heavy;     // bodies whose entry count exceeds kHeavy (summed by a block each)
  int nheavy;
  int* heavy_lazy;    // heavy driven bodies whose resultant feeds no state (summed on demand)
  int nheavy_lazy;
  uint8_t* is_heavy;  // n: 1 summed by k_gather_heavy in the step, 2 deferred, 3 summed by its warp (mixed form)
  uint8_t* needres;   // n: 1 when the body's resultant is used by the step (free or force-controlled)
  float* bnd;         // n: largest distance of a vertex from the body centre (world, rounded up)
  int* scene_of;      // n: scene index (bodies of different scenes never interact)
  int near_geometric;  // 1: distance-only NEAR tests in the rebuild (learned skin), 0: Rockable's predicates
  int fast_body;       // 1: per-body kernels built with fused multiply-adds (mixed form)
  int tpb[4];         // threads per block of the narrow phase, resultants, global vertices, drift (0: default)
  float* sk_path;     // n: path-length bound of each free body since its last refresh (learned skin), or null
  const float* sk_rsw;  // n: swing radius (largest vertex distance from the centre), with sk_path
  // learned-skin guard, evaluated at the end of the resultant kernel when sk_out is set
  const double* sk_ref_pos;
  const double* sk_ref_q;
  float* sk_maxd;
  uint8_t* sk_flag;
  unsigned int* sk_out;  // 8 words, zeroed by the resultant kernel's launcher (by k_skin_begin in a batch)
  float sk_flag_at;
  // batched skin steps (rk_skin.cu, skin_batch_step_end): when set, every step kernel
  // returns at once while sk_ctl[0] (halt) is set
  unsigned int* sk_ctl;
  float4* sph;        // per body: vertex, edge and face bounding spheres (world frame, float)
  int64_t* sph_ofs;   // n+1
  int* sph_body;      // body of every sphere
  // ---- interfaces
  int64_t nif;
  int *if_i, *if_j;
  double* if_dn0;
  double* if_par;   // 8 per interface
  int* if_inner;
  uint8_t* if_broken;
  uint8_t* if_break;  // set by the narrow phase when the yield criterion is met
  int64_t* if_ofs;    // n+1 (interfaces sorted by i)
  // ---- device flags and counters (pinned-readable block)
  unsigned long long* flags;  // [0] need_update, [1] n_active, [2] n_broken_step, [3] guard max pos2 bits,
                              // [4] guard max rot bits, [5] guard reset pending, [6] error code,
                              // [7] 1 + index of a body with non-finite state, [8..11] entries of
                              // each type in `slow` (zero between steps), [12] arrival ticket of
                              // the full-path kernel's blocks, [13..17] first nperm position of
                              // each type (and ne)
};

enum { FLAG_NEED_UPDATE = 0, FLAG_NACTIVE = 1, FLAG_NBROKEN = 2, FLAG_GPOS = 3, FLAG_GROT = 4, FLAG_GRESET = 5,
       FLAG_ERROR = 6, FLAG_NONFINITE = 7, FLAG_NSLOW = 8, FLAG_SLOW_TICKET = 12, FLAG_TOFS = 13, FLAG_COUNT = 18 };

// step kernels (rk_step.cu)
int launch_controls_pre(const Scene& s, cudaStream_t st);
int launch_drift(const Scene& s, cudaStream_t st);
// all = false: only bodies with neighbour-list entries (the step's use)
// all: every body's vertices (a list update), or with `mark` those of the marked bodies
int launch_glob_vertices(const Scene& s, cudaStream_t st, bool all = false, const uint8_t* mark = nullptr);
int launch_narrow_force(const Scene& s, cudaStream_t st);
int launch_narrow_force_mixed(const Scene& s, cudaStream_t st);
int launch_gather_accel(const Scene& s, int apply_kick, cudaStream_t st);
int launch_gather_heavy(const Scene& s, cudaStream_t st);
int launch_gather_heavy_lazy(const Scene& s, cudaStream_t st);
int launch_breakage(const Scene& s, cudaStream_t st);
int launch_guard(const Scene& s, cudaStream_t st);
int launch_kinetic_energy(const Scene& s, double* d_out2, cudaStream_t st);
int launch_kin_pack(const Scene& s, double* stage, int dir, cudaStream_t st);
int max_tpb(int which, int form_mixed);
// per-body kernels compiled with fused multiply-adds (rk_fast.cu, mixed form)
// a batched skin step after the guard asked for a refresh: the kernel does nothing
__device__ __forceinline__ bool step_halted(const Scene& s) { return s.sk_ctl != nullptr && s.sk_ctl[0] != 0u; }

int launch_fused_glob(const Scene& s, unsigned blocks, int threads, int only_listed, const uint8_t* mark,
                      cudaStream_t st);
// with_drift: the step's launch, which makes the free bodies' drift first (the mixed form
// has no separate drift launch: launch_drift returns 0 for it)
int launch_body_frames(const Scene& s, unsigned blocks, int threads, int with_drift, cudaStream_t st);
int launch_body_verts(const Scene& s, cudaStream_t st);
int launch_fused_gather(const Scene& s, unsigned blocks, int threads, int apply_kick, cudaStream_t st);
int launch_fused_heavy(const Scene& s, const int* list, int count, cudaStream_t st);
int launch_skin_begin(const Scene& s, cudaStream_t st);
cudaError_t fused_attributes(int which, cudaFuncAttributes* a);
cudaError_t narrow_mixed_attributes(cudaFuncAttributes* a);

// learned skin (rk_skin.cu)
int launch_skin_hist(const Scene& s, const double* rp, const double* rq, const float* rsw, float unit,
                     unsigned int* hist, cudaStream_t st);
int launch_skin_reset(const Scene& s, const uint8_t* only, double* rp, double* rq, float* maxd, float* path,
                      cudaStream_t st);
int mlp_num_params();
int mlp_max_batch();
void launch_mlp_infer(const void* w, const float* x, float* y, cudaStream_t st);
void launch_mlp_grad(const void* w, const float* X, const float* T, int nb, float* grad, float* loss,
                     cudaStream_t st);
void launch_mlp_adam(float* master, void* w, float* m, float* v, const float* grad, float lr, int step,
                     cudaStream_t st);
void launch_mlp_to_half(const float* master, void* w, cudaStream_t st);

// primitives (rk_prims.cu)
size_t scan_temp_bytes(int64_t n);
void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* temp, cudaStream_t st);
size_t sort_temp_bytes(int64_t n);
void radix_sort_u64(uint64_t* keys, uint64_t* tmp, int64_t n, int lo_bit, int hi_bit, void* temp, cudaStream_t st);

}  // namespace rk
