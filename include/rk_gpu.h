/*
 * rk_gpu.h -- C ABI of the GB300 DEM step engine (librk_gpu.so).
 *
 * One context owns all device memory of one scene on one GPU.  The entry
 * points replace the seams through which Rockable's step loop drives its
 * hot path (paths relative to the Rockable source tree):
 *
 *   rk_step          <- Rockable::integrationStep, the velocity-Verlet step
 *                       (src/Core/Rockable.hpp:231, Rockable.cpp:1979-2158)
 *                       plus the loop bookkeeping of Rockable::integrate that
 *                       schedules NL updates (Rockable.cpp:2584-2736)
 *   rk_update_nl     <- Rockable::UpdateNL (Rockable.hpp:274; bruteForce
 *                       Rockable.cpp:1614-1662, linkCells 1667-1809) with the
 *                       AddOrRemoveInteractions seam (Rockable.hpp:318,
 *                       Rockable.cpp:1309-1432)
 *   rk_accelerations <- Rockable::accelerations (Rockable.cpp:3562-3719), the
 *                       load-time "fake step" of Rockable::loadConf (1137)
 *   rk_upload_* / rk_download_*
 *                    <- the state Rockable::loadConf / saveConf read and
 *                       write (Rockable.cpp:440-610, 886-1002)
 *   rk_set_params    <- the force-law selection and DataTable parameters
 *                       (Rockable.cpp:763-781, ForceLaw.hpp:44-55)
 *   rk_set_controls  <- DrivingSystem controls and the tritri servo
 *                       (DrivingSystem.hpp:70-75, DrivingSystem.cpp:186-268)
 *   rk_get_stats     <- Rockable::getKineticEnergy (Rockable.cpp:3958-3970)
 *
 * Conventions: every call returns RK_OK (0) or a negative RK_ERR_* code and
 * never throws; rk_last_error() describes the last failure of the context.
 * Host buffers passed in are copied before the call returns.  One host thread
 * per context.  No call falls back to the CPU: without a usable CUDA device,
 * rk_create fails.
 */
#ifndef RK_GPU_H
#define RK_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RK_ABI_VERSION 1

enum {
  RK_OK = 0,
  RK_ERR_ARG = -1,         /* invalid argument (sizes, ordering, indices)      */
  RK_ERR_CUDA = -2,        /* CUDA runtime error                               */
  RK_ERR_CAPACITY = -3,    /* a fixed limit was exceeded (see rk_last_error)   */
  RK_ERR_UNSUPPORTED = -4, /* feature outside this engine (periodic, BCM, ...) */
  RK_ERR_TIMEOUT = -5,     /* a bounded device wait gave up                    */
  RK_ERR_STATE = -6,       /* call out of order (e.g. step before upload)      */
  RK_ERR_NUMERIC = -7      /* non-finite state detected                        */
};

enum { RK_LAW_DEFAULT = 0, RK_LAW_AVALANCHE = 1, RK_LAW_STICKEDLINKS = 2 };
enum { RK_FORM_FP64 = 0, RK_FORM_MIXED = 1 };
/* BodyForce plugins (src/BodyForces/BodyForce_*.cpp). */
enum { RK_BF_NONE = 0, RK_BF_ATTRACTING_POINT = 1, RK_BF_PREFERRED_DIRECTION = 2, RK_BF_VISCOUS_FLUID = 3 };

/* Parameter slots of the per-group-pair table (DataTable ids of
 * Rockable.cpp:96-123).  table[(p * ngroup + g1) * ngroup + g2]. */
enum {
  RK_P_KN = 0, RK_P_EN2, RK_P_KT, RK_P_MU, RK_P_KR, RK_P_MUR,
  RK_P_KN_IN, RK_P_KT_IN, RK_P_KR_IN, RK_P_EN2_IN, RK_P_FN0_IN, RK_P_FT0_IN, RK_P_MOM0_IN, RK_P_POW_IN,
  RK_P_KN_OUT, RK_P_KT_OUT, RK_P_KR_OUT, RK_P_EN2_OUT, RK_P_FN0_OUT, RK_P_FT0_OUT, RK_P_MOM0_OUT, RK_P_POW_OUT,
  RK_NPARAM
};

/* Control types (DrivingSystem.hpp:52-67). */
enum {
  RK_X_VEL = 0, RK_Y_VEL = 1, RK_Z_VEL = 2, RK_XROT_VEL = 3, RK_YROT_VEL = 4, RK_ZROT_VEL = 5,
  RK_X_FOR = 6, RK_Y_FOR = 7, RK_Z_FOR = 8, RK_XROT_MOM = 9, RK_YROT_MOM = 10, RK_ZROT_MOM = 11,
  RK_XYZROT_VEL = 100, RK_XYZROT_MOM = 101
};

typedef struct rk_ctx rk_ctx;

typedef struct rk_config {
  int device;              /* CUDA device ordinal                              */
  int form;                /* RK_FORM_FP64 (bit-parity form) or RK_FORM_MIXED   */
  int64_t entry_capacity;  /* initial neighbour-list capacity; 0 = automatic   */
} rk_config;

/* Shape library, flattened (Shape.hpp:58-111). */
typedef struct rk_shapes {
  int32_t nshapes;
  const int32_t* vert_ofs;   /* nshapes+1                                      */
  const double* vertices;    /* 3*vert_ofs[nshapes], shape frame               */
  const int32_t* edge_ofs;   /* nshapes+1                                      */
  const int32_t* edges;      /* 2*edge_ofs[nshapes], shape-local vertex ids    */
  const int32_t* face_ofs;   /* nshapes+1 (faces per shape)                    */
  const int32_t* face_vofs;  /* face_ofs[nshapes]+1, offsets into face_verts   */
  const int32_t* face_verts; /* shape-local vertex ids                         */
  const double* radius;      /* nshapes, Minkowski radius                      */
  const double* obb;         /* 15*nshapes: center, e1, e2, e3, extent         */
} rk_shapes;

/* Bodies (Particle.hpp:77-127); the first n_driven are driven walls. */
typedef struct rk_bodies {
  int64_t n;
  int64_t n_driven;
  const double* pos;       /* 3n */
  const double* vel;       /* 3n */
  const double* acc;       /* 3n */
  const double* Q;         /* 4n, (w, x, y, z) */
  const double* vrot;      /* 3n */
  const double* arot;      /* 3n */
  const double* homothety; /* n  */
  const double* mass;      /* n  */
  const double* inertia;   /* 3n */
  const int32_t* shape;    /* n  */
  const int32_t* group;    /* n  */
  const int32_t* cluster;  /* n  */
} rk_bodies;

typedef struct rk_params {
  double t;                /* current time                                    */
  double dt;
  double gravity[3];
  double DVerlet;          /* OBB enlargement for the body broad phase         */
  double dVerlet;          /* sub-element proximity distance                   */
  double interVerlet;      /* time between periodic NL updates                 */
  double interVerletC;     /* time elapsed since the last periodic NL update   */
  double numerical_damping;
  int32_t law;             /* RK_LAW_*                                         */
  int32_t params_in_interfaces;
  int32_t dynamic_update_nl;
  double disp_update_nl;   /* guard: max displacement                          */
  double angle_update_nl;  /* guard: max rotation angle (radians)              */
  int32_t ngroup;
  const double* table;     /* RK_NPARAM * ngroup * ngroup                      */
} rk_params;

/* Neighbour-list entries (Interaction.hpp:57-100), sorted by the key
 * (i, j, type, isub, jsub) and unique. */
typedef struct rk_entries {
  int64_t n;
  const int32_t* i;
  const int32_t* j;
  const int32_t* type;
  const int32_t* isub;
  const int32_t* jsub;
  const double* dn;     /* n  */
  const double* fn;     /* n  */
  const double* ft;     /* 3n */
  const double* mom;    /* 3n */
  const double* damp;   /* n  */
  const int32_t* bond;  /* n, interface index or -1 */
} rk_entries;

/* Breakable interfaces (BreakableInterface.hpp:48-77), sorted by (i, j). */
typedef struct rk_interfaces {
  int64_t n;
  const int32_t* i;
  const int32_t* j;
  const double* dn0;     /* n  */
  const double* params;  /* 8n: kn kt kr fn0 ft0 mom0 power Gc */
  const int32_t* is_inner;
} rk_interfaces;

typedef struct rk_control {
  int32_t type;   /* RK_X_VEL ... */
  int32_t body;
  double value;
  double vec[3];
} rk_control;

typedef struct rk_servo {
  int32_t kind;      /* 0 none, 1 tritriIsostaticCompression */
  int32_t icontr;    /* index of the servo's first control   */
  int32_t walls[6];  /* Xmin Xmax Ymin Ymax Zmin Zmax         */
  double pressure;
} rk_servo;

typedef struct rk_step_report {
  int64_t steps_done;
  int64_t nl_updates;
  int64_t n_entries;
  int64_t n_active;
  int64_t n_broken;
  double t;
} rk_step_report;

typedef struct rk_stats {
  double e_trans, e_rot;  /* kinetic energies of all bodies */
  int64_t n_entries, n_active, n_broken, nl_updates;
  double coordination;    /* 2 * active / free bodies       */
} rk_stats;

int rk_abi_version(void);
int rk_create(rk_ctx** out, const rk_config* cfg);
void rk_destroy(rk_ctx* ctx);
const char* rk_last_error(const rk_ctx* ctx);

int rk_upload_shapes(rk_ctx* ctx, const rk_shapes* s);
int rk_upload_bodies(rk_ctx* ctx, const rk_bodies* b);
int rk_set_params(rk_ctx* ctx, const rk_params* p);
int rk_upload_entries(rk_ctx* ctx, const rk_entries* e);
int rk_upload_interfaces(rk_ctx* ctx, const rk_interfaces* f);
int rk_set_controls(rk_ctx* ctx, const rk_control* c, int32_t n, const rk_servo* servo);
/* The body force of every free body, added at the start of each force
 * computation (replaces Rockable::bodyForce, Rockable.hpp:125, applied in
 * Rockable.cpp:2887-2901; the plugin is selected by the conf keyword
 * BodyForce, Rockable.cpp:1026-1040).  params are the plugin's conf values in
 * the order its read() takes them:
 *   RK_BF_NONE                 nparams 0 (no body force)
 *   RK_BF_ATTRACTING_POINT     point x y z, acceleration (nparams 4;
 *                              BodyForce_AttractingPoint.cpp:43-59)
 *   RK_BF_PREFERRED_DIRECTION  axisBody x y z, axis x y z, momentMax
 *                              (nparams 7; both axes are normalised here as
 *                              read() does; BodyForce_PreferredDirection.cpp:
 *                              43-80)
 *   RK_BF_VISCOUS_FLUID        fluidDensity (nparams 1; BodyForce_ViscousFluid.
 *                              cpp:42-58); body_volume[b] = V h^3 (the shape's
 *                              volume times the homothety cubed, multiplied in
 *                              that order) for every body, required
 * body_volume is ignored by the other kinds.  Unknown kinds, a wrong nparams
 * or a missing body_volume return RK_ERR_ARG.  Uploading bodies of another
 * count afterwards drops a viscous-fluid body force (its volumes no longer
 * match). */
int rk_set_body_force(rk_ctx* ctx, int kind, const double* params, int32_t nparams, const double* body_volume);
/* Select the arithmetic of the narrow phase and force laws for the next
 * steps: RK_FORM_FP64 (bit-identical to the reference CPU path) or
 * RK_FORM_MIXED (FP32 on body-relative coordinates, FP64 for positions, the
 * overlap dn and the integration).  No reference counterpart. */
int rk_set_form(rk_ctx* ctx, int form);
/* Broad phase of the NL rebuild: 0 automatic (all pairs up to 4096 bodies,
 * grid above), 1 all pairs (Rockable's UpdateNL bruteForce), 2 uniform grid
 * (the role of UpdateNL linkCells).  Both visit exactly the same pairs. */
int rk_set_broadphase(rk_ctx* ctx, int mode);
/* Several independent scenes in one context: scene_of[b] for every body
 * (NULL = one scene).  Bodies of different scenes never interact; every
 * kernel launch covers all scenes.  No reference counterpart. */
int rk_set_scenes(rk_ctx* ctx, const int32_t* scene_of);
/* When on (off by default), rk_step replays each step's launches as one CUDA
 * graph captured on the context stream, re-captured after a neighbour-list
 * rebuild or a parameter change; per-phase profiling turns it off.  Results
 * are identical to the launch-by-launch path.  No reference counterpart. */
int rk_set_graphs(rk_ctx* ctx, int on);
/* Number of step-graph captures and replays since the context was created. */
int rk_get_graph_stats(const rk_ctx* ctx, int64_t* captures, int64_t* replays);
/* Block-size autotuner: the next 5 * rounds steps run the narrow phase, the
 * resultants, the global vertices and the drift with block sizes 32, 64,
 * 128, 256 and 512 in turn, timed with events; each kernel then keeps its
 * fastest size.  These kernels give the same results at any block size, so the
 * tuning steps are ordinary steps.  No reference counterpart. */
int rk_set_autotune(rk_ctx* ctx, int rounds);
/* Current block sizes of those four kernels, in that order. */
int rk_get_block_sizes(const rk_ctx* ctx, int32_t* tpb);
/* When on, every step also stores each entry's contact normal, point and
 * relative velocity (needed to write a conf file); off by default. */
int rk_set_record_geometry(rk_ctx* ctx, int on);

int rk_accelerations(rk_ctx* ctx);
int rk_update_nl(rk_ctx* ctx);
int rk_step(rk_ctx* ctx, int64_t nsteps, rk_step_report* report);
int rk_synchronize(rk_ctx* ctx);

int64_t rk_num_bodies(const rk_ctx* ctx);
int64_t rk_num_entries(const rk_ctx* ctx);
int64_t rk_num_interfaces(const rk_ctx* ctx);
/* Any output pointer may be NULL. */
int rk_download_bodies(rk_ctx* ctx, double* pos, double* vel, double* acc, double* Q, double* vrot, double* arot,
                       double* force, double* moment);
/* The Particles and Interactions sections of a conf file, formatted on the
 * device as Rockable::saveConf writes them (Rockable.cpp:547-580): one line
 * per body, "name group cluster homothety pos vel acc Q vrot arot", then one
 * per entry with dn < 0 or a bond, in key order, "i j type isub jsub n dn pos
 * vel fn ft mom damp"; every real number as printf("%.*e", precision), the
 * contact normal rounded toward zero (Rockable.cpp:569-575), fields
 * separated by one space, lines ended by '\n'.  The section headers
 * ("Particles N", the "#name ..." comment line, "Interactions M") are the
 * caller's, with M = *n_active.  The contact geometry (n, pos, vel) is the one
 * recorded by the last step run with rk_set_record_geometry(1) (and by the
 * load-time rk_accelerations).  precision in [0, 17].  Writes the bodies'
 * text then the entries' into buf when cap is large enough (else returns
 * RK_ERR_CAPACITY), and their lengths in bytes; with buf NULL, only the
 * lengths.  rk_set_shape_names gives the shape names first (one per
 * uploaded shape, no spaces). */
int rk_set_shape_names(rk_ctx* ctx, const char* const* names, int32_t n);
int rk_format_conf(rk_ctx* ctx, int32_t precision, char* buf, int64_t cap, int64_t* particles_len,
                   int64_t* interactions_len, int64_t* n_active);
/* Per-entry terms of the last force evaluation, 3 doubles each per entry in
 * key order: the force on body i (body j receives its opposite) and the
 * moments on i and on j -- the terms Rockable adds into the resultants
 * (Rockable.cpp:2752-2789).  Meaningful for the active entries only. */
int rk_download_contributions(rk_ctx* ctx, double* f, double* mi, double* mj);

/* ---- data extractors on the device (src/DataExtractors/*.cpp; the host keeps
 * the DataExtractor classes, file formats and cadence, and calls these
 * instead of downloading the state).  Extremes, counts and the picked entry
 * are exact; means are tree sums in a fixed order (same value on every run;
 * they may differ from the reference's serial sum in the last bits).
 * MeanVelocity::record (DataExtractor_MeanVelocity.cpp:24-32): mean |v| over all bodies. */
int rk_extract_mean_velocity(rk_ctx* ctx, double* mean);
/* dnStat::record (DataExtractor_dnStat.cpp:35-68) over the active entries (dn < 0 or bonded):
 * out[10] = dnMin, dnMax, dnMean, dnMeanNeg, dnMeanPos, nbNeg, nbPos, contact point of the first
 * entry with dnMin (the stored geometry: record it on the last step, rk_set_record_geometry). */
int rk_extract_dn_stat(rk_ctx* ctx, double* out);
/* ClusterAABB::record (DataExtractor_ClusterAABB.cpp:31-65): out[7] = 1 when the cluster has a body
 * (else all zero, the reference's default box), then min[3], max[3] of its bodies' vertices
 * enlarged by their Minkowski radii. */
int rk_extract_cluster_aabb(rk_ctx* ctx, int32_t cluster, double* out);
/* DuoBalance::record (DataExtractor_DuoBalance.cpp:31-85): out[4] = sub-contacts of the pair
 * (i, j), either way round, with dn < 0, by type (VV, VE, VF, EE). */
int rk_extract_duo_balance(rk_ctx* ctx, int32_t i, int32_t j, int64_t* out);
/* TrackBody::record (DataExtractor_TrackBody.cpp:67-80): out[25] = pos[3], vel[3], acc[3], Q[4],
 * vrot[3], arot[3], force[3], moment[3] of body b. */
int rk_download_body(rk_ctx* ctx, int64_t b, double* out);
int rk_download_entries(rk_ctx* ctx, int32_t* i, int32_t* j, int32_t* type, int32_t* isub, int32_t* jsub, double* dn,
                        double* fn, double* ft, double* mom, double* damp, int32_t* bond, uint8_t* active, double* n,
                        double* pos, double* vel);
int rk_download_interfaces(rk_ctx* ctx, int32_t* i, int32_t* j, uint8_t* broken);
/* Overwrite the kinematic state of all bodies from host buffers (any pointer
 * may be NULL); the host-owned Particles of Rockable are pushed back this way
 * after a host-side plugin modified them. */
int rk_upload_kinematics(rk_ctx* ctx, const double* pos, const double* vel, const double* acc, const double* Q,
                         const double* vrot, const double* arot);
/* The same kinematics in one packed host buffer of 19 n doubles, in this
 * order: pos (3n), vel (3n), acc (3n), Q (4n), vrot (3n), arot (3n).  One
 * copy and one scatter (upload, asynchronous: keep the buffer alive until the
 * next synchronising call) or one gather and one copy (download, returns when
 * the buffer is filled).  With a pinned buffer this is the cheapest way to
 * hand the bodies' state to and from the host every step.  No reference
 * counterpart (Rockable keeps the state in host memory). */
int rk_upload_kinematics_packed(rk_ctx* ctx, const double* buf);
int rk_download_kinematics_packed(rk_ctx* ctx, double* buf);
int rk_get_stats(rk_ctx* ctx, rk_stats* out);
/* Device time (ms) of the last rk_step call, measured with CUDA events on the
 * context's stream, and the number of kernels it launched. */
int rk_last_step_timing(const rk_ctx* ctx, double* ms, int64_t* kernels);
/* Stable LSD radix sort of n 64-bit keys in device memory on bits
 * [lo_bit, hi_bit), in place, on `stream` (a cudaStream_t, NULL = default).
 * The primitive the neighbour-list rebuild orders its keys with (the
 * lexicographic key order of Interaction.hpp:106-122, and the j-side list);
 * temporary memory is allocated and freed by the call. */
int rk_sort_keys(uint64_t* keys, int64_t n, int lo_bit, int hi_bit, void* stream);
/* rk_sort_keys without any allocation; it has no counterpart in the reference.
 * For callers that cannot allocate device memory (an allocator that already
 * holds the device's memory, a serving loop with a footprint fixed at start-up,
 * streams that cannot take cudaFree's device-wide synchronisation).  The
 * temporary buffers are one static device array of about 4.5 MB shared by all
 * calls: n is limited to 524288 keys (RK_ERR_CAPACITY beyond), calls that
 * overlap on the GPU race on that array and must be ordered by the caller, and
 * the first call on each device looks up the array's address (make it before
 * any stream capture begins).  Asynchronous on `stream`: unlike rk_sort_keys
 * it does not synchronise. */
int rk_sort_keys_noalloc(uint64_t* keys, int64_t n, int lo_bit, int hi_bit, void* stream);
/* Per-phase device time: when on, rk_step brackets each phase with CUDA
 * events on the context stream (adds one event pair per phase and step).
 * Phases: 0 controls, 1 drift, 2 global vertices, 3 narrow phase + law,
 * 4 resultants + accelerations, 5 breakage, 6 NL rebuild, 7 guard. */
#define RK_NPHASE 8

/* Learned Verlet skin (no reference counterpart; replaces the fixed
 * interVerlet / dVerlet schedule and the dynamic guard of Rockable.cpp:
 * 1571-1596 while enabled).  An exact bound on every body's point motion
 * since the last rebuild forces a rebuild when it reaches dVerlet / 2; between
 * forced rebuilds, a 16-64-64-2 MLP (FP16, trained online on the run's own
 * displacement and churn history) predicts the next window's displacement
 * rate, from which the skin (dVerlet, DVerlet = ratio * dVerlet) and the
 * rebuild interval are chosen by minimising the measured step + rebuild cost. */
typedef struct rk_skin_config {
  int32_t enabled;
  int32_t use_mlp;        /* 0: predict the next window from the last one only */
  double skin_min, skin_max;
  double dverlet_ratio;   /* DVerlet / dVerlet */
  int32_t interval_min, interval_max;
  double learning_rate;
  int32_t train_steps;    /* optimiser steps per rebuild */
  uint64_t seed;
  double partial_fraction;  /* a forced update refreshes only the bodies near their guard
                               limit when they are at most this fraction of all bodies
                               (0: every update is a full rebuild) */
  int32_t exact_contacts;   /* 1: distance-only NEAR tests, so every sub-contact that touches
                               is listed (more entries); 0: Rockable's NEAR tests, whose
                               projection conditions can list a sliding vertex-face or
                               edge-edge contact one refresh late, like the fixed schedule */
} rk_skin_config;
typedef struct rk_skin_stats {
  int64_t rebuilds, forced, scheduled;
  double skin;            /* current dVerlet */
  int64_t interval;       /* current scheduled interval (steps) */
  double last_rate;       /* observed max displacement per step, last window */
  double predicted_rate;  /* prediction for the current window */
  double loss;            /* last training loss */
  int64_t partial;        /* partial refreshes */
  int64_t partial_bodies; /* bodies refreshed by them, summed */
  int64_t train_steps;    /* optimiser steps of the network so far */
  int64_t windows;        /* training windows in its replay buffer */
  double rebuild_ms;      /* device time of a full rebuild (exponential average of the measured ones) */
  double partial_ms;      /* device time of a partial refresh (the same) */
} rk_skin_stats;
int rk_set_skin(rk_ctx* ctx, const rk_skin_config* cfg);
int rk_get_skin_stats(rk_ctx* ctx, rk_skin_stats* out);
/* Direct access to the network (tests: gradient checks against a CPU model).
 * Parameters: W1[64][16] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]. */
int rk_mlp_num_params(void);
int rk_mlp_set_params(rk_ctx* ctx, const float* params);
int rk_mlp_get_params(rk_ctx* ctx, float* params);
int rk_mlp_forward(rk_ctx* ctx, const float* x, float* y);
int rk_mlp_gradient(rk_ctx* ctx, const float* X, const float* T, int32_t nbatch, float* grad, float* loss);
int rk_set_profiling(rk_ctx* ctx, int on);
int rk_get_profile(const rk_ctx* ctx, double* ms, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif
