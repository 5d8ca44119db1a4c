/*
 * rk_oracle.h -- C interface of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of Rockable's per-step DEM hot path
 * (velocity-Verlet, narrow phase, force laws, bruteForce / linkCells
 * neighbour list, bond breakage, conf I/O).  It exists to check the CUDA
 * path: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  Nothing in the product links or calls it.
 */
#ifndef RK_ORACLE_H
#define RK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* Arithmetic variants for the parts of the reference that live in the
 * unvendored toofus library (quaternion / vector kernels).  The default,
 * {qrot 1, qdot 0, qddot 0, qnorm 3, vnorm 1, vdiv 1}, is the pinned choice:
 * it reproduces the reference's 512_particles and 518_poly regression goldens
 * bit for bit.  The other values exist only for the pinning experiment. */
typedef struct {
  int qrot;   /* quaternion-vector rotation form              */
  int qdot;   /* first time-derivative of a quaternion        */
  int qddot;  /* second time-derivative of a quaternion       */
  int qnorm;  /* quaternion normalisation                     */
  int vnorm;  /* vec3 normalisation                           */
  int vdiv;   /* vec3 / scalar                                */
} orc_variant;

void orc_set_variant(const orc_variant* v);

/* Load a conf file (a "redirection" header is followed like the reference
 * does).  Runs the load-time "fake step" (accelerations) exactly like
 * Rockable::loadConf.  Returns NULL on error (message via orc_last_error). */
orc_sim* orc_load(const char* conf_path);
const char* orc_last_error(void);
void orc_free(orc_sim* s);

/* Read a drivingSystem.txt-format file (controls and tritri servos). */
int orc_read_driving(orc_sim* s, const char* path);

/* Neighbour-list update (the conf's UpdateNL choice). */
void orc_update_nl(orc_sim* s);

/* One pass of the integrate loop body: t += dt, velocity-Verlet step, NL
 * update when due (interVerlet counter or needUpdate), dynamic guard.
 * Conf files are not written.  Returns the number of NL updates done. */
int orc_run(orc_sim* s, int nsteps);

/* The reference's console run: initial NL update, then the integrate loop
 * writing conf<N> files into outdir until t > tmax.  max_steps <= 0 means no
 * limit.  Returns the number of steps done, or < 0 on error. */
long orc_integrate(orc_sim* s, const char* outdir, long max_steps);

int orc_save_conf(orc_sim* s, const char* path);

/* State access ------------------------------------------------------------ */
int orc_nbodies(const orc_sim* s);
int orc_ndriven(const orc_sim* s);
/* 29 doubles per body: pos3 vel3 acc3 Q(w,x,y,z) vrot3 arot3 force3 moment3
 * + homothety, mass, group(as double), cluster(as double) */
void orc_get_bodies(const orc_sim* s, double* out);
/* Overwrite the kinematic state of all bodies (pos vel acc Q vrot arot:
 * 19 doubles per body). */
void orc_set_bodies(orc_sim* s, const double* in);

/* All neighbour-list entries (active or not), in key order. */
long orc_nentries(const orc_sim* s);
/* keys: 5 int64 per entry (i, j, type, isub, jsub)
 * state: 21 doubles per entry:
 *   n3 dn prev_dn pos3 vel3 fn ft3 mom3 damp bond(index or -1) active(0/1) */
void orc_get_entries(const orc_sim* s, int64_t* keys, double* state);
long orc_nactive(const orc_sim* s);

long orc_ninterfaces(const orc_sim* s);
/* 12 doubles per interface: i j nbonds dn0 kn kt kr fn0 ft0 mom0 power isInner */
void orc_get_interfaces(const orc_sim* s, double* out);

/* Scalars: t, dt, tmax, interVerlet, interConf, DVerlet, dVerlet, iconf,
 * nDriven, numericalDampingCoeff, totalBrokenArea, nbroken, gravity3 */
void orc_get_scalars(const orc_sim* s, double* out);
/* The BodyForce plugin: returns its kind (0 none, 1 AttractingPoint,
 * 2 PreferredDirection, 3 ViscousFluid), its conf values as read into
 * params[8], and when body_volume is not NULL, V h^3 of every body. */
int orc_get_body_force(const orc_sim* s, double* params, double* body_volume);
void orc_get_stats(const orc_sim* s, double* out); /* Etrans Erot nactive coordination nbroken */
int orc_law_id(const orc_sim* s); /* 0 Default, 1 Avalanche, 2 StickedLinks */
const char* orc_option(const orc_sim* s, const char* key);

/* Shapes, flattened like rk_shapes of include/rk_gpu.h.
 * sizes: nshapes, total vertices, total edges, total faces, total face vertices */
int orc_nshapes(const orc_sim* s);
void orc_get_shape_sizes(const orc_sim* s, int64_t* sizes);
void orc_get_shapes(const orc_sim* s, int32_t* vert_ofs, double* vertices, int32_t* edge_ofs, int32_t* edges,
                    int32_t* face_ofs, int32_t* face_vofs, int32_t* face_verts, double* radius, double* obb);
/* Per-body constants: shape, group, cluster, homothety, mass, inertia(3). */
void orc_get_body_static(const orc_sim* s, int32_t* shape, int32_t* group, int32_t* cluster, double* homothety,
                         double* mass, double* inertia);
/* Law parameter table in the slot order of include/rk_gpu.h (RK_P_*):
 * table[(p * ngroup + g1) * ngroup + g2].  Returns ngroup. */
int orc_ngroup(const orc_sim* s);
void orc_get_table(const orc_sim* s, double* table);
/* Controls: type, body, value, vec(3); servo: kind icontr w0..w5, pressure. */
int orc_ncontrols(const orc_sim* s);
void orc_get_controls(const orc_sim* s, int32_t* type, int32_t* body, double* value, double* vec, int32_t* servo,
                      double* pressure);
/* Flow scalars: interVerletC, dynamicUpdateNL, dispUpdateNL, angleUpdateNL,
 * paramsInInterfaces, needUpdate */
void orc_get_flow(const orc_sim* s, double* out);
/* Set one DataTable entry (both (g1,g2) and (g2,g1)), e.g. "fn0InnerBond". */
int orc_set_param(orc_sim* s, const char* name, int g1, int g2, double value);

#ifdef __cplusplus
}
#endif
#endif
