/*
 * xdem_c.h -- C-ABI of the GB300 DEM time step.
 *
 * Two surfaces:
 *
 *  1. Launcher surface.  The functions below carry the names, parameter order
 *     and data layouts of the xdynamics DEM launchers declared in
 *     include/xdynamics_parallel/xParallelDEM_decl.cuh:280-424 of the
 *     reference, so a caller of that header can relink against
 *     libxdem_gb300.so.  Pointers are DEVICE pointers laid out exactly as the
 *     reference lays them out: positions double4 (x,y,z,radius), velocities
 *     double3, Euler parameters double4 (e0..e3), pair lists
 *     MAX_P2P_COUNT / MAX_P2PL_COUNT / MAX_P2MS_COUNT slots per particle with
 *     double2 tangential history keyed by the partner id.  Each returns an int
 *     status (XDEM_OK = 0) instead of void; `reduction` keeps its double
 *     return and reports errors through xdem_last_status().
 *
 *  2. Scene surface (xdem_sim_*).  One handle owns the whole particle state on
 *     the GPU and runs the step in the order of
 *     xIntegratorVV::OneStepSimulation (source/xdynamics_simulation/
 *     xIntegratorVV.cpp:26-63) with fused, sorted-order kernels.  The rigid
 *     bodies of a host multibody solver exchange one 15-double pose record in
 *     and one 6-double wrench out per body per step.
 *
 * Structs are byte-compatible with the reference (double3 = 3 packed doubles,
 * 8-byte aligned; uint3 = 3 packed uints).
 */
#ifndef XDEM_C_H
#define XDEM_C_H

#include <stddef.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define XDEM_API __declspec(dllexport)
#else
#define XDEM_API __attribute__((visibility("default")))
#endif

/* Pair-list capacities per particle (decl:13-16). */
#define MAX_P2P_COUNT 12
#define MAX_P2PL_COUNT 3
#define MAX_P2CY_COUNT 3
#define MAX_P2MS_COUNT 5
/* Size in bytes of the 15-double rigid-body record (decl:18). */
#define DEVICE_BODY_MEM_SIZE 120
/* Candidate buffers of the particle-mesh search (impl:1975-1977). */
#define XDEM_MAX_TRI_CANDIDATES 20

/* Index of each entry of the 15-double body record (decl:20). */
enum { XDEM_MM = 0, XDEM_PX, XDEM_PY, XDEM_PZ, XDEM_VX, XDEM_VY, XDEM_VZ,
       XDEM_E0, XDEM_E1, XDEM_E2, XDEM_E3, XDEM_ED0, XDEM_ED1, XDEM_ED2, XDEM_ED3 };

/* Status bits.  A launcher returns the OR of the bits its kernels raised. */
enum {
    XDEM_OK = 0,
    XDEM_ERR_P2P_OVERFLOW  = 1 << 0,  /* > MAX_P2P_COUNT particle contacts   */
    XDEM_ERR_P2PL_OVERFLOW = 1 << 1,  /* > MAX_P2PL_COUNT plane contacts     */
    XDEM_ERR_P2MS_OVERFLOW = 1 << 2,  /* > MAX_P2MS_COUNT triangle contacts  */
    XDEM_ERR_TRI_CANDIDATES = 1 << 3, /* > 20 face/edge/vertex candidates    */
    XDEM_ERR_NONFINITE     = 1 << 4,  /* NaN/Inf position seen by the hash   */
    XDEM_ERR_P2CY_OVERFLOW = 1 << 5,  /* > MAX_P2CY_COUNT cylinder contacts
                                         (the reference writes on past the
                                         particle's slots; here they are
                                         dropped and this bit is raised)     */
    XDEM_ERR_BARRIER       = 1 << 6,  /* a grid barrier of the persistent
                                         batched step waited past its time
                                         limit; the step is incomplete       */
    XDEM_ERR_CUDA          = 1 << 8,  /* a CUDA runtime call failed          */
    XDEM_ERR_ARG           = 1 << 9,  /* invalid argument (null, size, mode) */
    XDEM_ERR_NOT_SET       = 1 << 10, /* setDEMSymbolicParameter not called  */
    XDEM_ERR_ALLOC         = 1 << 11  /* device allocation failed            */
};

typedef struct { double x, y, z; } xdem_double3;
typedef struct { unsigned int x, y, z; } xdem_uint3;

/* decl:128-150 */
typedef struct device_dem_parameters {
    bool rollingCondition;
    int contact_model;            /* 0 = DHS, 1 = Hertz-Mindlin (no slip) */
    unsigned int np;
    unsigned int nmp;
    unsigned int nCluster;
    unsigned int nClusterObject;
    unsigned int nTsdaConnection;
    unsigned int nTsdaConnectionList;
    unsigned int nTsdaConnectionBodyData;
    unsigned int nsphere;
    unsigned int nplane;
    unsigned int ncylinder;
    unsigned int ncell;
    xdem_uint3 grid_size;         /* each a power of two */
    double dt;
    double half2dt;               /* 0.5 dt^2 */
    double cell_size;
    double cohesion;
    xdem_double3 gravity;
    xdem_double3 world_origin;
} device_dem_parameters;

/* decl:152-159 */
typedef struct device_triangle_info {
    int id;
    unsigned int tid;
    xdem_double3 P, Q, R;
} device_triangle_info;

/* decl:161-174 */
typedef struct device_plane_info {
    unsigned int id;
    double l1, l2;
    xdem_double3 u1, u2, uw, xw, pa, pb, w2, w3, w4;
} device_plane_info;

/* decl:220-228: a cylinder in its body frame -- base and top centres,
 * len_rr = (length, base radius, top radius), wall thickness, and which part
 * is open (empty_part, xCylinderObject.h:14: 0 none, 1 top circle, 2 bottom
 * circle, 3 both, 4 radial wall; the contact kernels test 1 and 2) */
typedef struct device_cylinder_info {
    unsigned int id;
    unsigned int empty_part;
    double thickness;
    xdem_double3 len_rr;
    xdem_double3 pbase;
    xdem_double3 ptop;
} device_cylinder_info;

/* decl:230-243; filled in the order of xContact.cpp:308-312 */
typedef struct device_contact_property {
    double Ei, Ej;
    double pri, prj;
    double Gi, Gj;
    double rest;
    double fric;
    double s_fric;
    double rfric;
    double coh;
    double sratio;
    double amp;
} device_contact_property;

/* include/xTypes.h:263 */
typedef struct xClusterInformation {
    unsigned int sid, scid, count, neach;
} xClusterInformation;

/* ------------------------------------------------------------------------ */
/* Library control                                                          */
/* ------------------------------------------------------------------------ */

/* Stream used by every launcher below (default: the legacy default stream,
 * as the reference).  `stream` is a cudaStream_t. */
XDEM_API int xdem_set_stream(void* stream);
/* Status of the most recent call on this host thread. */
XDEM_API int xdem_last_status(void);
/* Clears and returns the accumulated device status word (overflow bits). */
XDEM_API int xdem_take_device_status(void);
/* Per-particle body-force partial arrays (np doubles each) written by the
 * plane and mesh launchers, the role of xContact::deviceBodyForceX..MomentZ
 * (source/xdynamics_object/xContact.cpp:315-345).  NULL entries make the
 * library use its own arrays. */
XDEM_API int xdem_set_body_force_buffers(double* fx, double* fy, double* fz,
                                         double* mx, double* my, double* mz);
/* Device pointers of the arrays currently used as the body-force partials. */
XDEM_API int xdem_get_body_force_buffers(double** out6);
/* Wrench (fx,fy,fz,mx,my,mz) on the body of the last plane/mesh launch,
 * summed on the GPU; replaces the six `reduction` calls of
 * xParticlePlaneContact.cpp:159-168 / xParticleMeshObjectContact.cpp:209-216.
 * Synchronises the launcher stream. */
XDEM_API int xdem_last_body_wrench(double out6[6]);
/* Reference semantics switch: 1 reproduces the reference GPU sphere velocity
 * kernel, which writes the linear velocity back unchanged (impl:208,218);
 * 0 (default) applies the velocity-Verlet trapezoid to it as the CPU path and
 * the cluster kernel do (xIntegratorVV.cpp:143-149, impl:279-284). */
XDEM_API int xdem_set_velocity_compat(int reproduce_reference_gpu);
/* Rolling resistance of free spheres (cu_decide_rolling_friction_moment):
 * 0 (default) reads J = inertia[id] of the double3 inertia array as the
 * reference kernel does (impl:2434), i.e. an entry of sphere id/3; 1 reads
 * the sphere's own J = inertia[3 id]. */
XDEM_API int xdem_set_rolling_inertia(int per_sphere);
/* Library build string. */
XDEM_API const char* xdem_version(void);

/* ------------------------------------------------------------------------ */
/* Launcher surface (decl:280-424)                                          */
/* ------------------------------------------------------------------------ */

/* decl:280, def:16-19 */
XDEM_API int setDEMSymbolicParameter(device_dem_parameters* h_paras);

/* decl:282, def:36-49 */
XDEM_API int vv_update_position(double* pos, double* ep, double* vel,
                                double* ev, double* acc, double* ea,
                                unsigned int np);
/* decl:284, def:51-69 */
XDEM_API int vv_update_velocity(double* vel, double* acc, double* ep,
                                double* ev, double* ea, double* force,
                                double* moment, double* mass, double* iner,
                                unsigned int np);
/* decl:287, def:71-80 */
XDEM_API int cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index,
                                      double* pos, unsigned int sid,
                                      unsigned int np);
/* decl:288-290, def:82-91 */
XDEM_API int cu_calculateHashAndIndexForPolygonSphere(
    unsigned int* hash, unsigned int* index, unsigned int sid,
    unsigned int nsphere, double* sphere);
/* decl:291, def:94-124.  Stable sort of (hash,index) by hash in place, then
 * cell start (0xffffffff when empty) / end and sorted_index. */
XDEM_API int cu_reorderDataAndFindCellStart(unsigned int* hash,
                                            unsigned int* index,
                                            unsigned int* cstart,
                                            unsigned int* cend,
                                            unsigned int* sorted_index,
                                            unsigned int np,
                                            unsigned int ncell);
/* No counterpart in the reference.  Same arguments and result as
 * cu_reorderDataAndFindCellStart, but it allocates no device memory: the sort
 * scratch is a fixed array inside the library (about 2.2 MB on every GPU that
 * loads the library, kept until the process exits), for callers that may not
 * call cudaMalloc -- a real-time loop that cannot risk an allocation's
 * latency or an out-of-memory failure mid-run, a host whose device memory
 * belongs to an external pool.
 * np (particles + mesh spheres) must not exceed 262144; larger calls return
 * XDEM_ERR_ARG without touching the arrays.  The first call on a device looks
 * up the array's device address; make that first call before any stream
 * capture.  All calls share the array, so calls whose kernels overlap on the
 * GPU (e.g. on two streams) race and must be serialised by the caller. */
XDEM_API int cu_reorderDataAndFindCellStart_noalloc(unsigned int* hash,
                                                    unsigned int* index,
                                                    unsigned int* cstart,
                                                    unsigned int* cend,
                                                    unsigned int* sorted_index,
                                                    unsigned int np,
                                                    unsigned int ncell);
/* decl:293-299, def:126-143 */
XDEM_API int cu_calculate_p2p(double* pos, double* ep, double* vel,
                              double* omega, double* force, double* moment,
                              double* mass, double* tmax, double* rres,
                              unsigned int* pair_count, unsigned int* pair_id,
                              double* tsd, unsigned int* sorted_index,
                              unsigned int* cstart, unsigned int* cend,
                              device_contact_property* cp, unsigned int np);
/* decl:301-308, def:145-184 (one plane per launch; plan->id selects the
 * slot rule) */
XDEM_API int cu_plane_contact_force(device_plane_info* plan, double* dbi,
                                    device_contact_property* cp, double* pos,
                                    double* ep, double* vel, double* omega,
                                    double* force, double* moment,
                                    double* mass, double* tmax, double* rres,
                                    unsigned int* pair_count,
                                    unsigned int* pair_id, double* tsd,
                                    unsigned int np);
/* decl:316-324, def:238-263 */
XDEM_API int cu_particle_polygonObject_collision(
    device_triangle_info* dpi, double* dbi, double* pos, double* ep,
    double* vel, double* omega, double* force, double* moment, double* mass,
    double* tmax, double* rres, unsigned int* pair_count,
    unsigned int* pair_id, double* tsd, double* dsph, unsigned int* sidx,
    unsigned int* cstart, unsigned int* cend, device_contact_property* cp,
    unsigned int np, unsigned int ntriangle);
/* decl:336-343, def:265-283 */
XDEM_API int cu_decide_rolling_friction_moment(double* tmax, double* rres,
                                               double* inertia, double* ep,
                                               double* ev, double* moment,
                                               unsigned int np);
/* decl:344, def:285-317.  Sum of np doubles (device) returned to the host. */
XDEM_API double reduction(double* in, unsigned int np);
/* decl:345-347, def:319-331 */
XDEM_API int cu_update_meshObjectData(double* vList, double* sph,
                                      double* dlocal,
                                      device_triangle_info* poly, double* dbi,
                                      unsigned int ntriangle);
/* decl:349-354, def:333-349 */
XDEM_API int cu_clusters_contact(double* pos, double* cpos, double* ep,
                                 double* vel, double* omega, double* force,
                                 double* moment, double* mass, double* tmax,
                                 double* rres, unsigned int* pair_count,
                                 unsigned int* pair_id, double* tsd,
                                 unsigned int* sorted_index,
                                 unsigned int* cstart, unsigned int* cend,
                                 device_contact_property* cp,
                                 xClusterInformation* xci, unsigned int np);
/* decl:356-362, def:351-393 */
XDEM_API int cu_cluster_plane_contact(device_plane_info* plan, double* dbi,
                                      device_contact_property* cp,
                                      double* pos, double* cpos, double* ep,
                                      double* vel, double* omega,
                                      double* force, double* moment,
                                      double* mass, double* tmax,
                                      double* rres, unsigned int* pair_count,
                                      unsigned int* pair_id, double* tsd,
                                      xClusterInformation* xci,
                                      unsigned int np);
/* decl:326-335, def:209-238: particles against one cylinder posed by the
 * 15-double record bi; pairs in MAX_P2CY_COUNT slots per particle (the
 * reference's xParticleCylinderContact arrays); body force partials as the
 * plane launcher */
XDEM_API int cu_cylinder_contact_force(device_cylinder_info* cyl, double* bi,
                                       device_contact_property* cp,
                                       double* pos, double* ep, double* vel,
                                       double* omega, double* force,
                                       double* moment, double* mass,
                                       double* tmax, double* rres,
                                       unsigned int* pair_count,
                                       unsigned int* pair_id, double* tsd,
                                       unsigned int np);
/* decl:366-373, def:395-420 */
XDEM_API int cu_cluster_cylinder_contact(device_cylinder_info* cyl, double* bi,
                                         xClusterInformation* xci,
                                         device_contact_property* cp,
                                         double* pos, double* cpos,
                                         double* ep, double* vel,
                                         double* omega, double* force,
                                         double* moment, double* mass,
                                         double* tmax, double* rres,
                                         unsigned int* pair_count,
                                         unsigned int* pair_id, double* tsd,
                                         unsigned int np);
/* decl:373-381, def:422-471 */
XDEM_API int cu_cluster_meshes_contact(
    device_triangle_info* dpi, double* dbi, double* pos, double* cpos,
    double* ep, double* vel, double* ev, double* force, double* moment,
    device_contact_property* cp, double* mass, double* tmax, double* rres,
    unsigned int* pair_count, unsigned int* pair_id, double* tsd,
    unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend,
    xClusterInformation* xci, unsigned int np, unsigned int ntriangle);
/* decl:383-391, def:473-493 */
XDEM_API int cu_decide_cluster_rolling_friction_moment(
    double* tmax, double* rres, double* inertia, double* ep, double* ev,
    double* moment, xClusterInformation* xci, unsigned int np);
/* decl:393-396, def:495-513 */
XDEM_API int vv_update_cluster_position(double* pos, double* cpos, double* ep,
                                        double* rloc, double* vel,
                                        double* acc, double* omega,
                                        double* alpha,
                                        xClusterInformation* xci,
                                        unsigned int np);
/* decl:398-401, def:515-536 */
XDEM_API int vv_update_cluster_velocity(double* cpos, double* ep, double* vel,
                                        double* acc, double* omega,
                                        double* alpha, double* force,
                                        double* moment, double* rloc,
                                        double* mass, double* iner,
                                        xClusterInformation* xci,
                                        unsigned int np);

/* ------------------------------------------------------------------------ */
/* Scene surface: handle API over the fused sorted-order step               */
/* ------------------------------------------------------------------------ */

enum { XDEM_FP64 = 0, XDEM_MIXED = 1 };

typedef struct xdem_sim xdem_sim;

typedef struct xdem_sim_config {
    unsigned int np;          /* spheres (cluster members included)          */
    unsigned int ns;          /* clusters; 0 = free spheres (ns = np)        */
    int precision;            /* XDEM_FP64 or XDEM_MIXED.  Mixed cluster
                                 handles need one member count for every
                                 cluster type and no rolling resistance or
                                 cohesion; xdem_sim_step returns
                                 XDEM_ERR_ARG otherwise                      */
    int contact_model;        /* 0 DHS, 1 Hertz-Mindlin                      */
    int velocity_compat;      /* see xdem_set_velocity_compat                */
    double dt;
    double gravity[3];
    double world_origin[3];
    double cell_size;
    unsigned int grid_size[3];/* powers of two; 128^3 in the reference      */
    int launcher_path;        /* 1: run the launcher kernels in the order of
                                 xIntegratorVV (reference structure); 0: the
                                 fused sorted-order step (default)           */
} xdem_sim_config;

XDEM_API int xdem_sim_create(const xdem_sim_config* cfg, xdem_sim** out);
XDEM_API int xdem_sim_destroy(xdem_sim* sim);
/* Host arrays, reference layout: pos[np*4], vel/acc[ns*3], ep/ev/ea[ns*4],
 * mass[ns], inertia[ns*3].  Any pointer but pos/mass/inertia may be NULL
 * (zero; ep defaults to (1,0,0,0)).  A NaN or infinite entry returns
 * XDEM_ERR_NONFINITE | XDEM_ERR_ARG before anything is uploaded. */
XDEM_API int xdem_sim_set_state(xdem_sim* sim, const double* pos,
                                const double* vel, const double* acc,
                                const double* ep, const double* ev,
                                const double* ea, const double* mass,
                                const double* inertia);
/* Clusters: cpos[ns*4], xci[nco], rloc[nrloc*3] (host). */
XDEM_API int xdem_sim_set_clusters(xdem_sim* sim, const double* cpos,
                                   const xClusterInformation* xci,
                                   unsigned int nco, const double* rloc,
                                   unsigned int nrloc);
XDEM_API int xdem_sim_set_pp_contact(xdem_sim* sim,
                                     const device_contact_property* cp);
/* Batched scenes (parameter sweeps): declares that the handle's particles
 * form nscene independent scenes -- particles [first[s], first[s+1]) with
 * particle-particle contact property pp_cp[s] and planes
 * [plane_first[s], plane_first[s+1]) (plane indices in the order of
 * xdem_sim_add_plane; planes must all be added before the next step).
 * Particles of different scenes never form contacts; each scene's first
 * plane starts its plane list as plane 0 does in a single scene.  A batch
 * runs the fused step only (no clusters, meshes or launcher_path) and keeps
 * no body wrenches (xdem_sim_body_wrench returns XDEM_ERR_ARG).  For speed
 * the scenes should sit apart in space (the same grid serves all of them). */
XDEM_API int xdem_sim_set_scenes(xdem_sim* sim, unsigned int nscene,
                                 const unsigned int* first,
                                 const device_contact_property* pp_cp,
                                 const unsigned int* plane_first);
/* Kinetic energy and stored particle-particle + particle-plane contacts of
 * every scene of a batch (host arrays of nscene entries). */
XDEM_API int xdem_sim_scene_energy(xdem_sim* sim, double* ke,
                                   unsigned int* ncontact);
/* Adds a plane; returns its body index through *body (planes and meshes
 * share one body numbering). */
XDEM_API int xdem_sim_add_plane(xdem_sim* sim, const device_plane_info* plane,
                                const double body[15],
                                const device_contact_property* cp,
                                int* body_index);
/* Adds a cylinder (xParticleCylinderContact): its id is its rank among the
 * handle's cylinders.  Planes come first, then cylinders, then meshes.  An
 * XDEM_FP64 handle with cylinders steps on the FP64 launcher kernels; an
 * XDEM_MIXED handle (spheres or clusters) runs them in its fused step (FP64
 * region geometry, FP32 forces).  xdem_sim_step returns XDEM_ERR_ARG for a
 * mixed handle with cylinders and batched scenes, or with cohesion in a
 * cylinder's contact property. */
XDEM_API int xdem_sim_add_cylinder(xdem_sim* sim, const device_cylinder_info* cyl,
                                   const double body[15],
                                   const device_contact_property* cp,
                                   int* body_index);
/* Adds a triangle mesh.  vlist_local[ntri*9] holds each triangle's P,Q,R in
 * the body frame (as xParticleMeshObjectContact::define uploads dvList). */
XDEM_API int xdem_sim_add_mesh(xdem_sim* sim, unsigned int ntri,
                               const double* vlist_local,
                               const double body[15],
                               const device_contact_property* cp,
                               int* body_index);
/* Triangles (current pose) and bounding spheres of a mesh body, host
 * arrays of ntri entries / ntri*4 doubles. */
XDEM_API int xdem_sim_get_mesh(xdem_sim* sim, int body_index,
                               device_triangle_info* tri, double* sphere,
                               unsigned int* ntri);
/* Pose exchange with the host solver: new 15-double record (and, for a
 * plane, its frame) for the next step.  plane may be NULL. */
XDEM_API int xdem_sim_set_body(xdem_sim* sim, int body_index,
                               const double body[15],
                               const device_plane_info* plane);
/* Advances nsteps steps (no host synchronisation). */
XDEM_API int xdem_sim_step(xdem_sim* sim, unsigned int nsteps);
/* Wrench of the last step on a body: (fx,fy,fz,mx,my,mz).  Synchronises. */
XDEM_API int xdem_sim_body_wrench(xdem_sim* sim, int body_index,
                                  double out6[6]);
/* The same exchange for several bodies in one call each way.  The reference
 * exchanges body by body: xParticlePlaneContact::update and
 * xParticleMeshObjectContact::update copy each pose in
 * (xParticlePlaneContact.cpp:96-131, xParticleMeshObjectContact.cpp:169-184)
 * and `reduction` + xPointMass::addContactForce read each wrench back
 * (decl:285-317, xPointMass.cpp:159-168).
 * xdem_sim_set_bodies: bodies is count x 15 doubles, planes count entries
 * (read for plane bodies; NULL keeps every frame).  Results equal count
 * xdem_sim_set_body calls in list order; the body records and plane tables
 * go up in one copy each from pinned staging, and the call does not wait
 * for the copies.  xdem_sim_body_wrenches: out is count x 6 doubles, from one
 * device-to-host copy of every body's wrench; synchronises. */
XDEM_API int xdem_sim_set_bodies(xdem_sim* sim, int count,
                                 const int* body_index, const double* bodies,
                                 const device_plane_info* planes);
XDEM_API int xdem_sim_body_wrenches(xdem_sim* sim, int count,
                                    const int* body_index, double* out);
/* Copies the state back to host arrays (reference layout); NULL skips. */
XDEM_API int xdem_sim_get_state(xdem_sim* sim, double* pos, double* vel,
                                double* acc, double* ep, double* ev,
                                double* ea, double* cpos);
/* kind: 0 particle-particle, 1 particle-plane, 2 particle-triangle,
 * 3 particle-cylinder (MAX_P2CY_COUNT slots).  set_pairs (and load_part, for
 * the lists of a file) returns XDEM_ERR_ARG, uploading nothing, when a count
 * exceeds the kind's slots or a stored id names no particle (kind 0), plane
 * (1), triangle (2) or cylinder (3: id, or id + 1000 for an inner cap) of the
 * handle. */
XDEM_API int xdem_sim_get_pairs(xdem_sim* sim, int kind, unsigned int* count,
                                unsigned int* ids, double* tsd);
XDEM_API int xdem_sim_set_pairs(xdem_sim* sim, int kind,
                                const unsigned int* count,
                                const unsigned int* ids, const double* tsd);
/* Kinetic energy (translational + rotational) and stored contact count. */
XDEM_API int xdem_sim_energy(xdem_sim* sim, double* ke, unsigned int* ncontact);
/* Part files (xResultManager::export_step_data_to_file,
 * source/xdynamics_manager/xResultManager.cpp:828-903, version 2): time,
 * counts, mass, state (and cluster centres), then the particle-pair, plane
 * and triangle pair lists with their tangential history, for the contact
 * kinds the handle has.  No multibody block: the handle's bodies are posed by
 * the caller.  load_part checks the counts and the file size against the
 * handle and restores the state and every pair list, history included (the
 * reference's resume leaves the lists empty, xContactManager.cpp:316-322);
 * the inertia stays the handle's. */
XDEM_API int xdem_sim_save_part(xdem_sim* sim, const char* path, double time);
XDEM_API int xdem_sim_load_part(xdem_sim* sim, const char* path, double* time);
/* Status bits accumulated since the last call. */
XDEM_API int xdem_sim_status(xdem_sim* sim);
/* The same switch as xdem_set_rolling_inertia, for this handle's steps. */
XDEM_API int xdem_sim_set_rolling_inertia(xdem_sim* sim, int per_sphere);
/* Stream the handle's kernels run on (cudaStream_t).  The stream stays the
 * caller's: keep it alive while the handle uses it; xdem_sim_destroy never
 * destroys it.  NULL returns to the handle's own stream. */
XDEM_API int xdem_sim_set_stream(xdem_sim* sim, void* stream);
/* Kernel timing of the last xdem_sim_step call: number of launches and the
 * time of the particle-particle contact kernel, in milliseconds, from CUDA
 * events recorded on the handle's stream when profiling is on. */
XDEM_API int xdem_sim_set_profiling(xdem_sim* sim, int on);
/* Replays the fused step from CUDA graphs (one per arrangement of the
 * double-buffered arrays, captured on first use and again after any change
 * of state arrays, bodies or contact tables), one graph launch per step
 * instead of about 14 kernel launches.  Profiling (xdem_sim_set_profiling)
 * runs the steps eagerly.  Results are identical either way. */
XDEM_API int xdem_sim_set_graph(xdem_sim* sim, int on);
/* Persistent batched step: with on != 0, each list step of a batched mixed
 * handle (xdem_sim_set_scenes, candidate lists) is one cooperative kernel
 * launch -- the gated cell sort, the particle-pair phase, the body phase and
 * the list-flag roll separated by grid barriers -- instead of four to
 * sixteen kernels; with xdem_sim_set_graph the step graph holds that one
 * kernel (after a memset of the barrier's two words).  Results are identical
 * either way.  Each barrier waits at most barrier_limit_ns (0: one second)
 * on the GPU's global timer; a block that waits longer raises
 * XDEM_ERR_BARRIER in the status and the kernel returns, leaving the step
 * incomplete (restore a state, e.g. with xdem_sim_set_state, to go on).
 * Other handles and the first step after a new state run the usual
 * kernels.  Returns XDEM_OK or XDEM_ERR_ARG. */
XDEM_API int xdem_sim_set_persistent(xdem_sim* sim, int on, unsigned long long barrier_limit_ns);
XDEM_API int xdem_sim_profile(xdem_sim* sim, unsigned int* launches,
                              double* contact_ms, unsigned int* contact_launches);

/* Block shapes of the mixed contact stage (XDEM_MIXED handles): threads per
 * block of the pair kernel and of the body kernel (64, 128 or 256), the
 * depth of the pair kernel's per-thread candidate stage (8 or 16), and the
 * resident threads per SM each kernel is compiled for, i.e. its register
 * budget (occ_pairs 768 or 1024; occ_bodies 512, 768 or 1024).  A handle
 * that keeps body wrenches (one scene with planes or meshes) needs
 * nt_pairs == nt_bodies.  Shapes never change results.  contact_ms: mean
 * event-timed contact stage of a step (autotune only).  No counterpart in
 * the reference, whose launchers fix 256 threads per block. */
typedef struct xdem_tune {
    unsigned int nt_pairs, stage, nt_bodies, occ_pairs, occ_bodies;
    unsigned int skin_div;  /* pair search: 0 walks the 27-cell stencil every step; 8, 16 or 32 keep a
                               candidate list per sphere with a skin of cell_size / skin_div, rebuilt on
                               the device when a sphere has moved more than half the skin */
    double contact_ms;
} xdem_tune;
XDEM_API int xdem_sim_set_tune(xdem_sim* sim, const xdem_tune* tune);
XDEM_API int xdem_sim_get_tune(xdem_sim* sim, xdem_tune* tune);
/* Times candidate shapes for trial_steps steps each (after 2 warm-up steps)
 * on the handle's scene, keeps the fastest in *best and on the handle, and
 * puts the state back as it was: tuning does not advance the simulation.
 * A wrench-keeping handle tries every joint shape with equal block sizes
 * (36); a batch tunes the pair kernel (12 shapes), then the body kernel (9).
 * Either then tries the four pair searches (skin_div 0, 8, 16, 32).
 * all[0..*nall) receives every candidate with its time when given (*nall is
 * its capacity on entry, the number of candidates on return).  FP64 and
 * launcher-path handles have nothing to tune: *best is their fixed shape. */
XDEM_API int xdem_sim_autotune(xdem_sim* sim, unsigned int trial_steps, xdem_tune* best, xdem_tune* all,
                               unsigned int* nall);
/* Candidate-list rebuilds triggered by motion since the handle's tables were
 * made (the build on the first step after a state change is not counted). */
XDEM_API int xdem_sim_list_rebuilds(xdem_sim* sim, unsigned int* rebuilds);

/* ------------------------------------------------------------------------ */
/* Adjoint of the FP64 trajectory (reverse mode, checkpointed)              */
/* ------------------------------------------------------------------------ */
/* Gradients of a loss on the final positions / velocities of a trajectory
 * of the handle with respect to each contact property's friction,
 * restitution and Young's moduli (device_contact_property fric, rest, Ei,
 * Ej).  Supported: XDEM_FP64 handles of free spheres and planes, contact
 * model 0 or 1, no cohesion, no rolling resistance, one scene, at most 16
 * planes.  The forward stores the state every `checkpoint_every` steps; the
 * backward re-runs each segment from its checkpoint and reverses it.
 * Bodies must not be moved (xdem_sim_set_body) between forward and
 * backward.  The reference has no adjoint: this is new surface. */
typedef struct xdem_adj xdem_adj;
XDEM_API int xdem_adj_create(xdem_sim* sim, unsigned int checkpoint_every, xdem_adj** out);
XDEM_API int xdem_adj_destroy(xdem_adj* adj);
/* Advances the handle nsteps from its current state, keeping checkpoints.
 * Returns the handle's status bits of those steps (pair-list overflow or
 * non-finite positions leave no usable adjoint). */
XDEM_API int xdem_adj_forward(xdem_adj* adj, unsigned int nsteps);
/* dl_dpos, dl_dvel: DEVICE arrays [np*3] of the loss gradient at the final
 * state (NULL = 0).  grad: HOST array [4 * nprop], per contact property
 * (0 = particle-particle, 1 + k = plane k) d/dfric, d/drest, d/dEi, d/dEj.
 * dl_dpos0, dl_dvel0: optional DEVICE arrays [np*3] receiving the gradient
 * with respect to the initial positions and velocities.  Leaves the handle
 * at the end of the first segment's re-run. */
XDEM_API int xdem_adj_backward(xdem_adj* adj, const double* dl_dpos, const double* dl_dvel, double* grad,
                               double* dl_dpos0, double* dl_dvel0);
/* Forward mode of the same linearisation (an independent check of the
 * adjoint): re-runs the trajectory of the last xdem_adj_forward from its
 * first checkpoint and carries the derivative of the state along it in
 * ndir <= 3 parameter directions at once.  dparam: HOST array [ndir][nprop]
 * [4] of d(fric, rest, Ei, Ej) per contact property.  tpos, tvel: optional
 * DEVICE arrays [ndir][np*3] receiving the derivative of the final
 * positions and velocities in each direction.  For a loss L of the final
 * state, dL/dx . tpos[k] equals grad . dparam[k] of xdem_adj_backward.
 * Leaves the handle at the end of the trajectory; returns the re-run's
 * status bits. */
XDEM_API int xdem_adj_tangent(xdem_adj* adj, unsigned int ndir, const double* dparam, double* tpos, double* tvel);
/* Properties (1 + planes), steps of the last forward, device bytes held. */
XDEM_API int xdem_adj_info(xdem_adj* adj, unsigned int* nprop, unsigned int* nsteps, unsigned long long* bytes);

/* ------------------------------------------------------------------------ */
/* Host multibody side of the coupling: HHT-alpha over rigid bodies         */
/* ------------------------------------------------------------------------ */
/* The rigid bodies the DEM bed pushes on (a wheel on its carriage) advanced
 * on the host by the HHT-alpha integrator of xIntegratorHHT
 * (source/xdynamics_simulation/xIntegratorHHT.cpp:51-183): Euler-parameter
 * coordinates, revolute and translational joints, a rotation driver on a
 * revolute joint, a Newton loop with a dense solve, the DEM wrench in the
 * force vector as xMultiBodySimulation::ConstructForceVector adds the
 * contact force and moment (xMultiBodySimulation.cpp:341-360).  Body 0 is
 * the ground.  Joints and the driver are defined at the bodies' poses when
 * they are added; xdem_mbd_initialize then solves the consistent
 * accelerations.  Host only: these calls touch no GPU.  Returns XDEM_OK or
 * XDEM_ERR_ARG (bad argument, singular system, or a step whose Newton loop
 * did not converge in 100 iterations; a failed step leaves the bodies, the
 * time and the multipliers as they were before it). */
typedef struct xdem_mbd xdem_mbd;
/* alpha in [-1/3, 0] (the reference uses -0.3); gravity may be NULL. */
XDEM_API int xdem_mbd_create(double dt, double alpha, const double gravity[3], xdem_mbd** out);
XDEM_API int xdem_mbd_destroy(xdem_mbd* mbd);
/* Newton tolerance on the residual norm (default 1e-5, the reference's). */
XDEM_API int xdem_mbd_set_tolerance(xdem_mbd* mbd, double eps);
/* Rigid body: mass, principal inertia (body frame), centre, Euler
 * parameters; vel and ed (Euler-parameter rates) may be NULL. */
XDEM_API int xdem_mbd_add_body(xdem_mbd* mbd, double mass, const double inertia[3], const double pos[3],
                               const double ep[4], const double vel[3], const double ed[4], int* body);
/* Revolute joint between bodies i and j at global point loc about the
 * global axis (5 equations); translational joint letting j slide along the
 * axis relative to i (5 equations). */
XDEM_API int xdem_mbd_add_revolute(xdem_mbd* mbd, int body_i, int body_j, const double loc[3],
                                   const double axis[3], int* joint);
XDEM_API int xdem_mbd_add_translational(xdem_mbd* mbd, int body_i, int body_j, const double loc[3],
                                        const double axis[3], int* joint);
/* Drives the rotation of a revolute joint's body j relative to body i about
 * the joint axis at omega rad/s from its present angle. */
XDEM_API int xdem_mbd_add_rotation_driver(xdem_mbd* mbd, int revolute_joint, double omega);
XDEM_API int xdem_mbd_initialize(xdem_mbd* mbd);
/* Contact force and moment (global frame, fx fy fz mx my mz) on a body,
 * held until replaced: the out6 of xdem_sim_body_wrench for that body. */
XDEM_API int xdem_mbd_set_contact_wrench(xdem_mbd* mbd, int body, const double w6[6]);
/* One HHT-alpha step of dt (prediction + Newton correction). */
XDEM_API int xdem_mbd_step(xdem_mbd* mbd, int* iterations);
/* Coordinates (r, p), their rates and accelerations; NULL skips. */
XDEM_API int xdem_mbd_get_body(xdem_mbd* mbd, int body, double q[7], double qd[7], double qdd[7]);
/* The body's 15-double record (decl:20) for xdem_sim_set_body(ies). */
XDEM_API int xdem_mbd_body_record(xdem_mbd* mbd, int body, double rec[15]);
XDEM_API int xdem_mbd_info(xdem_mbd* mbd, double* time, int* iterations, int* nconstraint);
/* Lagrange multipliers (joints 5 each, drivers, normalisations). */
XDEM_API int xdem_mbd_multipliers(xdem_mbd* mbd, double* lambda, int cap);

#ifdef __cplusplus
}
#endif

#endif /* XDEM_C_H */
