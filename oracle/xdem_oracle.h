/*
 * xdem_oracle.h -- CPU oracle of the xdynamics DEM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64, contraction-free
 * (-ffp-contract=off) restatement of the reference's DEM kernels
 * (include/xdynamics_parallel/xParallelDEM_impl.cuh of miniwooki/xdynamics_dll)
 * used by the tests as the checker and by bench.py as the CPU baseline.  The
 * library under test never links, loads or calls it.
 *
 * Every function takes host arrays in the reference layout and follows one
 * reference kernel; each cites the lines it restates.  Per-particle loops are
 * OpenMP-parallel when built with -fopenmp: each iteration writes only its own
 * particle's outputs, as each GPU thread of the reference does, so results do
 * not depend on the thread count.
 *
 * Documented deviations from the literal reference (also applied by the GPU
 * library, so both agree):
 *  - pair-list and candidate overflow: the reference writes past the
 *    particle's slots into its neighbour's (impl:704-706,727-728); here the
 *    contact force is still applied, the pair is not stored, and a status bit
 *    (XDEM_ERR_*) is raised.
 *  - pow(x, 2.0) in the plane test (impl:738-739) is computed as x*x.
 *  - the double->int conversion of the cell coordinate saturates (as the
 *    GPU's cvt.rzi does) instead of being undefined for huge/NaN values.
 *  - sphere velocity: see xo_vv_update_velocity.
 */
#ifndef XDEM_ORACLE_H
#define XDEM_ORACLE_H

#include "../include/xdem_c.h"

#ifdef __cplusplus
extern "C" {
#endif

int xo_num_threads(void);
void xo_set_num_threads(int n);

/* impl:135-147 */
void xo_vv_update_position(const device_dem_parameters* prm, double* pos,
                           double* ep, const double* vel, const double* ev,
                           const double* acc, const double* ea,
                           unsigned int np);
/* impl:192-222; vel_compat=1 keeps the reference GPU's unchanged velocity */
void xo_vv_update_velocity(const device_dem_parameters* prm, double* vel,
                           double* acc, const double* ep, double* ev,
                           double* ea, double* force, double* moment,
                           const double* mass, const double* iner,
                           unsigned int np, int vel_compat);
/* impl:290-315 (spheres of particles or of triangles: same arithmetic) */
void xo_hash(const device_dem_parameters* prm, unsigned int* hash,
             unsigned int* index, const double* pos, unsigned int sid,
             unsigned int np, unsigned int* status);
/* def:94-124 + impl:317-360 (stable sort then cell start/end) */
void xo_reorder_cellstart(unsigned int* hash, unsigned int* index,
                          unsigned int* cstart, unsigned int* cend,
                          unsigned int* sorted_index, unsigned int n,
                          unsigned int ncell);
/* impl:613-733 */
void xo_p2p(const device_dem_parameters* prm, const double* pos,
            const double* ep, const double* vel, const double* ev,
            double* force, double* moment, const double* mass, double* tmax,
            double* rres, unsigned int* pair_count, unsigned int* pair_id,
            double* tsd, const unsigned int* sorted_index,
            const unsigned int* cstart, const unsigned int* cend,
            const device_contact_property* cp, unsigned int np,
            unsigned int* status);
/* impl:950-1080 (one plane) */
void xo_plane(const device_dem_parameters* prm, const device_plane_info* plane,
              const double* dbi, const device_contact_property* cp,
              double* fx, double* fy, double* fz, double* mx, double* my,
              double* mz, const double* pos, const double* ep,
              const double* vel, const double* ev, double* force,
              double* moment, const double* mass, double* tmax, double* rres,
              unsigned int* pair_count, unsigned int* pair_id, double* tsd,
              unsigned int np, unsigned int* status);
/* impl:1930-2109 */
void xo_mesh(const device_dem_parameters* prm, const device_triangle_info* dti,
             const double* dbi, double* fx, double* fy, double* fz, double* mx,
             double* my, double* mz, const double* pos, const double* ep,
             const double* vel, const double* ev, double* force,
             double* moment, const double* mass, double* tmax, double* rres,
             unsigned int* pair_count, unsigned int* pair_id, double* tsd,
             const unsigned int* sorted_index, const unsigned int* cstart,
             const unsigned int* cend, const device_contact_property* cp,
             unsigned int np, unsigned int ntriangle, unsigned int* status);
/* impl:2420-2454 */
void xo_rolling(const device_dem_parameters* prm, double* tmax, double* rres,
                const double* inertia, const double* ep, const double* ev,
                double* moment, unsigned int np);
/* xo_rolling with per_sphere = 1: J = inertia[3 i], the sphere's own entry
 * (impl:2434 reads the flat entry i of the double3 array) */
void xo_rolling_ex(const device_dem_parameters* prm, double* tmax, double* rres,
                   const double* inertia, const double* ep, const double* ev,
                   double* moment, unsigned int np, int per_sphere);
/* impl:2544-2601 */
void xo_update_mesh(const double* dbi, const double* vList, double* sphere,
                    const double* dlocal, device_triangle_info* dpi,
                    unsigned int ntriangle);
/* impl:485-611 */
void xo_clusters_p2p(const device_dem_parameters* prm, const double* pos,
                     const double* cpos, const double* ep, const double* vel,
                     const double* ev, double* force, double* moment,
                     const double* mass, double* tmax, double* rres,
                     unsigned int* pair_count, unsigned int* pair_id,
                     double* tsd, const unsigned int* sorted_index,
                     const unsigned int* cstart, const unsigned int* cend,
                     const device_contact_property* cp,
                     const xClusterInformation* xci, unsigned int np,
                     unsigned int* status);
/* impl:817-948 */
void xo_cluster_plane(const device_dem_parameters* prm,
                      const device_plane_info* plane, const double* dbi,
                      double* fx, double* fy, double* fz, double* mx,
                      double* my, double* mz, const double* pos,
                      const double* cpos, const double* ep, const double* vel,
                      const double* ev, double* force, double* moment,
                      const device_contact_property* cp, const double* mass,
                      double* tmax, double* rres, unsigned int* pair_count,
                      unsigned int* pair_id, double* tsd,
                      const xClusterInformation* xci, unsigned int np,
                      unsigned int* status);
/* impl:1083-1601: one cylinder against every particle; cpos == NULL for
 * free spheres, else cluster members (xci, cluster state) */
void xo_cylinder(const device_dem_parameters* prm, const device_cylinder_info* cyl,
                 const double* bi, const device_contact_property* cp, double* fx,
                 double* fy, double* fz, double* mx, double* my, double* mz,
                 const double* pos, const double* cpos, const double* ep,
                 const double* vel, const double* ev, double* force,
                 double* moment, const double* mass, double* tmax, double* rres,
                 unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                 const xClusterInformation* xci, unsigned int np,
                 unsigned int* status);
/* impl:2111-2268 */
void xo_cluster_mesh(const device_dem_parameters* prm,
                     const device_triangle_info* dti, const double* dbi,
                     double* fx, double* fy, double* fz, double* mx,
                     double* my, double* mz, const double* pos,
                     const double* cpos, const double* ep, const double* vel,
                     const double* ev, double* force, double* moment,
                     const device_contact_property* cp, const double* mass,
                     double* tmax, double* rres, unsigned int* pair_count,
                     unsigned int* pair_id, double* tsd,
                     const unsigned int* sorted_index,
                     const unsigned int* cstart, const unsigned int* cend,
                     const xClusterInformation* xci, unsigned int np,
                     unsigned int ntriangle, unsigned int* status);
/* impl:2456-2500 */
void xo_cluster_rolling(const device_dem_parameters* prm, double* tmax,
                        double* rres, const double* inertia, const double* ep,
                        const double* ev, double* moment,
                        const xClusterInformation* xci, unsigned int np);
/* impl:149-190 */
void xo_vv_cluster_position(const device_dem_parameters* prm, double* pos,
                            double* cpos, double* ep, const double* rloc,
                            const double* vel, const double* acc,
                            const double* ev, const double* ea,
                            const xClusterInformation* xci, unsigned int ns);
/* impl:224-287 */
void xo_vv_cluster_velocity(const device_dem_parameters* prm,
                            const double* cpos, const double* ep, double* vel,
                            double* acc, double* ev, double* ea, double* force,
                            double* moment, const double* rloc,
                            const double* mass, const double* iner,
                            const xClusterInformation* xci, unsigned int ns);
/* xUtilityFunction.cpp:379-416 */
void xo_fit_sphere_to_triangle(const double P[3], const double Q[3],
                               const double R[3], double ft, double out[4]);
/* Sum of n doubles in index order (def:285-317 reduces with thrust). */
double xo_sum(const double* in, unsigned int n);

/* ------------------------------------------------------------------------ */
/* Whole step (xIntegratorVV.cpp:26-63 with xContactManager.cpp:458-472).   */
/* ------------------------------------------------------------------------ */
typedef struct xo_scene {
    device_dem_parameters prm;
    unsigned int np, ns;        /* spheres, clusters (ns == np: no clusters) */
    int vel_compat;
    double *pos, *cpos, *vel, *acc, *ep, *ev, *ea;
    double *force, *moment, *mass, *inertia, *tmax, *rres;
    /* clusters */
    xClusterInformation* xci; unsigned int nco; double* rloc;
    /* grid over np + sum(ntri) entries */
    unsigned int nentry, ncell;
    unsigned int *hash, *index, *cstart, *cend, *sorted_index;
    /* particle-particle */
    int has_pp; device_contact_property pp_cp;
    unsigned int *pp_count, *pp_id; double* pp_tsd;
    /* planes */
    unsigned int nplane;
    device_plane_info* plane; double* plane_body; /* 15 per plane */
    device_contact_property* plane_cp;
    unsigned int *pl_count, *pl_id; double* pl_tsd;
    /* meshes: triangles of all meshes in one array, mesh m owns
       [tri_begin[m], tri_begin[m]+ntri[m]) */
    unsigned int nmesh; unsigned int *tri_begin, *ntri;
    device_triangle_info* tri; double *tri_sphere, *tri_vlist, *tri_local;
    double* mesh_body;          /* 15 per mesh */
    device_contact_property* mesh_cp;
    unsigned int *ms_count, *ms_id; double* ms_tsd;
    /* body partials and per-body wrench of the last step (6 per body:
       planes first, then meshes) */
    double *bfx, *bfy, *bfz, *bmx, *bmy, *bmz;
    double* wrench;
    unsigned int status;
} xo_scene;

/* Advances the scene one step; returns accumulated status bits. */
unsigned int xo_step(xo_scene* s);

#ifdef __cplusplus
}
#endif
#endif
