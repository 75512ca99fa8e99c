/*
 * xdem_compat.hpp -- the reference's launcher signatures for C++ callers.
 *
 * The reference declares its DEM launchers as C++ functions returning void
 * (include/xdynamics_parallel/xParallelDEM_decl.cuh:280-403 of xdynamics).
 * This header gives those exact names and signatures, as inline wrappers
 * around the extern "C" entry points of libxdem_gb300.so (xdem_c.h), which
 * discard the int status.  A source file of the reference includes this
 * header where it included xParallelDEM_decl.cuh and compiles unchanged.
 *
 * The C declarations live in namespace xdem_c_abi (their link names stay
 * the plain C names); the structs are brought into the global namespace.
 * Include either this header or xdem_c.h in a translation unit, not both:
 * xdem_c.h would declare the C functions in the global namespace, where
 * these wrappers already use the names.  The status of the last call on a
 * thread stays readable through xdem_c_abi::xdem_last_status().
 */
#ifndef XDEM_COMPAT_HPP
#define XDEM_COMPAT_HPP

namespace xdem_c_abi {
extern "C" {
#include "xdem_c.h"
}
}  // namespace xdem_c_abi

using xdem_c_abi::device_contact_property;
using xdem_c_abi::device_cylinder_info;
using xdem_c_abi::device_dem_parameters;
using xdem_c_abi::device_plane_info;
using xdem_c_abi::device_triangle_info;
using xdem_c_abi::xClusterInformation;

/* decl:280 */
inline void setDEMSymbolicParameter(device_dem_parameters* h_paras)
{
    (void)xdem_c_abi::setDEMSymbolicParameter(h_paras);
}
/* decl:282 */
inline void vv_update_position(double* pos, double* ep, double* vel, double* ev, double* acc, double* ea,
                               unsigned int np)
{
    (void)xdem_c_abi::vv_update_position(pos, ep, vel, ev, acc, ea, np);
}
/* decl:284 */
inline void vv_update_velocity(double* vel, double* acc, double* ep, double* ev, double* ea, double* force,
                               double* moment, double* mass, double* iner, unsigned int np)
{
    (void)xdem_c_abi::vv_update_velocity(vel, acc, ep, ev, ea, force, moment, mass, iner, np);
}
/* decl:287 */
inline void cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double* pos, unsigned int sid,
                                     unsigned int np)
{
    (void)xdem_c_abi::cu_calculateHashAndIndex(hash, index, pos, sid, np);
}
/* decl:288 */
inline void cu_calculateHashAndIndexForPolygonSphere(unsigned int* hash, unsigned int* index, unsigned int sid,
                                                     unsigned int nsphere, double* sphere)
{
    (void)xdem_c_abi::cu_calculateHashAndIndexForPolygonSphere(hash, index, sid, nsphere, sphere);
}
/* decl:291 */
inline void cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                                           unsigned int* cend, unsigned int* sorted_index, unsigned int np,
                                           unsigned int ncell)
{
    (void)xdem_c_abi::cu_reorderDataAndFindCellStart(hash, index, cstart, cend, sorted_index, np, ncell);
}
/* decl:293 */
inline void cu_calculate_p2p(double* pos, double* ep, double* vel, double* omega, double* force, double* moment,
                             double* mass, double* tmax, double* rres, unsigned int* pair_count,
                             unsigned int* pair_id, double* tsd, unsigned int* sorted_index, unsigned int* cstart,
                             unsigned int* cend, device_contact_property* cp, unsigned int np)
{
    (void)xdem_c_abi::cu_calculate_p2p(pos, ep, vel, omega, force, moment, mass, tmax, rres, pair_count, pair_id,
                                       tsd, sorted_index, cstart, cend, cp, np);
}
/* decl:302 */
inline void cu_plane_contact_force(device_plane_info* plan, double* dbi, device_contact_property* cp, double* pos,
                                   double* ep, double* vel, double* omega, double* force, double* moment,
                                   double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                   unsigned int* pair_id, double* tsd, unsigned int np)
{
    (void)xdem_c_abi::cu_plane_contact_force(plan, dbi, cp, pos, ep, vel, omega, force, moment, mass, tmax, rres,
                                             pair_count, pair_id, tsd, np);
}
/* decl:317 */
inline void cu_particle_polygonObject_collision(device_triangle_info* dpi, double* dbi, double* pos, double* ep,
                                                double* vel, double* omega, double* force, double* moment,
                                                double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                                unsigned int* pair_id, double* tsd, double* dsph,
                                                unsigned int* sidx, unsigned int* cstart, unsigned int* cend,
                                                device_contact_property* cp, unsigned int np,
                                                unsigned int ntriangle)
{
    (void)xdem_c_abi::cu_particle_polygonObject_collision(dpi, dbi, pos, ep, vel, omega, force, moment, mass, tmax,
                                                          rres, pair_count, pair_id, tsd, dsph, sidx, cstart, cend,
                                                          cp, np, ntriangle);
}
/* decl:327 */
inline void cu_cylinder_contact_force(device_cylinder_info* cyl, double* bi, device_contact_property* cp,
                                      double* pos, double* ep, double* vel, double* omega, double* force,
                                      double* moment, double* mass, double* tmax, double* rres,
                                      unsigned int* pair_count, unsigned int* pair_id, double* tsd, unsigned int np)
{
    (void)xdem_c_abi::cu_cylinder_contact_force(cyl, bi, cp, pos, ep, vel, omega, force, moment, mass, tmax, rres,
                                                pair_count, pair_id, tsd, np);
}
/* decl:336 */
inline void cu_decide_rolling_friction_moment(double* tmax, double* rres, double* inertia, double* ep, double* ev,
                                              double* moment, unsigned int np)
{
    (void)xdem_c_abi::cu_decide_rolling_friction_moment(tmax, rres, inertia, ep, ev, moment, np);
}
/* decl:345 */
inline double reduction(double* in, unsigned int np) { return xdem_c_abi::reduction(in, np); }
/* decl:346 */
inline void cu_update_meshObjectData(double* vList, double* sph, double* dlocal, device_triangle_info* poly,
                                     double* dbi, unsigned int ntriangle)
{
    (void)xdem_c_abi::cu_update_meshObjectData(vList, sph, dlocal, poly, dbi, ntriangle);
}
/* decl:350 */
inline void cu_clusters_contact(double* pos, double* cpos, double* ep, double* vel, double* omega, double* force,
                                double* moment, double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                unsigned int* pair_id, double* tsd, unsigned int* sorted_index,
                                unsigned int* cstart, unsigned int* cend, device_contact_property* cp,
                                xClusterInformation* xci, unsigned int np)
{
    (void)xdem_c_abi::cu_clusters_contact(pos, cpos, ep, vel, omega, force, moment, mass, tmax, rres, pair_count,
                                          pair_id, tsd, sorted_index, cstart, cend, cp, xci, np);
}
/* decl:358 */
inline void cu_cluster_plane_contact(device_plane_info* plan, double* dbi, device_contact_property* cp, double* pos,
                                     double* cpos, double* ep, double* vel, double* omega, double* force,
                                     double* moment, double* mass, double* tmax, double* rres,
                                     unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                     xClusterInformation* xci, unsigned int np)
{
    (void)xdem_c_abi::cu_cluster_plane_contact(plan, dbi, cp, pos, cpos, ep, vel, omega, force, moment, mass, tmax,
                                               rres, pair_count, pair_id, tsd, xci, np);
}
/* decl:366 */
inline void cu_cluster_cylinder_contact(device_cylinder_info* cyl, double* bi, xClusterInformation* xci,
                                        device_contact_property* cp, double* pos, double* cpos, double* ep,
                                        double* vel, double* omega, double* force, double* moment, double* mass,
                                        double* tmax, double* rres, unsigned int* pair_count,
                                        unsigned int* pair_id, double* tsd, unsigned int np)
{
    (void)xdem_c_abi::cu_cluster_cylinder_contact(cyl, bi, xci, cp, pos, cpos, ep, vel, omega, force, moment, mass,
                                                  tmax, rres, pair_count, pair_id, tsd, np);
}
/* decl:375 */
inline void cu_cluster_meshes_contact(device_triangle_info* dpi, double* dbi, double* pos, double* cpos, double* ep,
                                      double* vel, double* ev, double* force, double* moment,
                                      device_contact_property* cp, double* mass, double* tmax, double* rres,
                                      unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                      unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend,
                                      xClusterInformation* xci, unsigned int np, unsigned int ntriangle)
{
    (void)xdem_c_abi::cu_cluster_meshes_contact(dpi, dbi, pos, cpos, ep, vel, ev, force, moment, cp, mass, tmax, rres,
                                                pair_count, pair_id, tsd, sorted_index, cstart, cend, xci, np,
                                                ntriangle);
}
/* decl:385 */
inline void cu_decide_cluster_rolling_friction_moment(double* tmax, double* rres, double* inertia, double* ep,
                                                      double* ev, double* moment, xClusterInformation* xci,
                                                      unsigned int np)
{
    (void)xdem_c_abi::cu_decide_cluster_rolling_friction_moment(tmax, rres, inertia, ep, ev, moment, xci, np);
}
/* decl:395 */
inline void vv_update_cluster_position(double* pos, double* cpos, double* ep, double* rloc, double* vel,
                                       double* acc, double* omega, double* alpha, xClusterInformation* xci,
                                       unsigned int np)
{
    (void)xdem_c_abi::vv_update_cluster_position(pos, cpos, ep, rloc, vel, acc, omega, alpha, xci, np);
}
/* decl:400 */
inline void vv_update_cluster_velocity(double* cpos, double* ep, double* vel, double* acc, double* omega,
                                       double* alpha, double* force, double* moment, double* rloc, double* mass,
                                       double* iner, xClusterInformation* xci, unsigned int np)
{
    (void)xdem_c_abi::vv_update_cluster_velocity(cpos, ep, vel, acc, omega, alpha, force, moment, rloc, mass, iner,
                                                 xci, np);
}

#endif /* XDEM_COMPAT_HPP */
