/*
 * ref_driver.cpp -- runs the reference's own DEM kernels on the host.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file against the
 * unmodified include/xdynamics_parallel/xParallelDEM_impl.cuh of the
 * reference (read in place, never copied) with the stand-in headers of
 * oracle/ref_shim, producing oracle/_ref/libxdem_ref.so.  The tests use it to
 * check the C oracle (xdem_oracle.c) and the golden fixtures against the
 * reference's own arithmetic.
 *
 * Each ref_* entry point emulates one launch: every thread id runs the
 * kernel body with blockIdx/threadIdx set as CUDA would set them for
 * 128-thread blocks (def:30-34).  The sort of cu_reorderDataAndFindCellStart
 * (thrust::sort_by_key, def:107-109) is a stable sort here; its cell
 * start/end kernel runs with one-thread blocks so that the shared-memory
 * neighbour compare (impl:317-360) sees the previous key through
 * sharedHash[0].
 */
#include "xdynamics_decl.h"
#include "xdynamics_parallel/xParallelDEM_impl.cuh"

#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
unsigned int sharedHash[2];

template <class F>
static void launch(unsigned int n, F body)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 128)
#endif
    for (long id = 0; id < (long)n; ++id) {
        blockDim = dim3(128, 1, 1);
        gridDim = dim3((n + 127) / 128, 1, 1);
        blockIdx = make_uint3((unsigned int)(id / 128), 0, 0);
        threadIdx = make_uint3((unsigned int)(id % 128), 0, 0);
        body();
    }
}

extern "C" {

void ref_set_params(const void* p) { memcpy(&cte, p, sizeof(cte)); }
int ref_params_size(void) { return (int)sizeof(device_dem_parameters); }
int ref_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ref_vv_update_position(double* pos, double* ep, double* vel, double* ev, double* acc, double* ea,
                            unsigned int np)
{
    launch(np, [&] { vv_update_position_kernel((double4*)pos, (double4*)ep, (double3*)vel, (double4*)ev,
                                               (double3*)acc, (double4*)ea, np); });
}

void ref_vv_update_velocity(double* vel, double* acc, double* ep, double* ev, double* ea, double* force,
                            double* moment, double* mass, double* iner, unsigned int np)
{
    launch(np, [&] { vv_update_velocity_kernel((double3*)vel, (double3*)acc, (double4*)ep, (double4*)ev,
                                               (double4*)ea, (double3*)force, (double3*)moment, mass,
                                               (double3*)iner, np); });
}

void ref_hash(unsigned int* hash, unsigned int* index, double* pos, unsigned int sid, unsigned int np)
{
    launch(np, [&] { calculateHashAndIndex_kernel(hash, index, (double4*)pos, sid, np); });
}

void ref_reorder(unsigned int* hash, unsigned int* index, unsigned int* cstart, unsigned int* cend,
                 unsigned int* sorted_index, unsigned int np, unsigned int ncell)
{
    std::vector<std::pair<unsigned int, unsigned int>> kv(np);
    for (unsigned int i = 0; i < np; ++i) kv[i] = std::make_pair(hash[i], index[i]);
    std::stable_sort(kv.begin(), kv.end(),
                     [](const std::pair<unsigned int, unsigned int>& a,
                        const std::pair<unsigned int, unsigned int>& b) { return a.first < b.first; });
    for (unsigned int i = 0; i < np; ++i) { hash[i] = kv[i].first; index[i] = kv[i].second; }
    memset(cstart, 0xff, sizeof(unsigned int) * (size_t)ncell);
    memset(cend, 0, sizeof(unsigned int) * (size_t)ncell);
    for (unsigned int id = 0; id < np; ++id) {
        blockDim = dim3(1, 1, 1);
        blockIdx = make_uint3(id, 0, 0);
        threadIdx = make_uint3(0, 0, 0);
        reorderDataAndFindCellStart_kernel(hash, index, cstart, cend, sorted_index, np);
    }
}

void ref_p2p(double* pos, double* ep, double* vel, double* ev, double* force, double* moment, double* mass,
             double* tmax, double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
             unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend, void* cp, unsigned int np)
{
    launch(np, [&] {
        calculate_p2p_kernel((double4*)pos, (double4*)ep, (double3*)vel, (double4*)ev, (double3*)force,
                             (double3*)moment, mass, (double3*)tmax, rres, pair_count, pair_id, (double2*)tsd,
                             sorted_index, cstart, cend, (device_contact_property*)cp, np);
    });
}

void ref_plane(void* plane, double* dbi, void* cp, double* fx, double* fy, double* fz, double* mx, double* my,
               double* mz, double* pos, double* ep, double* vel, double* ev, double* force, double* moment,
               double* mass, double* tmax, double* rres, unsigned int* pair_count, unsigned int* pair_id,
               double* tsd, unsigned int np)
{
    launch(np, [&] {
        plane_contact_force_kernel((device_plane_info*)plane, dbi, (device_contact_property*)cp, fx, fy, fz, mx,
                                   my, mz, (double4*)pos, (double4*)ep, (double3*)vel, (double4*)ev,
                                   (double3*)force, (double3*)moment, mass, (double3*)tmax, rres, pair_count,
                                   pair_id, (double2*)tsd, np);
    });
}

void ref_mesh(void* dti, double* dbi, double* fx, double* fy, double* fz, double* mx, double* my, double* mz,
              double* pos, double* ep, double* vel, double* ev, double* force, double* moment, double* mass,
              double* tmax, double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
              double* dsph, unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend, void* cp,
              unsigned int np, unsigned int ntriangle)
{
    launch(np, [&] {
        particle_polygonObject_collision_kernel((device_triangle_info*)dti, dbi, fx, fy, fz, mx, my, mz,
                                                (double4*)pos, (double4*)ep, (double3*)vel, (double4*)ev,
                                                (double3*)force, (double3*)moment, mass, (double3*)tmax, rres,
                                                pair_count, pair_id, (double2*)tsd, (double4*)dsph,
                                                sorted_index, cstart, cend, (device_contact_property*)cp, np,
                                                ntriangle);
    });
}

void ref_rolling(double* tmax, double* rres, double* inertia, double* ep, double* ev, double* moment,
                 unsigned int np)
{
    launch(np, [&] {
        decide_rolling_friction_moment_kernel((double3*)tmax, rres, inertia, (double4*)ep, (double4*)ev,
                                              (double3*)moment, np);
    });
}

void ref_update_mesh(double* dbi, double* vList, double* sphere, double* dlocal, void* dpi,
                     unsigned int ntriangle)
{
    launch(ntriangle, [&] {
        updateMeshObjectData_kernel(dbi, vList, (double4*)sphere, (double3*)dlocal, (device_triangle_info*)dpi,
                                    ntriangle);
    });
}

void ref_clusters_p2p(double* pos, double* cpos, double* ep, double* vel, double* ev, double* force,
                      double* moment, double* mass, double* tmax, double* rres, unsigned int* pair_count,
                      unsigned int* pair_id, double* tsd, unsigned int* sorted_index, unsigned int* cstart,
                      unsigned int* cend, void* cp, void* xci, unsigned int np)
{
    launch(np, [&] {
        calcluate_clusters_contact_kernel((double4*)pos, (double4*)cpos, (double4*)ep, (double3*)vel,
                                          (double4*)ev, (double3*)force, (double3*)moment, mass, (double3*)tmax,
                                          rres, pair_count, pair_id, (double2*)tsd, sorted_index, cstart, cend,
                                          (device_contact_property*)cp, (xClusterInformation*)xci, np);
    });
}

void ref_cluster_plane(void* plane, double* dbi, double* fx, double* fy, double* fz, double* mx, double* my,
                       double* mz, double* pos, double* cpos, double* ep, double* vel, double* ev, double* force,
                       double* moment, void* cp, double* mass, double* tmax, double* rres,
                       unsigned int* pair_count, unsigned int* pair_id, double* tsd, void* xci, unsigned int np)
{
    launch(np, [&] {
        cluster_plane_contact_kernel((device_plane_info*)plane, dbi, fx, fy, fz, mx, my, mz, (double4*)pos,
                                     (double4*)cpos, (double4*)ep, (double3*)vel, (double4*)ev, (double3*)force,
                                     (double3*)moment, (device_contact_property*)cp, mass, (double3*)tmax, rres,
                                     pair_count, pair_id, (double2*)tsd, (xClusterInformation*)xci, np);
    });
}

void ref_cluster_mesh(void* dti, double* dbi, double* fx, double* fy, double* fz, double* mx, double* my,
                      double* mz, double* pos, double* cpos, double* ep, double* vel, double* ev, double* force,
                      double* moment, void* cp, double* mass, double* tmax, double* rres,
                      unsigned int* pair_count, unsigned int* pair_id, double* tsd, unsigned int* sorted_index,
                      unsigned int* cstart, unsigned int* cend, void* xci, unsigned int np, unsigned int ntriangle)
{
    launch(np, [&] {
        cluster_meshes_contact_kernel((device_triangle_info*)dti, dbi, fx, fy, fz, mx, my, mz, (double4*)pos,
                                      (double4*)cpos, (double4*)ep, (double3*)vel, (double4*)ev, (double3*)force,
                                      (double3*)moment, (device_contact_property*)cp, mass, (double3*)tmax, rres,
                                      pair_count, pair_id, (double2*)tsd, sorted_index, cstart, cend,
                                      (xClusterInformation*)xci, np, ntriangle);
    });
}

void ref_cylinder(void* cyl, double* bi, double* fx, double* fy, double* fz, double* mx, double* my, double* mz,
                  double* pos, double* ep, double* vel, double* ev, double* force, double* moment, void* cp,
                  double* mass, double* tmax, double* rres, unsigned int* pair_count, unsigned int* pair_id,
                  double* tsd, unsigned int np)
{
    launch(np, [&] {
        cylinder_contact_force_kernel((device_cylinder_info*)cyl, bi, fx, fy, fz, mx, my, mz, (double4*)pos,
                                      (double4*)ep, (double3*)vel, (double4*)ev, (double3*)force,
                                      (double3*)moment, (device_contact_property*)cp, mass, (double3*)tmax, rres,
                                      pair_count, pair_id, (double2*)tsd, np);
    });
}

void ref_cluster_cylinder(void* cyl, double* bi, double* fx, double* fy, double* fz, double* mx, double* my,
                          double* mz, double* pos, double* cpos, double* ep, double* vel, double* ev,
                          double* force, double* moment, void* xci, void* cp, double* mass, double* tmax,
                          double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                          unsigned int np)
{
    launch(np, [&] {
        cluster_cylinder_contact_force_kernel((device_cylinder_info*)cyl, bi, fx, fy, fz, mx, my, mz,
                                              (double4*)pos, (double4*)cpos, (double4*)ep, (double3*)vel,
                                              (double4*)ev, (double3*)force, (double3*)moment,
                                              (xClusterInformation*)xci, (device_contact_property*)cp, mass,
                                              (double3*)tmax, rres, pair_count, pair_id, (double2*)tsd, np);
    });
}

void ref_cluster_rolling(double* tmax, double* rres, double* inertia, double* ep, double* ev, double* moment,
                         void* xci, unsigned int np)
{
    launch(np, [&] {
        decide_cluster_rolling_friction_moment_kernel((double3*)tmax, rres, (double3*)inertia, (double4*)ep,
                                                      (double4*)ev, (double3*)moment,
                                                      (xClusterInformation*)xci, np);
    });
}

void ref_vv_cluster_position(double* pos, double* cpos, double* ep, double* rloc, double* vel, double* acc,
                             double* ev, double* ea, void* xci, unsigned int ns)
{
    launch(ns, [&] {
        vv_update_position_cluster_kernel((double4*)pos, (double4*)cpos, (double4*)ep, (double3*)rloc,
                                          (double3*)vel, (double3*)acc, (double4*)ev, (double4*)ea,
                                          (xClusterInformation*)xci, ns);
    });
}

void ref_vv_cluster_velocity(double* cpos, double* ep, double* vel, double* acc, double* ev, double* ea,
                             double* force, double* moment, double* rloc, double* mass, double* iner,
                             void* xci, unsigned int ns)
{
    launch(ns, [&] {
        vv_update_cluster_velocity_kernel((double4*)cpos, (double4*)ep, (double3*)vel, (double3*)acc,
                                          (double4*)ev, (double4*)ea, (double3*)force, (double3*)moment,
                                          (double3*)rloc, mass, (double3*)iner, (xClusterInformation*)xci, ns);
    });
}

} /* extern "C" */
