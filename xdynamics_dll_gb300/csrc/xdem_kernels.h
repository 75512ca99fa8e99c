// xdem_kernels.h -- host-side launch wrappers of the DEM kernels.
//
// Every wrapper enqueues its kernel(s) on `st` and returns the launch error
// (cudaSuccess when the launch was accepted).  Pointers are device pointers
// in the reference layout (see include/xdem_c.h).  `status` is a device word
// the kernels OR their XDEM_ERR_* bits into.
#pragma once

#include <cuda_runtime.h>

#include "../../include/xdem_c.h"

namespace xdem {

struct mat_pair;

struct BodyPartials {
    double *fx, *fy, *fz, *mx, *my, *mz;  // per particle (np each), may be null
    double* block_sums;                   // [nblocks * 6] or null
};

constexpr int kThreads = 128;
inline unsigned int blocks_for(unsigned int n, unsigned int t = kThreads) { return (n + t - 1) / t; }

cudaError_t launch_vv_position(const device_dem_parameters& p, double* pos, double* ep, const double* vel,
                               const double* ev, const double* acc, const double* ea, unsigned int n,
                               cudaStream_t st);
cudaError_t launch_vv_velocity(const device_dem_parameters& p, double* vel, double* acc, const double* ep,
                               double* ev, double* ea, double* force, double* moment, const double* mass,
                               const double* iner, unsigned int n, int compat, cudaStream_t st);
cudaError_t launch_hash(const device_dem_parameters& p, unsigned int* hash, unsigned int* index,
                        const double* pos, unsigned int sid, unsigned int n, unsigned int* status, cudaStream_t st);
// Cell start/end of sorted keys into pre-cleared tables (impl:317-360) and
// sorted_index = index.
cudaError_t launch_cell_bounds(const unsigned int* skey, const unsigned int* sval, unsigned int* cstart,
                               unsigned int* cend, unsigned int* sorted_index, unsigned int n, cudaStream_t st);
// Marks the cells listed in `keys` empty again (0xffffffff / 0).  With a
// gate, only when *gate is nonzero (decided on the device).
cudaError_t launch_clear_cells(const unsigned int* keys, unsigned int n, unsigned int* cstart, unsigned int* cend,
                               cudaStream_t st, const unsigned int* gate = nullptr);
cudaError_t launch_fill_u32(unsigned int* a, unsigned int v, size_t n, cudaStream_t st);

cudaError_t launch_p2p(const device_dem_parameters& p, const double* pos, const double* ep, const double* vel,
                       const double* ev, double* force, double* moment, const double* mass, double* tmax,
                       double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                       const unsigned int* sorted_index, const unsigned int* cstart, const unsigned int* cend,
                       const mat_pair* mp, unsigned int n, unsigned int* status, cudaStream_t st);
cudaError_t launch_plane(const device_dem_parameters& p, const device_plane_info* plane, const double* dbi,
                         const mat_pair* mp, const BodyPartials& bp, const double* pos,
                         const double* ep, const double* vel, const double* ev, double* force, double* moment,
                         const double* mass, double* tmax, double* rres, unsigned int* pair_count,
                         unsigned int* pair_id, double* tsd, unsigned int n, unsigned int* status, cudaStream_t st);
// Particle-triangle contact.  The first sorted-entry index of this mesh's
// triangle spheres is lo_base (lo_field 0), lo_base + dti[0].tid
// (lo_field 1, sphere kernel) or lo_base + dti[0].id (lo_field 2, cluster
// kernel); ntri triangles.  cpos/xci non-null selects the cluster kernel.
cudaError_t launch_mesh(const device_dem_parameters& p, const device_triangle_info* dti, unsigned int lo_base,
                        int lo_field, const double* dbi, const mat_pair* mp, const BodyPartials& bp,
                        const double* pos, const double* cpos, const double* ep, const double* vel,
                        const double* ev, double* force, double* moment, const double* mass, double* tmax,
                        double* rres, unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                        const unsigned int* sorted_index, const unsigned int* cstart, const unsigned int* cend,
                        const xClusterInformation* xci, unsigned int n, unsigned int ntri, unsigned int* status,
                        cudaStream_t st);
cudaError_t launch_rolling(const device_dem_parameters& p, double* tmax, double* rres, const double* inertia,
                           const double* ep, const double* ev, double* moment, unsigned int n, cudaStream_t st,
                           int per_sphere = 0);
cudaError_t launch_update_mesh(const double* dbi, const double* vlist, double* sphere, const double* dlocal,
                               device_triangle_info* dpi, unsigned int ntri, cudaStream_t st);
cudaError_t launch_clusters_p2p(const device_dem_parameters& p, const double* pos, const double* cpos,
                                const double* ep, const double* vel, const double* ev, double* force,
                                double* moment, const double* mass, double* tmax, double* rres,
                                unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                const unsigned int* sorted_index, const unsigned int* cstart,
                                const unsigned int* cend, const mat_pair* mp,
                                const xClusterInformation* xci, unsigned int n, unsigned int* status,
                                cudaStream_t st);
// impl:1324-1601; cpos != null: cluster members (xci)
cudaError_t launch_cylinder(const device_dem_parameters& p, const device_cylinder_info* cyl, const double* bi,
                            const mat_pair* mp, const BodyPartials& bp, const double* pos, const double* cpos,
                            const double* ep, const double* vel, const double* ev, double* force, double* moment,
                            const double* mass, double* tmax, double* rres, unsigned int* pair_count,
                            unsigned int* pair_id, double* tsd, const xClusterInformation* xci, unsigned int n,
                            unsigned int* status, cudaStream_t st);
cudaError_t launch_cluster_plane(const device_dem_parameters& p, const device_plane_info* plane, const double* dbi,
                                 const mat_pair* mp, const BodyPartials& bp, const double* pos,
                                 const double* cpos, const double* ep, const double* vel, const double* ev,
                                 double* force, double* moment, const double* mass, double* tmax, double* rres,
                                 unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                 const xClusterInformation* xci, unsigned int n, unsigned int* status,
                                 cudaStream_t st);
cudaError_t launch_cluster_rolling(const device_dem_parameters& p, double* tmax, double* rres, const double* inertia,
                                   const double* ep, const double* ev, double* moment,
                                   const xClusterInformation* xci, unsigned int n, cudaStream_t st);
cudaError_t launch_vv_cluster_position(const device_dem_parameters& p, double* pos, double* cpos, double* ep,
                                       const double* rloc, const double* vel, const double* acc, const double* ev,
                                       const double* ea, const xClusterInformation* xci, unsigned int ns,
                                       cudaStream_t st);
cudaError_t launch_vv_cluster_velocity(const device_dem_parameters& p, double* vel, double* acc, const double* ep,
                                       double* ev, double* ea, double* force, double* moment, const double* mass,
                                       const double* iner, const xClusterInformation* xci, unsigned int ns,
                                       cudaStream_t st);
// Material-pair constants of a device contact property into *out (device),
// with the cluster-plane friction swap when swap_fric != 0.
cudaError_t launch_make_mat_pair(const device_contact_property* cp, int model, int swap_fric, mat_pair* out,
                                 cudaStream_t st);
size_t mat_pair_size();
// Sum of n doubles into *out (device), two passes through `tmp`
// (>= reduce_tmp_size(n) doubles).
size_t reduce_tmp_size(unsigned int n);
cudaError_t launch_reduce_sum(const double* in, unsigned int n, double* tmp, double* out, cudaStream_t st);
// Sum of nblocks x 6 block partials into out[6] (device).
cudaError_t launch_sum_block_partials(const double* partials, unsigned int nblocks, double* out6, cudaStream_t st);

// Stream of the launcher surface on this host thread (xdem_set_stream) and
// the per-thread status of its last call.
cudaStream_t launcher_stream();
int launcher_set_status(int s);

// ---------------------------------------------------------------- radix sort
// Stable LSD sort of (keys, vals) by the low `bits` bits of the keys.  Uses
// ping-pong buffers k1/v1 (n each) and `hist` (radix_hist_size(n) uints).
// The sorted result ends in the buffers returned through out_k/out_v.  With
// a gate the kernels do nothing unless *gate is nonzero (a device-side skip
// that keeps the launch sequence fixed, for CUDA graphs).
size_t radix_hist_size(unsigned int n);
cudaError_t radix_sort_pairs(unsigned int* k0, unsigned int* v0, unsigned int* k1, unsigned int* v1,
                             unsigned int* hist, unsigned int n, int bits, unsigned int** out_k,
                             unsigned int** out_v, cudaStream_t st, const unsigned int* gate = nullptr);

}  // namespace xdem
