// xdem_api.cu -- the C-ABI of include/xdem_c.h.
//
// Launcher surface: the names and argument order of the reference's
// XDYNAMICS_API launchers (include/xdynamics_parallel/xParallelDEM_decl.cuh:
// 280-424, source/xdynamics_parallel/xParallelDEM_def.cu:16-536), returning a
// status instead of void.  Scratch the launchers need (sort buffers, block
// partial sums, material constants, the status word) is owned by the library,
// one set per device, grown on demand.
//
// Scene surface: xdem_sim owns the particle state and runs the step in the
// order of xIntegratorVV::OneStepSimulation (source/xdynamics_simulation/
// xIntegratorVV.cpp:26-63), contact dispatch as xContactManager::
// deviceCollision (source/xdynamics_manager/xContactManager.cpp:458-472).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <new>
#include <vector>

#include "xdem_device.cuh"
#include "xdem_kernels.h"

using namespace xdem;

namespace {

constexpr int kMaxDevices = 64;

struct DevCtx {
    // set (release) once every pointer below is allocated; read (acquire)
    // outside the lock by the fast path of ctx()
    std::atomic<bool> init{false};
    unsigned int* status = nullptr;
    double* red_tmp = nullptr;     // 1024 partials + 1 result
    mat_pair* mp = nullptr;        // scratch material constants
    unsigned int* sort_k1 = nullptr;
    unsigned int* sort_v1 = nullptr;
    unsigned int* sort_hist = nullptr;
    size_t sort_cap = 0, sort_vcap = 0, hist_cap = 0;
    double* bsums = nullptr;       // block partials of the last plane/mesh launch
    size_t bsums_cap = 0;
    unsigned int last_blocks = 0;
    double* wrench = nullptr;      // [6]
    double* own_bf = nullptr;      // 6 x cap internal body-force partials
    size_t own_bf_cap = 0;
};

DevCtx g_dev[kMaxDevices];
std::mutex g_mu;
device_dem_parameters g_params;
bool g_params_set = false;
double* g_bf[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
int g_vel_compat = 0;
int g_roll_per_sphere = 0;
thread_local cudaStream_t t_stream = 0;
thread_local int t_status = XDEM_OK;

int set_status(int s)
{
    t_status = s;
    return s;
}

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return XDEM_OK;
    fprintf(stderr, "xdem: CUDA error %s\n", cudaGetErrorString(e));
    return XDEM_ERR_CUDA;
}

template <class T>
cudaError_t grow(T*& p, size_t& cap, size_t want)
{
    if (want <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t n = std::max<size_t>(want, 1);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), n * sizeof(T));
    if (e == cudaSuccess) cap = n;
    return e;
}

// Returns the context of the current device, allocating its fixed scratch on
// first use.
DevCtx* ctx(int* err)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        *err = XDEM_ERR_CUDA;
        return nullptr;
    }
    DevCtx& c = g_dev[dev];
    if (!c.init.load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!c.init.load(std::memory_order_relaxed)) {
            e = cudaMalloc(&c.status, sizeof(unsigned int));
            if (e == cudaSuccess) e = cudaMemset(c.status, 0, sizeof(unsigned int));
            if (e == cudaSuccess) e = cudaMalloc(&c.red_tmp, 1025 * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&c.mp), 4 * mat_pair_size());
            if (e == cudaSuccess) e = cudaMalloc(&c.wrench, 6 * sizeof(double));
            if (e == cudaSuccess) e = cudaMemset(c.wrench, 0, 6 * sizeof(double));
            if (e != cudaSuccess) {
                *err = XDEM_ERR_ALLOC;
                return nullptr;
            }
            c.init.store(true, std::memory_order_release);
        }
    }
    return &c;
}

int need_params()
{
    return g_params_set ? XDEM_OK : XDEM_ERR_NOT_SET;
}

int bits_for_cells(unsigned long long ncell)
{
    int b = 0;
    while (b < 32 && (1ull << b) < ncell) ++b;
    return b == 0 ? 1 : b;
}

// Body partial arrays used by the plane/mesh launchers: the registered ones,
// else the library's own (grown to np).
int body_partials(DevCtx* c, unsigned int np, BodyPartials& bp)
{
    bool reg = true;
    for (int i = 0; i < 6; ++i) reg = reg && g_bf[i];
    if (reg) {
        bp.fx = g_bf[0]; bp.fy = g_bf[1]; bp.fz = g_bf[2];
        bp.mx = g_bf[3]; bp.my = g_bf[4]; bp.mz = g_bf[5];
    } else {
        if (grow(c->own_bf, c->own_bf_cap, (size_t)np * 6) != cudaSuccess) return XDEM_ERR_ALLOC;
        const size_t s = c->own_bf_cap / 6;
        bp.fx = c->own_bf; bp.fy = c->own_bf + s; bp.fz = c->own_bf + 2 * s;
        bp.mx = c->own_bf + 3 * s; bp.my = c->own_bf + 4 * s; bp.mz = c->own_bf + 5 * s;
    }
    const unsigned int nb = blocks_for(np);
    if (grow(c->bsums, c->bsums_cap, (size_t)std::max(nb, 1u) * 6) != cudaSuccess) return XDEM_ERR_ALLOC;
    bp.block_sums = c->bsums;
    c->last_blocks = nb;
    return XDEM_OK;
}

int finish_wrench(DevCtx* c)
{
    if (c->last_blocks == 0) return cuda_status(cudaMemsetAsync(c->wrench, 0, 6 * sizeof(double), t_stream));
    return cuda_status(launch_sum_block_partials(c->bsums, c->last_blocks, c->wrench, t_stream));
}

}  // namespace

namespace xdem {
cudaStream_t launcher_stream() { return t_stream; }
int launcher_set_status(int s) { return set_status(s); }
}  // namespace xdem

// ============================================================================
// Library control
// ============================================================================
extern "C" {

XDEM_API const char* xdem_version(void)
{
    return "xdem-gb300 1.0 (sm_103a, FP64 + mixed)";
}

XDEM_API int xdem_set_stream(void* stream)
{
    t_stream = reinterpret_cast<cudaStream_t>(stream);
    return set_status(XDEM_OK);
}

XDEM_API int xdem_last_status(void) { return t_status; }

XDEM_API int xdem_take_device_status(void)
{
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    unsigned int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->status, sizeof(h), cudaMemcpyDeviceToHost, t_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t_stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status, 0, sizeof(unsigned int), t_stream);
    if (e != cudaSuccess) return set_status(XDEM_ERR_CUDA);
    set_status(XDEM_OK);
    return (int)h;
}

XDEM_API int xdem_set_body_force_buffers(double* fx, double* fy, double* fz, double* mx, double* my, double* mz)
{
    g_bf[0] = fx; g_bf[1] = fy; g_bf[2] = fz;
    g_bf[3] = mx; g_bf[4] = my; g_bf[5] = mz;
    return set_status(XDEM_OK);
}

XDEM_API int xdem_get_body_force_buffers(double** out6)
{
    if (!out6) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    bool reg = true;
    for (int i = 0; i < 6; ++i) reg = reg && g_bf[i];
    if (reg) {
        for (int i = 0; i < 6; ++i) out6[i] = g_bf[i];
    } else {
        const size_t s = c->own_bf_cap / 6;
        for (int i = 0; i < 6; ++i) out6[i] = c->own_bf ? c->own_bf + i * s : nullptr;
    }
    return set_status(XDEM_OK);
}

XDEM_API int xdem_last_body_wrench(double out6[6])
{
    if (!out6) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    cudaError_t e = cudaMemcpyAsync(out6, c->wrench, 6 * sizeof(double), cudaMemcpyDeviceToHost, t_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t_stream);
    return set_status(cuda_status(e));
}

XDEM_API int xdem_set_velocity_compat(int reproduce_reference_gpu)
{
    g_vel_compat = reproduce_reference_gpu ? 1 : 0;
    return set_status(XDEM_OK);
}

XDEM_API int xdem_set_rolling_inertia(int per_sphere)
{
    g_roll_per_sphere = per_sphere ? 1 : 0;
    return set_status(XDEM_OK);
}

// ============================================================================
// Launcher surface
// ============================================================================
XDEM_API int setDEMSymbolicParameter(device_dem_parameters* h_paras)
{
    if (!h_paras) return set_status(XDEM_ERR_ARG);
    const xdem_uint3 g = h_paras->grid_size;
    auto pow2 = [](unsigned int v) { return v && !(v & (v - 1)); };
    if (!pow2(g.x) || !pow2(g.y) || !pow2(g.z) || !(h_paras->cell_size > 0)) return set_status(XDEM_ERR_ARG);
    g_params = *h_paras;
    g_params_set = true;
    return set_status(XDEM_OK);
}

XDEM_API int vv_update_position(double* pos, double* ep, double* vel, double* ev, double* acc, double* ea,
                                unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    return set_status(cuda_status(launch_vv_position(g_params, pos, ep, vel, ev, acc, ea, np, t_stream)));
}

XDEM_API int vv_update_velocity(double* vel, double* acc, double* ep, double* ev, double* ea, double* force,
                                double* moment, double* mass, double* iner, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    return set_status(cuda_status(launch_vv_velocity(g_params, vel, acc, ep, ev, ea, force, moment, mass, iner, np,
                                                     g_vel_compat, t_stream)));
}

XDEM_API int cu_calculateHashAndIndex(unsigned int* hash, unsigned int* index, double* pos, unsigned int sid,
                                      unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    return set_status(cuda_status(launch_hash(g_params, hash, index, pos, sid, np, c->status, t_stream)));
}

XDEM_API int cu_calculateHashAndIndexForPolygonSphere(unsigned int* hash, unsigned int* index, unsigned int sid,
                                                      unsigned int nsphere, double* sphere)
{
    return cu_calculateHashAndIndex(hash, index, sphere, sid, nsphere);
}

XDEM_API int cu_reorderDataAndFindCellStart(unsigned int* hash, unsigned int* index, unsigned int* cstart,
                                            unsigned int* cend, unsigned int* sorted_index, unsigned int np,
                                            unsigned int ncell)
{
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    if (!hash || !index || !cstart || !cend || !sorted_index) return set_status(XDEM_ERR_ARG);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (grow(c->sort_k1, c->sort_cap, np) != cudaSuccess) return set_status(XDEM_ERR_ALLOC);
        if (grow(c->sort_v1, c->sort_vcap, np) != cudaSuccess) return set_status(XDEM_ERR_ALLOC);
        if (grow(c->sort_hist, c->hist_cap, radix_hist_size(np)) != cudaSuccess) return set_status(XDEM_ERR_ALLOC);
    }
    cudaError_t e = launch_fill_u32(cstart, 0xffffffffu, ncell, t_stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(cend, 0, (size_t)ncell * sizeof(unsigned int), t_stream);
    unsigned int *sk = hash, *sv = index;
    if (e == cudaSuccess)
        e = radix_sort_pairs(hash, index, c->sort_k1, c->sort_v1, c->sort_hist, np, bits_for_cells(ncell), &sk, &sv,
                             t_stream);
    if (e == cudaSuccess && sk != hash) {
        e = cudaMemcpyAsync(hash, sk, (size_t)np * sizeof(unsigned int), cudaMemcpyDeviceToDevice, t_stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(index, sv, (size_t)np * sizeof(unsigned int), cudaMemcpyDeviceToDevice, t_stream);
    }
    if (e == cudaSuccess) e = launch_cell_bounds(hash, index, cstart, cend, sorted_index, np, t_stream);
    return set_status(cuda_status(e));
}

XDEM_API int cu_calculate_p2p(double* pos, double* ep, double* vel, double* omega, double* force, double* moment,
                              double* mass, double* tmax, double* rres, unsigned int* pair_count,
                              unsigned int* pair_id, double* tsd, unsigned int* sorted_index, unsigned int* cstart,
                              unsigned int* cend, device_contact_property* cp, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_p2p(g_params, pos, ep, vel, omega, force, moment, mass, tmax, rres, pair_count, pair_id, tsd,
                       sorted_index, cstart, cend, c->mp, np, c->status, t_stream);
    return set_status(cuda_status(e));
}

XDEM_API int cu_plane_contact_force(device_plane_info* plan, double* dbi, device_contact_property* cp, double* pos,
                                    double* ep, double* vel, double* omega, double* force, double* moment,
                                    double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                    unsigned int* pair_id, double* tsd, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_plane(g_params, plan, dbi, c->mp, bp, pos, ep, vel, omega, force, moment, mass, tmax, rres,
                         pair_count, pair_id, tsd, np, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_cylinder_contact_force(device_cylinder_info* cyl, double* bi, device_contact_property* cp,
                                       double* pos, double* ep, double* vel, double* omega, double* force,
                                       double* moment, double* mass, double* tmax, double* rres,
                                       unsigned int* pair_count, unsigned int* pair_id, double* tsd, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    if (!cyl || !bi || !cp) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_cylinder(g_params, cyl, bi, c->mp, bp, pos, nullptr, ep, vel, omega, force, moment, mass, tmax,
                            rres, pair_count, pair_id, tsd, nullptr, np, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_cluster_cylinder_contact(device_cylinder_info* cyl, double* bi, xClusterInformation* xci,
                                         device_contact_property* cp, double* pos, double* cpos, double* ep,
                                         double* vel, double* omega, double* force, double* moment, double* mass,
                                         double* tmax, double* rres, unsigned int* pair_count,
                                         unsigned int* pair_id, double* tsd, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    if (!cyl || !bi || !cp || !xci || !cpos) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_cylinder(g_params, cyl, bi, c->mp, bp, pos, cpos, ep, vel, omega, force, moment, mass, tmax,
                            rres, pair_count, pair_id, tsd, xci, np, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_particle_polygonObject_collision(device_triangle_info* dpi, double* dbi, double* pos, double* ep,
                                                 double* vel, double* omega, double* force, double* moment,
                                                 double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                                 unsigned int* pair_id, double* tsd, double* dsph,
                                                 unsigned int* sidx, unsigned int* cstart, unsigned int* cend,
                                                 device_contact_property* cp, unsigned int np,
                                                 unsigned int ntriangle)
{
    (void)dsph;
    if (int s = need_params()) return set_status(s);
    if (!dpi || ntriangle == 0) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    // first triangle entry = cte.np + dti[0].tid (impl:1970,1994), read by the kernel
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_mesh(g_params, dpi, g_params.np, 1, dbi, c->mp, bp, pos, nullptr, ep, vel, omega, force,
                        moment, mass, tmax, rres, pair_count, pair_id, tsd, sidx, cstart, cend, nullptr, np,
                        ntriangle, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_decide_rolling_friction_moment(double* tmax, double* rres, double* inertia, double* ep, double* ev,
                                               double* moment, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    return set_status(
        cuda_status(launch_rolling(g_params, tmax, rres, inertia, ep, ev, moment, np, t_stream, g_roll_per_sphere)));
}

XDEM_API double reduction(double* in, unsigned int np)
{
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) {
        set_status(err);
        return NAN;
    }
    double h = 0.0;
    cudaError_t e = launch_reduce_sum(in, np, c->red_tmp, c->red_tmp + 1024, t_stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&h, c->red_tmp + 1024, sizeof(double), cudaMemcpyDeviceToHost, t_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t_stream);
    set_status(cuda_status(e));
    return e == cudaSuccess ? h : NAN;
}

XDEM_API int cu_update_meshObjectData(double* vList, double* sph, double* dlocal, device_triangle_info* poly,
                                      double* dbi, unsigned int ntriangle)
{
    return set_status(cuda_status(launch_update_mesh(dbi, vList, sph, dlocal, poly, ntriangle, t_stream)));
}

XDEM_API int cu_clusters_contact(double* pos, double* cpos, double* ep, double* vel, double* omega, double* force,
                                 double* moment, double* mass, double* tmax, double* rres, unsigned int* pair_count,
                                 unsigned int* pair_id, double* tsd, unsigned int* sorted_index,
                                 unsigned int* cstart, unsigned int* cend, device_contact_property* cp,
                                 xClusterInformation* xci, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_clusters_p2p(g_params, pos, cpos, ep, vel, omega, force, moment, mass, tmax, rres, pair_count,
                                pair_id, tsd, sorted_index, cstart, cend, c->mp, xci, np, c->status, t_stream);
    return set_status(cuda_status(e));
}

XDEM_API int cu_cluster_plane_contact(device_plane_info* plan, double* dbi, device_contact_property* cp, double* pos,
                                      double* cpos, double* ep, double* vel, double* omega, double* force,
                                      double* moment, double* mass, double* tmax, double* rres,
                                      unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                      xClusterInformation* xci, unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 1, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_cluster_plane(g_params, plan, dbi, c->mp, bp, pos, cpos, ep, vel, omega, force, moment, mass,
                                 tmax, rres, pair_count, pair_id, tsd, xci, np, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_cluster_meshes_contact(device_triangle_info* dpi, double* dbi, double* pos, double* cpos,
                                       double* ep, double* vel, double* ev, double* force, double* moment,
                                       device_contact_property* cp, double* mass, double* tmax, double* rres,
                                       unsigned int* pair_count, unsigned int* pair_id, double* tsd,
                                       unsigned int* sorted_index, unsigned int* cstart, unsigned int* cend,
                                       xClusterInformation* xci, unsigned int np, unsigned int ntriangle)
{
    if (int s = need_params()) return set_status(s);
    if (!dpi || ntriangle == 0) return set_status(XDEM_ERR_ARG);
    int err = 0;
    DevCtx* c = ctx(&err);
    if (!c) return set_status(err);
    // first triangle entry = np + dti[0].id (impl:2180,2193), read by the kernel
    BodyPartials bp{};
    if (int s = body_partials(c, np, bp)) return set_status(s);
    cudaError_t e = launch_make_mat_pair(cp, g_params.contact_model, 0, c->mp, t_stream);
    if (e == cudaSuccess)
        e = launch_mesh(g_params, dpi, np, 2, dbi, c->mp, bp, pos, cpos, ep, vel, ev, force,
                        moment, mass, tmax, rres, pair_count, pair_id, tsd, sorted_index, cstart, cend, xci, np,
                        ntriangle, c->status, t_stream);
    if (e != cudaSuccess) return set_status(cuda_status(e));
    return set_status(finish_wrench(c));
}

XDEM_API int cu_decide_cluster_rolling_friction_moment(double* tmax, double* rres, double* inertia, double* ep,
                                                       double* ev, double* moment, xClusterInformation* xci,
                                                       unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    return set_status(
        cuda_status(launch_cluster_rolling(g_params, tmax, rres, inertia, ep, ev, moment, xci, np, t_stream)));
}

XDEM_API int vv_update_cluster_position(double* pos, double* cpos, double* ep, double* rloc, double* vel,
                                        double* acc, double* omega, double* alpha, xClusterInformation* xci,
                                        unsigned int np)
{
    if (int s = need_params()) return set_status(s);
    return set_status(cuda_status(
        launch_vv_cluster_position(g_params, pos, cpos, ep, rloc, vel, acc, omega, alpha, xci, np, t_stream)));
}

XDEM_API int vv_update_cluster_velocity(double* cpos, double* ep, double* vel, double* acc, double* omega,
                                        double* alpha, double* force, double* moment, double* rloc, double* mass,
                                        double* iner, xClusterInformation* xci, unsigned int np)
{
    (void)cpos; (void)rloc;
    if (int s = need_params()) return set_status(s);
    return set_status(cuda_status(launch_vv_cluster_velocity(g_params, vel, acc, ep, omega, alpha, force, moment,
                                                             mass, iner, xci, np, t_stream)));
}

}  // extern "C"
