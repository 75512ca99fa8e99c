// xdem_sim_impl.h -- the scene handle's state (struct xdem_sim), shared by
// the step (xdem_sim.cu) and the adjoint (xdem_adjoint.cu).  Not part of the
// public C-ABI: callers only see the opaque xdem_sim of include/xdem_c.h.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "xdem_device.cuh"
#include "xdem_fused.h"
#include "xdem_kernels.h"

using namespace xdem;

// Planes and meshes a handle can hold (batched scenes bring several planes
// each).
constexpr size_t kMaxBodies = 1u << 16;

struct SimBody {
    int kind;              // 0 plane, 1 mesh, 2 cylinder
    int index;             // plane index or mesh index
    double rec[15];
};

struct SimMesh {
    unsigned int ntri, first;  // triangles [first, first + ntri) of the global arrays
    int body;
    double c_local[3];         // centroid of the vertices (body frame)
    double reach;              // largest vertex distance from it
};

struct xdem_sim {
    xdem_sim_config cfg{};
    device_dem_parameters prm{};
    cudaStream_t st = 0;       // the stream steps run on (the handle's own or the caller's)
    cudaStream_t own_st = 0;   // created with the handle; the only stream destroy releases
    unsigned int np = 0, ns = 0, nco = 0, nrloc = 0;
    bool clusters = false;
    int rolling_per_sphere = 0;  // xdem_sim_set_rolling_inertia
    unsigned int status_host = 0;
    // state (reference layout)
    double *pos = nullptr, *cpos = nullptr, *vel = nullptr, *acc = nullptr, *ep = nullptr, *ev = nullptr,
           *ea = nullptr;
    double *force = nullptr, *moment = nullptr, *mass = nullptr, *inertia = nullptr, *tmax = nullptr,
           *rres = nullptr, *rloc = nullptr;
    xClusterInformation* xci = nullptr;
    std::vector<xClusterInformation> h_xci;  // host copy of the cluster table
    // grid
    unsigned int nentry = 0;
    size_t ncell = 0;
    unsigned int *k0 = nullptr, *v0 = nullptr, *k1 = nullptr, *v1 = nullptr, *hist = nullptr;
    unsigned int *cstart = nullptr, *cend = nullptr, *sorted_index = nullptr;
    unsigned int* skey = nullptr;  // sorted keys of the last step (k0 or k1)
    bool cells_clean = false;
    // contacts
    bool has_pp = false;
    device_contact_property pp_cp{};
    mat_pair* d_mp = nullptr;  // [nscene] particle pairs of each scene, then one per body
    unsigned int *pp_count = nullptr, *pp_id = nullptr;
    double* pp_tsd = nullptr;
    unsigned int *pl_count = nullptr, *pl_id = nullptr;
    double* pl_tsd = nullptr;
    unsigned int *ms_count = nullptr, *ms_id = nullptr;
    double* ms_tsd = nullptr;
    unsigned int *cy_count = nullptr, *cy_id = nullptr;  // cylinder pairs, MAX_P2CY_COUNT slots
    double* cy_tsd = nullptr;
    std::vector<SimBody> bodies;
    std::vector<device_plane_info> planes;
    std::vector<device_cylinder_info> cylinders;
    device_cylinder_info* d_cyl = nullptr;
    std::vector<device_contact_property> body_cp;
    std::vector<SimMesh> meshes;
    device_plane_info* d_planes = nullptr;
    double* d_body = nullptr;      // 15 per body
    unsigned int ntri_total = 0;
    std::vector<double> h_vlist, h_dlocal, h_sphere;  // host copies for setup
    std::vector<device_triangle_info> h_tri;
    device_triangle_info* d_tri = nullptr;
    double *d_vlist = nullptr, *d_dlocal = nullptr, *d_sphere = nullptr;
    double* bsums = nullptr;       // per body: nblocks * 6
    double* wrench = nullptr;      // per body: 6
    void* h_pin = nullptr;         // pinned staging of the batched body exchange
    size_t h_pin_cap = 0;
    cudaEvent_t pin_ev = nullptr;  // the last upload from h_pin
    unsigned int* d_status = nullptr;
    bool dirty_bodies = true;      // device body tables need upload
    bool dirty_alloc = true;       // contact tables need (re)allocation
    bool dirty_mesh_bs = true;     // the fused step's mesh bounding spheres need refreshing
    // fused path
    FusedState fs{};
    bool precision_mixed() const;
    // profiling: events around the contact kernel, a ring of kProfEvents
    // pairs read once at the end of xdem_sim_step
    static constexpr int kProfEvents = 64;
    bool profiling = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t pe0[kProfEvents] = {}, pe1[kProfEvents] = {};
    double prof_ms = 0.0;
    unsigned int prof_launches = 0, prof_contact_launches = 0, launches = 0;
    // CUDA graphs of one fused step, one per arrangement of the double-
    // buffered arrays (they alternate between two); key is the arrangement
    // the graph starts from
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        const void* key[8] = {};
        unsigned int launches = 0;
    };
    bool use_graph = false;
    bool capture_failed_noted = false;  // a failed step-graph capture is reported once
    StepGraph graphs[2];
    // batched scenes (nscene == 1: one scene)
    unsigned int nscene = 1;
    std::vector<unsigned int> scene_first, scene_plane_first;
    std::vector<device_contact_property> scene_cp;
    unsigned int* d_scene_of = nullptr;           // [np]
    unsigned int* d_scene_first = nullptr;        // [nscene + 1]
    unsigned int* d_scene_plane_first = nullptr;  // [nscene + 1]
    double* d_scene_energy = nullptr;             // [2 * nscene]
    // capacities of the body tables
    size_t plane_cap = 0, body_cap = 0, mp_cap = 0, cyl_cap = 0;
};

// XDEM_OK when every count of a host pair list (kind as xdem_sim_get_pairs)
// is within its slot capacity and every stored id names a particle, plane,
// triangle or cylinder of the handle; XDEM_ERR_ARG otherwise.
extern "C" int sim_check_pairs(const xdem_sim* s, int kind, const unsigned int* count,
                                const unsigned int* ids);
