// xdem_fused.h -- host interface of the fused, sorted-order DEM step.
//
// One step = [hash of mesh spheres] -> clear last step's cells -> radix sort
// of (cell, id) -> reorder (cell ranges + a cell-sorted snapshot of position,
// velocity, spin and mass) -> one contact kernel per sorted particle that
// does particle-particle, plane and mesh contact, rolling resistance, the
// velocity update, the next position update and the next hash -> per-body
// wrench sums.  The contact kernel reads only the snapshot for neighbours, so
// it updates the particle's own state in place without racing other threads.
//
// Position and Euler parameters are double-buffered: between steps the
// handle's buffers hold the committed state and the alternate buffers the
// already computed positions of the next step.  Particle-particle pair lists
// are double-buffered (old list read, new list written).
//
// FP64 form: the snapshot holds FP64 position / velocity / spin (exact
// classification) plus an FP32 copy of the position for a conservative
// prefilter.  Mixed form: the snapshot is FP32 only -- each sphere's position
// as an offset from the corner of its own cell plus the cell's integer
// coordinates, so the relative position of two neighbours is formed in FP32
// to about 1e-9 m without FP64 arithmetic in the neighbour loop; the state
// stays FP64 and only receives FP32 increments (xdem_fused_mixed.cu).
//
// Batched scenes: a handle may hold several independent scenes (particles
// tagged by scene, each scene with its own particle-particle material and
// its own range of planes); contacts between particles of different scenes
// are not formed.  Batched handles produce no body wrenches.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/xdem_c.h"

namespace xdem {

struct mat_pair;
constexpr unsigned int kMaxFusedMeshes = 8;
// Cluster types (xClusterInformation entries) the mixed cluster step holds.
constexpr unsigned int kMaxClusterTypes = 8;

// Clusters of the mixed step: ns rigid clusters of neach member spheres
// each, the members of cluster c at c*neach .. c*neach + neach - 1 (one
// member count for every type, so that id / neach is the cluster of any
// sphere as impl:485-611 computes it).  Clusters of type t start at
// first[t] and place their members at rloc[(t*neach + j)*3] in the body
// frame.  ns == 0: no clusters.
struct ClusterTab {
    unsigned int ns = 0, neach = 0, ntype = 0;
    unsigned int first[kMaxClusterTypes + 1] = {};
};
__host__ __device__ inline unsigned int cluster_type(const ClusterTab& t, unsigned int cid)
{
    unsigned int k = 0;
    for (unsigned int i = 1; i < t.ntype; ++i)
        if (cid >= t.first[i]) k = i;
    return k;
}
constexpr unsigned int kBboxBlocks = 1024;
constexpr int kPlaneF = 16;  // floats per plane in the prefilter table

// FP32 view of a plane for the conservative "is this sphere near the plane"
// test: corner xw (relative to the grid origin), unit edges u1, u2, unit
// normal, edge lengths.  Layout: xw[3], u1[3], u2[3], un[3], l1, l2, pad[2].
struct PlaneF { float v[kPlaneF]; };

// Float-pair view of a plane for the mixed form's contact geometry: corner
// xw, the frame rows u1, u2, unit normal, and the edge lengths, each as
// hi + lo floats.  rect = 1 when the plane is an orthonormal rectangle
// (w2 = xw + l1 u1, w4 = xw + l2 u2, w3 = w2 + l2 u2, normal = u1 x u2 of
// unit length), which the local-coordinate contact test needs; other planes
// use the FP64 test.  coh = 1 when the plane's contact has cohesion.
struct PlaneDF {
    float xw_hi[3], xw_lo[3];
    float u_hi[9], u_lo[9];
    float l1_hi, l1_lo, l2_hi, l2_lo;
    int rect, coh, pad[2];
};

// Material constants of one contact pair in FP32 (the mixed form's copy of
// mat_pair): equivalent Young's modulus, 8 G*, damping ratio beta, the
// tangential damping factor, stiffness ratio, friction, rolling friction,
// and whether cohesion is on.
struct MatF {
    float Eeq, Seq8, beta, vs1, sratio, fric, rfric;
    int coh;
};

// Block shapes of the mixed contact stage, chosen by the autotuner
// (xdem_sim_autotune): threads per block of the pair kernel and of the body
// kernel (64, 128 or 256), the pair kernel's candidate-stage depth (8 or 16
// entries a thread) and the resident threads per SM each kernel is compiled
// for (pairs 768 or 1024, bodies 512, 768 or 1024: the register budget).
// Results do not depend on them.
// skin_div selects the pair search: 0 walks the 27-cell stencil every step;
// d > 0 keeps a candidate list per sphere with a skin of (cell size) / d,
// rebuilt by a stencil walk only when some sphere has moved more than half
// the skin since the last build.
struct MixedTune {
    unsigned int nt_pairs = 128, stage = 16, nt_bodies = 128, occ_pairs = 768, occ_bodies = 512, skin_div = 0;
};
// Record k of sphere i: rec[4 i + k] (kRecA, kRecL, kRecB, kRecC).
enum { kRecA = 0, kRecL = 1, kRecB = 2, kRecC = 3 };
__device__ __forceinline__ unsigned int rec_cell(float4 C) { return __float_as_uint(C.w); }

// Cell ranges of the sorted keys (impl:317-360) for sorted entry s with key k.
__device__ __forceinline__ void cell_bounds(const unsigned int* sk, unsigned int s, unsigned int n,
                                            unsigned int* cstart, unsigned int* cend, unsigned int k)
{
    const unsigned int prev = s ? sk[s - 1] : 0u;
    if (s == 0 || k != prev) {
        cstart[k] = s;
        if (s > 0) cend[prev] = s;
    }
    if (s == n - 1) cend[k] = s + 1;
}

// Mixed form, sorted entry s < n: its cell range bounds, and its FP32
// records permuted into sorted order (entries >= np, mesh spheres, get an
// empty record).
__device__ __forceinline__ void reorder_mixed_entry(unsigned int s, const unsigned int* sk, const unsigned int* sv,
                                                    unsigned int n, unsigned int np, unsigned int* cstart,
                                                    unsigned int* cend, unsigned int* sorted_index,
                                                    unsigned int* skey, const float4* rec, float4* mA, float4* mL,
                                                    float4* mB, float4* mC, uint2* mIT)
{
    const unsigned int k = sk[s];
    cell_bounds(sk, s, n, cstart, cend, k);
    const unsigned int oid = sv[s];
    sorted_index[s] = oid;
    skey[s] = k;
    if (oid < np) {
        const float4* r = rec + 4 * (size_t)oid;
        mA[s] = r[kRecA];
        mL[s] = r[kRecL];
        mB[s] = r[kRecB];
        const float4 C = r[kRecC];
        mC[s] = C;
        mIT[s] = make_uint2(oid, rec_cell(C));
    } else {
        mA[s] = make_float4(0.f, 0.f, 0.f, -1.f);
        mIT[s] = make_uint2(oid, 0xffffffffu);
    }
}

// Candidates a sphere's list holds; a sphere with more walks the stencil.
constexpr unsigned int kListCap = 24;
// Blocks per body of the wrench reduction.
constexpr unsigned int kWrenchChunks = 32;
// Words of the candidate-list flags: rebuild this step, a sphere moved more
// than half the skin (this step), rebuilds counted, a list overflowed at the
// last build, the cell sort is needed this step (rebuild or overflow).
enum { kVlRebuild = 0, kVlMoved = 1, kVlCount = 2, kVlOverflow = 3, kVlSort = 4, kVlWords = 5 };

struct FusedState {
    MixedTune tune;
    bool mixed = false;
    bool primed = false;       // next positions + keys hold the next step's input
    bool have_prev = false;    // skey_prev lists the occupied cells of the last step
    unsigned int np = 0, nentry = 0;
    double* pos_alt = nullptr;  // [np*4] other position buffer
    double* cpos_alt = nullptr; // [ns*4] other cluster-centre buffer (clusters)
    double* ep_alt = nullptr;   // [np*4] other Euler-parameter buffer
    // FP64 snapshot (sorted order)
    double* snap_pos = nullptr; // [nentry*4] x, y, z, r
    double* snap_vel = nullptr; // [nentry*4] vx, vy, vz, mass
    double* snap_om = nullptr;  // [nentry*4] wx, wy, wz, 0
    float* snap_f = nullptr;    // [nentry*4] x-o, y-o, z-o, r (FP32 prefilter; w < 0: no filter)
    // mixed snapshot (sorted order) and its per-sphere source (original order)
    float* mA = nullptr;        // [nentry*4] offset from own cell corner, r
    float* mL = nullptr;        // [nentry*4] low parts of mA (float pairs)
    float* mB = nullptr;        // [nentry*4] vx, vy, vz, mass
    float* mC = nullptr;        // [nentry*4] wx, wy, wz, 0
    unsigned int* mIT = nullptr; // [nentry*2] (original id, packed unwrapped cell)
    // next-step records written by the contact kernel, one 64-byte record
    // per sphere in original order: A (cell offsets, radius), L (their low
    // parts), B (velocity, mass), C (spin, packed cell bits in w) -- a
    // neighbour's record is two sectors
    float4* rec = nullptr;      // [np*4]
    // FP32 copies of a mixed sphere handle's acceleration, Euler-parameter
    // acceleration, and principal inertia + mass (np entries each): the body
    // kernel reads and writes these instead of the FP64 arrays, which are
    // brought up to date only when something reads them.  f32_ready: the
    // copies hold the state; f64_stale: the FP64 acc and ea arrays lag them.
    float4* accf = nullptr;
    float4* eaf = nullptr;
    float4* jm = nullptr;
    bool f32_ready = false, f64_stale = false;
    float* fA = nullptr;        // [np*4] particle-particle force, rolling resistance (original order)
    float* fB = nullptr;        // [np*4] particle-particle moment
    float* fC = nullptr;        // [np*4] rolling: sum of contact moments
    // candidate lists (skin_div > 0): ids ascending, count (> kListCap:
    // overflowed, walk), FP32 centre at the build, rebuild flags [in, out]
    unsigned int* vl_ids = nullptr;  // [np * kListCap]
    unsigned int* vl_cnt = nullptr;  // [np]
    float* vl_xb = nullptr;          // [np*4]
    unsigned int* vl_flag = nullptr; // [kVlWords], indices kVl* below
    bool any_coh = false;            // cohesion in a particle-pair material (no lists)
    // persistent batched step (xdem_sim_set_persistent): on, the grid
    // barriers' time limit, their two words (arrivals, generation), and the
    // co-resident grid of each register budget (768 / 1024 threads per SM)
    bool persist = false;
    unsigned long long persist_limit_ns = 1000000000ull;
    unsigned int* d_bar = nullptr;   // [2]
    unsigned int persist_grid[2] = {0u, 0u};
    // bounding sphere of each mesh (centre relative to the grid origin,
    // radius): a sphere that cannot reach it skips the triangle search
    cudaStream_t side_st = nullptr;  // captures the conditional sort section of a step graph
    float4* d_mesh_bs = nullptr;     // [kMaxFusedMeshes]
    float4 h_mesh_bs[kMaxFusedMeshes] = {};
    // body wrench reduction: per-chunk sums and per-body finish counters
    double* wsum = nullptr;          // [wsum_cap * kWrenchChunks * 6]
    unsigned int* wcnt = nullptr;    // [wsum_cap]
    unsigned int wsum_cap = 0;
    MatF* d_mpf = nullptr;      // FP32 material table (scenes' particle pairs, then bodies)
    size_t mpf_cap = 0;
    unsigned int* pp_count2 = nullptr;
    unsigned int* pp_id2 = nullptr;
    double* pp_tsd2 = nullptr;
    unsigned int* skey_prev = nullptr;  // [nentry] sorted keys of the last step
    double* d_energy = nullptr;
    double* d_bbox = nullptr;   // [kBboxBlocks * 6] block min/max of positions
    PlaneF* d_planef = nullptr; // [plane_cap]
    PlaneDF* d_planedf = nullptr; // [plane_cap]
    size_t plane_cap = 0;
    std::vector<PlaneF> h_planef;     // host copies (sources of the uploads)
    std::vector<PlaneDF> h_planedf;
    double origin[3] = {0.0, 0.0, 0.0};
    double frame_far2 = 0.0;    // squared radius (from the grid origin) of the FP32 frame
    float frame_margin = 0.f;   // prefilter slack for FP32 rounding
    const device_plane_info* planes = nullptr;
    unsigned int nplane = 0;
    const double* body = nullptr;
    const mat_pair* mp = nullptr;
};

struct FusedArgs {
    device_dem_parameters prm;
    unsigned int np, nentry;
    size_t ncell;
    int sort_bits;
    int vel_compat;
    int rolling_per_sphere;    // rolling resistance reads inertia[3 i] (else the flat entry i)
    // state: pos/ep are swapped with the alternate buffers by fused_step
    double** pos;
    double** ep;
    double *vel, *acc, *ev, *ea, *mass, *inertia, *tmax, *rres;
    unsigned int *k0, *v0, *k1, *v1, *hist, *cstart, *cend, *sorted_index;
    bool has_pp;
    unsigned int** pp_count;
    unsigned int** pp_id;
    double** pp_tsd;
    unsigned int *pl_count, *pl_id;
    double* pl_tsd;
    unsigned int nplane, nbody, nmesh;
    unsigned int mesh_first[kMaxFusedMeshes], mesh_ntri[kMaxFusedMeshes];
    int mesh_body[kMaxFusedMeshes];
    const device_triangle_info* tri;
    const double* tri_sphere;
    unsigned int *ms_count, *ms_id;
    double* ms_tsd;
    // cylinders (mixed sphere scenes): bodies nplane .. nplane + ncyl - 1
    unsigned int ncyl = 0;
    const device_cylinder_info* cyl = nullptr;
    unsigned int *cy_count = nullptr, *cy_id = nullptr;
    double* cy_tsd = nullptr;
    const double* body;
    const mat_pair* mp;
    double *bsums, *wrench;
    unsigned int* status;
    bool rolling;              // any contact property with rolling friction
    // batched scenes (nscene == 1: a single scene, scene_of unused)
    unsigned int nscene = 1;
    const unsigned int* scene_of = nullptr;          // [np]
    const unsigned int* scene_plane_first = nullptr; // [nscene + 1]
    // clusters (mixed form only); ns_state: length of the per-body state
    // arrays (vel, ep, mass, ...), np for sphere scenes
    unsigned int ns_state = 0;
    ClusterTab cl;
    double** cpos = nullptr;    // [ns*4]: swapped with the alternate buffer
    const double* rloc = nullptr;
};

int fused_alloc(FusedState& fs, unsigned int np, unsigned int nentry, bool mixed, cudaStream_t st,
                unsigned int ns = 0);
void fused_free(FusedState& fs);
void fused_invalidate(FusedState& fs);
// The handle's state arrays were written from outside the step (state
// upload, restore): the next step starts over and refreshes the FP32 copies.
void fused_state_written(FusedState& fs);
// Brings the FP64 acc and ea arrays up to date from the FP32 copies before
// something reads them (np sphere entries).
int fused_sync_fp64(FusedState& fs, double* acc, double* ea, cudaStream_t st);
// host_mp holds nscene particle-pair entries followed by one per body.
int fused_set_bodies(FusedState& fs, const device_plane_info* planes, unsigned int nplane, const double* body,
                     const mat_pair* mp, const device_plane_info* host_planes, const mat_pair* host_mp,
                     unsigned int nmp, unsigned int nscene, const double origin[3], cudaStream_t st);
// New frame of plane k (its body moved): refreshes the plane tables on the
// stream; the host copy it uploads from stays owned by the state.
int fused_update_plane(FusedState& fs, unsigned int k, const device_plane_info& host_plane, bool coh,
                       cudaStream_t st);
// Bounding sphere of mesh m (centre relative to the grid origin, radius;
// a radius of 1e18 searches every sphere): refreshed on the stream.
// Host copies of plane k's FP32 and float-pair tables (fs.h_planef,
// fs.h_planedf) from its frame, without the upload; false when the tables
// do not exist yet.
bool fused_plane_tables_host(FusedState& fs, unsigned int k, const device_plane_info& host_plane, bool coh);
int fused_set_mesh_bounds(FusedState& fs, unsigned int m, float4 b, cudaStream_t st);
// The next step sorts the cell table even when the candidate lists hold
// (a mesh moved: its spheres' cells changed).
int fused_force_sort(FusedState& fs, cudaStream_t st);
// Runs one step.  When e0/e1 are given they bracket the contact kernel.
int fused_step(FusedState& fs, FusedArgs& a, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
               unsigned int* nlaunch);
// Kinetic energy and stored particle-particle + plane contacts of each scene
// of a batch (d_first [nscene + 1] particle ranges, d_out [2 * nscene]).
int fused_scene_energy(const double* vel, const double* ep, const double* ev, const double* mass,
                       const double* inertia, const unsigned int* d_first, unsigned int nscene, const unsigned int* c0,
                       const unsigned int* c1, double* d_out, double* ke, unsigned int* ncontact, cudaStream_t st);
// Kinetic energy (translational + rotational) and number of stored contacts.
int fused_energy(FusedState& fs, const double* vel, const double* ep, const double* ev, const double* mass,
                 const double* inertia, unsigned int ns, const unsigned int* c0, const unsigned int* c1,
                 const unsigned int* c2, unsigned int np, double* ke, unsigned int* ncontact, cudaStream_t st);

// Contact kernels (one translation unit per arithmetic type).
struct ContactLaunch {
    device_dem_parameters prm;
    MixedTune tune;
    unsigned int np, nentry;
    int vel_compat;
    int rolling_per_sphere;
    bool rolling;
    const double* snap_pos;
    const double* snap_vel;
    const double* snap_om;
    const float* snap_f;
    float margin;
    const float* mA;
    const float* mL;
    const float* mB;
    const float* mC;
    const unsigned int* mIT;
    float4* rec;  // [np*4] records (see FusedState)
    float* fA;
    float* fB;
    float* fC;
    // candidate lists (use_list): see FusedState
    bool use_list;
    unsigned int* vl_ids;
    unsigned int* vl_cnt;
    float* vl_xb;
    unsigned int* vl_flag;      // [kVlWords]: see FusedState
    float skin_f, half_skin2_f;
    const PlaneF* planef;
    const PlaneDF* planedf;
    double inv_cs;   // 1 / cell size
    float cs_f;      // cell size in FP32 (hi of the float pair)
    float cs_lo;     // cell size - cs_f
    float inv_cs_f;
    float o_hi[3], o_lo[3];  // grid origin as float pairs
    float dt_f, hdt_f, h2_f; // dt, dt/2, dt^2/2
    float g_f[3];            // gravity
    const unsigned int* sorted_index;
    const unsigned int* cstart;
    const unsigned int* cend;
    const unsigned int* skey;
    // state (original order)
    const double* pos_cur;  // x_{n+1} (this step's positions)
    double* pos_next;       // x_{n+2} out
    const double* ep_cur;
    double* ep_next;
    double *vel, *acc, *ev, *ea;
    const double *mass, *inertia;
    float4 *accf, *eaf;         // FP32 copies (see FusedState), sphere handles
    const float4* jm;
    unsigned int *k_out, *v_out;
    // contacts
    bool has_pp;
    const unsigned int* pp_count_old;
    const unsigned int* pp_id_old;
    const double* pp_tsd_old;
    unsigned int* pp_count_new;
    unsigned int* pp_id_new;
    double* pp_tsd_new;
    const device_plane_info* planes;
    unsigned int nplane, nmesh;
    unsigned int mesh_first[kMaxFusedMeshes], mesh_ntri[kMaxFusedMeshes];
    int mesh_body[kMaxFusedMeshes];
    unsigned int *pl_count, *pl_id;
    double* pl_tsd;
    const device_triangle_info* tri;
    unsigned int *ms_count, *ms_id;
    double* ms_tsd;
    const float4* mesh_bs;  // [nmesh] bounding spheres (see FusedState)
    const double* tri_sphere;  // [ntri*4] fitted sphere of every triangle (x, y, z, r)
    // cylinders (sphere scenes): cylinder k is body nplane + k; its pair
    // list (MAX_P2CY_COUNT slots) is updated in place like the plane list
    unsigned int ncyl;
    const device_cylinder_info* cyl;
    unsigned int *cy_count, *cy_id;
    double* cy_tsd;
    const double* body;
    const mat_pair* mp;
    const MatF* mpf;
    double* bsums;  // [nbody][nblocks][6]
    unsigned int nblocks;
    unsigned int* status;
    // batched scenes: material tables hold nscene particle-pair entries, then
    // one per body; a particle only meets particles and planes of its scene
    unsigned int nscene;
    const unsigned int* scene_of;          // [np] or null (one scene)
    const unsigned int* scene_plane_first; // [nscene + 1] or null
    // clusters (cl.ns > 0).  The records of a member carry its cluster's
    // mass, spin and velocity at the member's centre, so the particle-pair
    // kernels treat members as spheres apart from the exclusion of partners
    // |id - k| <= neach (impl:556-558)
    ClusterTab cl;
    const double* rloc;
    const double* cpos_cur;  // x_c of this step
    double* cpos_next;       // x_c of the next step out
};

// Scene of a particle and the range of planes it sees.
__host__ __device__ inline unsigned int scene_index(const ContactLaunch& c, unsigned int oid)
{
    return c.scene_of ? c.scene_of[oid] : 0u;
}

cudaError_t launch_fused_contact_fp64(const ContactLaunch& c, cudaStream_t st);
cudaError_t launch_fused_contact_mixed(const ContactLaunch& c, cudaStream_t st);

// The cell sort of a step as the persistent batched step runs it: gated by
// *gate (rebuild or overflowed list), the clear of last step's cells (when
// have_prev), the radix passes over (k0, v0) with (k1, v1) as the other
// buffer, and the reorder into the mixed records; bar and limit_ns: the
// grid barriers (FusedState::d_bar, persist_limit_ns).
struct BatchSort {
    const unsigned int* gate;
    unsigned int *k0, *v0, *k1, *v1, *hist;
    unsigned int n, np, bits, ntiles;
    int have_prev;
    unsigned int *skey_prev, *cstart, *cend, *sorted_index;
    const float4* rec;
    float4 *mA, *mL, *mB, *mC;
    uint2* mIT;
    unsigned int* bar;
    unsigned long long limit_ns;
};
// One cooperative launch for a whole list step of a batched mixed handle
// (sphere scenes, candidate lists): the gated sort, the list pair phase,
// the body phase and the flag roll, with grid barriers between the phases.
// occ: 768 or 1024 threads per SM (80 or 64 registers); *grid caches the
// co-resident grid of that budget (0: not yet known).  Zeroes the barrier
// words first.
cudaError_t launch_batch_step(const ContactLaunch& c, const BatchSort& b, unsigned int occ, unsigned int* grid,
                              cudaStream_t st);
// The mixed pair kernels' mesh forms and the cluster body kernel
// (xdem_fused_mixed_mesh.cu, compiled with FMA contraction).
cudaError_t launch_mixed_mesh_pairs(const ContactLaunch& c, cudaStream_t st);
cudaError_t launch_mixed_cluster_bodies(const ContactLaunch& c, cudaStream_t st);
constexpr int kFusedThreads = 128;

// Packed unwrapped cell coordinates: 11 bits x, 11 bits y, 10 bits z, each
// modulo its field size.  Two cells whose packed difference is within one
// cell per axis are neighbours unless 2048 / 1024 cells apart.
__host__ __device__ inline unsigned int pack_cell(int x, int y, int z)
{
    return ((unsigned int)x & 2047u) | (((unsigned int)y & 2047u) << 11) | (((unsigned int)z & 1023u) << 22);
}

}  // namespace xdem
