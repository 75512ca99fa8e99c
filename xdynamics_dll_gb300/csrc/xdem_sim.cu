// xdem_sim.cu -- scene handle: the whole DEM step on the GPU.
//
// The handle owns particle state (reference layout), pair lists, the cell
// grid, planes and triangle meshes.  xdem_sim_step advances it in the order of
// xIntegratorVV::OneStepSimulation (source/xdynamics_simulation/
// xIntegratorVV.cpp:26-63): position update, hashing of particles and mesh
// spheres, sort and cell ranges, particle-particle contact, planes in id
// order, meshes, rolling resistance, velocity update.  Every allocation
// happens in create / set / add; a step allocates nothing.
//
// Two step paths share the state:
//  * launcher_path = 1: the launcher kernels (xdem_kernels.cu) one after the
//    other, the reference's own structure;
//  * launcher_path = 0: the fused sorted-order step (xdem_fused.cuh), one
//    contact+integration kernel per step over a cell-sorted snapshot.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "xdem_sim_impl.h"

namespace {

int cerr(cudaError_t e)
{
    if (e == cudaSuccess) return XDEM_OK;
    fprintf(stderr, "xdem_sim: CUDA error %s\n", cudaGetErrorString(e));
    return XDEM_ERR_CUDA;
}

template <class T>
cudaError_t dalloc(T*& p, size_t n)
{
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T));
}

template <class T>
void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

int bits_for(unsigned long long ncell)
{
    int b = 0;
    while (b < 32 && (1ull << b) < ncell) ++b;
    return b == 0 ? 1 : b;
}

// ---- host restatement of the mesh setup (xParticleMeshObjectContact.cpp:77-135)
struct h3 { double x, y, z; };
h3 hsub(h3 a, h3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
h3 hadd(h3 a, h3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
h3 hmul(double s, h3 a) { return {s * a.x, s * a.y, s * a.z}; }
h3 hdiv(h3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
double hdot(h3 a, h3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
double hlen(h3 a) { return std::sqrt(hdot(a, a)); }
h3 hcross(h3 a, h3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
void hrot(const double e[4], h3 r[3])
{
    r[0] = {2.0 * (e[0] * e[0] + e[1] * e[1] - 0.5), 2.0 * (e[1] * e[2] - e[0] * e[3]), 2.0 * (e[1] * e[3] + e[0] * e[2])};
    r[1] = {2.0 * (e[1] * e[2] + e[0] * e[3]), 2.0 * (e[0] * e[0] + e[2] * e[2] - 0.5), 2.0 * (e[2] * e[3] - e[0] * e[1])};
    r[2] = {2.0 * (e[1] * e[3] - e[0] * e[2]), 2.0 * (e[2] * e[3] + e[0] * e[1]), 2.0 * (e[0] * e[0] + e[3] * e[3] - 0.5)};
}
h3 hglobal(const h3 r[3], h3 v) { return {hdot(r[0], v), hdot(r[1], v), hdot(r[2], v)}; }
h3 hlocal(const h3 r[3], h3 v)
{
    return {r[0].x * v.x + r[1].x * v.y + r[2].x * v.z, r[0].y * v.x + r[1].y * v.y + r[2].y * v.z,
            r[0].z * v.x + r[1].z * v.y + r[2].z * v.z};
}

// FitSphereToTriangle (source/xdynamics_algebra/xUtilityFunction.cpp:379-416):
// circumcentre of the triangle moved along the normal until the triangle
// subtends the fraction ft of the sphere.
void fit_sphere(h3 P, h3 Q, h3 R, double ft, double out[4])
{
    const h3 V = hsub(Q, P), W = hsub(R, P);
    h3 N = hcross(V, W);
    N = hdiv(N, hlen(N));
    const h3 M1 = hdiv(hadd(Q, P), 2), M2 = hdiv(hadd(R, P), 2);
    const h3 D1 = hcross(N, V), D2 = hcross(N, W);
    double t = 0.0;
    if (std::fabs(D1.x * D2.y - D1.y * D2.x) > 1E-13)
        t = (D2.x * (M1.y - M2.y)) / (D1.x * D2.y - D1.y * D2.x) - (D2.y * (M1.x - M2.x)) / (D1.x * D2.y - D1.y * D2.x);
    else if (std::fabs(D1.x * D2.z - D1.z * D2.x) > 1E-13)
        t = (D2.x * (M1.z - M2.z)) / (D1.x * D2.z - D1.z * D2.x) - (D2.z * (M1.x - M2.x)) / (D1.x * D2.z - D1.z * D2.x);
    else if (std::fabs(D1.y * D2.z - D1.z * D2.y) > 1E-13)
        t = (D2.y * (M1.z - M2.z)) / (D1.y * D2.z - D1.z * D2.y) - (D2.z * (M1.y - M2.y)) / (D1.y * D2.z - D1.z * D2.y);
    const h3 Ctri = hadd(M1, hmul(t, D1));
    h3 Csph{0, 0, 0};
    double fc = 0, r = hlen(hsub(P, Ctri));
    for (int it = 0; std::fabs(fc - ft) > 1e-4 && it < 1000; ++it) {
        const double d = ft * r;
        const double p = d / hlen(N);
        Csph = hsub(Ctri, hmul(p, N));
        r = hlen(hsub(P, Csph));
        fc = d / r;
    }
    out[0] = Csph.x; out[1] = Csph.y; out[2] = Csph.z; out[3] = r;
}

// (Re)allocates grid and contact tables after the body set changed.
int ensure_tables(xdem_sim* s)
{
    if (!s->dirty_alloc) return XDEM_OK;
    const unsigned int n = s->np;
    s->nentry = n + s->ntri_total;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto*& p, size_t cnt) {
        if (e == cudaSuccess) e = dalloc(p, cnt);
    };
    A(s->k0, s->nentry); A(s->v0, s->nentry); A(s->k1, s->nentry); A(s->v1, s->nentry);
    A(s->hist, radix_hist_size(s->nentry));
    A(s->sorted_index, s->nentry);
    // partial rows: one per warp (the mixed sphere body kernel writes one
    // row per warp; every other emitter writes one per block of at least 64)
    const unsigned int nb = blocks_for(s->nentry, 32);
    const size_t nbody = std::max<size_t>(s->bodies.size(), 1);
    // batched handles keep no body wrenches: no per-block partials
    A(s->bsums, (size_t)nb * 6 * (s->nscene > 1 ? 1 : nbody));
    A(s->wrench, 6 * nbody);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->wrench, 0, 6 * nbody * sizeof(double), s->st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s->bsums, 0, (size_t)nb * 6 * (s->nscene > 1 ? 1 : nbody) * sizeof(double), s->st);
    if (e != cudaSuccess) return XDEM_ERR_ALLOC;
    if (int r = fused_alloc(s->fs, n, s->nentry, s->precision_mixed(), s->st,
                            s->clusters && s->precision_mixed() ? s->ns : 0))
        return r;
    s->skey = nullptr;
    s->cells_clean = false;
    s->dirty_alloc = false;
    s->dirty_mesh_bs = true;
    return XDEM_OK;
}

// Bounding sphere of mesh m at its body's pose for the fused step: centre
// p + A(e) c_local relative to the grid origin, radius = reach plus the FP32
// slack of the test (a cohesive mesh material reaches beyond contact: every
// sphere searches it).
int push_mesh_bounds(xdem_sim* s, unsigned int m)
{
    const SimMesh& sm = s->meshes[m];
    const double* rec = s->bodies[sm.body].rec;
    h3 R[3];
    hrot(rec + XDEM_E0, R);
    const h3 c = hadd(h3{rec[XDEM_PX], rec[XDEM_PY], rec[XDEM_PZ]},
                      hglobal(R, h3{sm.c_local[0], sm.c_local[1], sm.c_local[2]}));
    const h3 rel = hsub(c, h3{s->prm.world_origin.x, s->prm.world_origin.y, s->prm.world_origin.z});
    const double slack = 1e-6 + 1e-6 * (hlen(rel) + sm.reach);
    const bool coh = s->body_cp[sm.body].coh != 0.0;
    const float4 b = make_float4((float)rel.x, (float)rel.y, (float)rel.z,
                                 coh ? 1e18f : (float)(sm.reach + slack));
    return fused_set_mesh_bounds(s->fs, m, b, s->st);
}

int upload_bodies(xdem_sim* s)
{
    if (!s->dirty_bodies) return XDEM_OK;
    cudaError_t e = cudaSuccess;
    const size_t nb = s->bodies.size();
    const size_t S = s->nscene;
    if (s->planes.size()) {
        if (s->planes.size() > s->plane_cap) {
            e = dalloc(s->d_planes, s->planes.size());
            s->plane_cap = e == cudaSuccess ? s->planes.size() : 0;
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_planes, s->planes.data(), s->planes.size() * sizeof(device_plane_info),
                                cudaMemcpyHostToDevice, s->st);
    }
    if (e == cudaSuccess && s->cylinders.size()) {
        if (s->cylinders.size() > s->cyl_cap) {
            e = dalloc(s->d_cyl, s->cylinders.size());
            s->cyl_cap = e == cudaSuccess ? s->cylinders.size() : 0;
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_cyl, s->cylinders.data(), s->cylinders.size() * sizeof(device_cylinder_info),
                                cudaMemcpyHostToDevice, s->st);
    }
    std::vector<double> rec(std::max<size_t>(nb, 1) * 15, 0.0);
    for (size_t i = 0; i < nb; ++i) std::memcpy(&rec[i * 15], s->bodies[i].rec, sizeof(double) * 15);
    if (e == cudaSuccess && rec.size() / 15 > s->body_cap) {
        e = dalloc(s->d_body, rec.size());
        s->body_cap = e == cudaSuccess ? rec.size() / 15 : 0;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_body, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice, s->st);
    // material constants: [s] particle-particle of scene s, [nscene + b] body b
    std::vector<mat_pair> mps(S + nb);
    for (size_t k = 0; k < S; ++k)
        mps[k] = make_mat_pair(S > 1 ? s->scene_cp[k] : s->pp_cp, s->prm.contact_model, false);
    for (size_t i = 0; i < nb; ++i)
        mps[S + i] = make_mat_pair(s->body_cp[i], s->prm.contact_model,
                                   s->clusters && s->bodies[i].kind == 0 /* cluster-plane swap */);
    if (e == cudaSuccess && mps.size() > s->mp_cap) {
        e = dalloc(s->d_mp, mps.size());
        s->mp_cap = e == cudaSuccess ? mps.size() : 0;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_mp, mps.data(), mps.size() * sizeof(mat_pair), cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return cerr(e);
    s->dirty_bodies = false;
    const double org[3] = {s->prm.world_origin.x, s->prm.world_origin.y, s->prm.world_origin.z};
    return fused_set_bodies(s->fs, s->d_planes, (unsigned int)s->planes.size(), s->d_body, s->d_mp,
                            s->planes.data(), mps.data(), (unsigned int)mps.size(), (unsigned int)S, org, s->st);
}

// ---------------------------------------------------------------- launcher-order step
int step_launcher(xdem_sim* s, cudaEvent_t e0, cudaEvent_t e1)
{
    const cudaStream_t st = s->st;
    const device_dem_parameters& p = s->prm;
    const unsigned int n = s->np;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
        s->launches++;
    };
    if (s->clusters)
        ok(launch_vv_cluster_position(p, s->pos, s->cpos, s->ep, s->rloc, s->vel, s->acc, s->ev, s->ea, s->xci, s->ns, st));
    else
        ok(launch_vv_position(p, s->pos, s->ep, s->vel, s->ev, s->acc, s->ea, n, st));
    // empty the cells the previous step filled, then hash, sort, cell ranges
    if (!s->cells_clean) {
        ok(launch_fill_u32(s->cstart, 0xffffffffu, s->ncell, st));
        ok(cudaMemsetAsync(s->cend, 0, s->ncell * sizeof(unsigned int), st));
        s->cells_clean = true;
    } else if (s->skey) {
        ok(launch_clear_cells(s->skey, s->nentry, s->cstart, s->cend, st));
    }
    ok(launch_hash(p, s->k0, s->v0, s->pos, 0, n, s->d_status, st));
    for (const SimMesh& m : s->meshes)
        ok(launch_hash(p, s->k0, s->v0, s->d_sphere + 4 * (size_t)m.first, n + m.first, m.ntri, s->d_status, st));
    unsigned int *sk = nullptr, *sv = nullptr;
    ok(radix_sort_pairs(s->k0, s->v0, s->k1, s->v1, s->hist, s->nentry, bits_for(s->ncell), &sk, &sv, st));
    s->launches += 3 * ((bits_for(s->ncell) + 7) / 8) - 1;
    ok(launch_cell_bounds(sk, sv, s->cstart, s->cend, s->sorted_index, s->nentry, st));
    s->skey = sk;
    // contacts (xContactManager.cpp:458-472)
    const unsigned int nb = blocks_for(n);
    if (e0) cudaEventRecord(e0, st);
    if (s->has_pp) {
        if (s->clusters)
            ok(launch_clusters_p2p(p, s->pos, s->cpos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax,
                                   s->rres, s->pp_count, s->pp_id, s->pp_tsd, s->sorted_index, s->cstart, s->cend,
                                   s->d_mp, s->xci, n, s->d_status, st));
        else
            ok(launch_p2p(p, s->pos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass, s->tmax, s->rres,
                          s->pp_count, s->pp_id, s->pp_tsd, s->sorted_index, s->cstart, s->cend, s->d_mp, n,
                          s->d_status, st));
    }
    if (e1) cudaEventRecord(e1, st);
    for (size_t b = 0; b < s->bodies.size(); ++b) {
        const SimBody& bd = s->bodies[b];
        BodyPartials bp{};
        bp.block_sums = s->bsums + (size_t)b * nb * 6;
        const double* dbi = s->d_body + 15 * b;
        const mat_pair* mp = s->d_mp + s->nscene + b;
        if (bd.kind == 0) {
            const device_plane_info* pl = s->d_planes + bd.index;
            if (s->clusters)
                ok(launch_cluster_plane(p, pl, dbi, mp, bp, s->pos, s->cpos, s->ep, s->vel, s->ev, s->force,
                                        s->moment, s->mass, s->tmax, s->rres, s->pl_count, s->pl_id, s->pl_tsd,
                                        s->xci, n, s->d_status, st));
            else
                ok(launch_plane(p, pl, dbi, mp, bp, s->pos, s->ep, s->vel, s->ev, s->force, s->moment, s->mass,
                                s->tmax, s->rres, s->pl_count, s->pl_id, s->pl_tsd, n, s->d_status, st));
        } else if (bd.kind == 2) {
            ok(launch_cylinder(p, s->d_cyl + bd.index, dbi, mp, bp, s->pos, s->clusters ? s->cpos : nullptr, s->ep,
                               s->vel, s->ev, s->force, s->moment, s->mass, s->tmax, s->rres, s->cy_count, s->cy_id,
                               s->cy_tsd, s->clusters ? s->xci : nullptr, n, s->d_status, st));
        } else {
            const SimMesh& m = s->meshes[bd.index];
            ok(launch_mesh(p, s->d_tri + m.first, n, s->clusters ? 2 : 1, dbi, mp, bp, s->pos,
                           s->clusters ? s->cpos : nullptr, s->ep, s->vel, s->ev, s->force, s->moment, s->mass,
                           s->tmax, s->rres, s->ms_count, s->ms_id, s->ms_tsd, s->sorted_index, s->cstart, s->cend,
                           s->clusters ? s->xci : nullptr, n, m.ntri, s->d_status, st));
        }
        ok(launch_sum_block_partials(bp.block_sums, nb, s->wrench + 6 * b, st));
    }
    if (s->clusters)
        ok(launch_cluster_rolling(p, s->tmax, s->rres, s->inertia, s->ep, s->ev, s->moment, s->xci, n, st));
    else
        ok(launch_rolling(p, s->tmax, s->rres, s->inertia, s->ep, s->ev, s->moment, n, st, s->rolling_per_sphere));
    if (s->clusters)
        ok(launch_vv_cluster_velocity(p, s->vel, s->acc, s->ep, s->ev, s->ea, s->force, s->moment, s->mass,
                                      s->inertia, s->xci, s->ns, st));
    else
        ok(launch_vv_velocity(p, s->vel, s->acc, s->ep, s->ev, s->ea, s->force, s->moment, s->mass, s->inertia, n,
                              s->cfg.velocity_compat, st));
    return cerr(e);
}

// The cluster table of the mixed step, when the handle's clusters fit it:
// every type with the same member count (so id / neach is the cluster of any
// sphere, as impl:485-611 takes it), types tiling the clusters and spheres
// in order, member offsets for every type, no rolling resistance and no
// cohesion (the FP64 launcher kernels carry those).  XDEM_ERR_ARG otherwise.
int mixed_cluster_tab(const xdem_sim* s, ClusterTab& t)
{
    t = ClusterTab{};
    const size_t nco = s->h_xci.size();
    if (!nco || nco > kMaxClusterTypes) return XDEM_ERR_ARG;
    const unsigned int neach = s->h_xci[0].neach;
    if (!neach || s->nrloc < nco * neach) return XDEM_ERR_ARG;
    unsigned long long ncl = 0;
    for (size_t k = 0; k < nco; ++k) {
        const xClusterInformation& x = s->h_xci[k];
        if (x.neach != neach || x.scid != ncl || (unsigned long long)x.sid != ncl * neach) return XDEM_ERR_ARG;
        t.first[k] = x.scid;
        ncl += x.count;
    }
    if (ncl != s->ns || ncl * neach != s->np) return XDEM_ERR_ARG;
    auto plain = [](const device_contact_property& c) { return c.rfric == 0.0 && c.coh == 0.0; };
    if (s->has_pp && !plain(s->pp_cp)) return XDEM_ERR_ARG;
    for (const device_contact_property& c : s->body_cp)
        if (!plain(c)) return XDEM_ERR_ARG;
    t.ns = s->ns;
    t.neach = neach;
    t.ntype = (unsigned int)nco;
    t.first[nco] = s->ns;
    return XDEM_OK;
}

// Pair tables of one contact kind: 0 particle pairs, 1 planes, 2 triangle
// meshes, 3 cylinders.
struct PairTables {
    unsigned int cap;
    unsigned int *count, *id;
    double* tsd;
};
PairTables pair_tables(xdem_sim* s, int kind)
{
    switch (kind) {
    case 0: return PairTables{MAX_P2P_COUNT, s->pp_count, s->pp_id, s->pp_tsd};
    case 1: return PairTables{MAX_P2PL_COUNT, s->pl_count, s->pl_id, s->pl_tsd};
    case 2: return PairTables{MAX_P2MS_COUNT, s->ms_count, s->ms_id, s->ms_tsd};
    default: return PairTables{MAX_P2CY_COUNT, s->cy_count, s->cy_id, s->cy_tsd};
    }
}

// Steps run on the fused step (sphere scenes of either precision, and
// mixed cluster scenes) unless the launcher path was asked for; an FP64
// scene with cylinders runs the launcher kernels, a mixed scene with
// cylinders (spheres or clusters) the fused step's cylinder loops.
bool fused_path(const xdem_sim* s)
{
    if (s->cfg.launcher_path || (s->clusters && !s->precision_mixed())) return false;
    return s->cylinders.empty() || s->precision_mixed();
}

// The particle-pair tangential history of a mixed handle on the fused step
// is stored as float2 (ds, previous s_dot) in the first half of its double2
// buffer: the mixed kernels compute it in FP32, so the FP32 copy is exact
// and halves its traffic.  The pair-list calls convert at the boundary.
bool pp_history_f32(const xdem_sim* s) { return s->precision_mixed() && fused_path(s); }

FusedArgs fused_args(xdem_sim* s)
{
    FusedArgs a{};
    a.prm = s->prm;
    a.np = s->np;
    a.nentry = s->nentry;
    a.ncell = s->ncell;
    a.sort_bits = bits_for(s->ncell);
    a.vel_compat = s->cfg.velocity_compat;
    a.rolling_per_sphere = s->rolling_per_sphere;
    a.pos = &s->pos; a.vel = s->vel; a.acc = s->acc; a.ep = &s->ep; a.ev = s->ev; a.ea = s->ea;
    a.mass = s->mass; a.inertia = s->inertia; a.tmax = s->tmax; a.rres = s->rres;
    a.k0 = s->k0; a.v0 = s->v0; a.k1 = s->k1; a.v1 = s->v1; a.hist = s->hist;
    a.cstart = s->cstart; a.cend = s->cend; a.sorted_index = s->sorted_index;
    a.has_pp = s->has_pp;
    a.pp_count = &s->pp_count; a.pp_id = &s->pp_id; a.pp_tsd = &s->pp_tsd;
    a.pl_count = s->pl_count; a.pl_id = s->pl_id; a.pl_tsd = s->pl_tsd;
    a.nplane = (unsigned int)s->planes.size();
    a.nbody = (unsigned int)s->bodies.size();
    a.nmesh = (unsigned int)s->meshes.size();
    for (unsigned int m = 0; m < a.nmesh && m < kMaxFusedMeshes; ++m) {
        a.mesh_first[m] = s->meshes[m].first;
        a.mesh_ntri[m] = s->meshes[m].ntri;
        a.mesh_body[m] = s->meshes[m].body;
    }
    a.tri = s->d_tri; a.tri_sphere = s->d_sphere;
    a.ms_count = s->ms_count; a.ms_id = s->ms_id; a.ms_tsd = s->ms_tsd;
    a.ncyl = (unsigned int)s->cylinders.size();
    a.cyl = s->d_cyl;
    a.cy_count = s->cy_count; a.cy_id = s->cy_id; a.cy_tsd = s->cy_tsd;
    a.body = s->d_body; a.mp = s->d_mp;
    a.bsums = s->bsums; a.wrench = s->wrench;
    a.status = s->d_status;
    a.rolling = s->has_pp && s->pp_cp.rfric != 0.0;
    for (const device_contact_property& cp : s->body_cp) a.rolling = a.rolling || cp.rfric != 0.0;
    for (const device_contact_property& cp : s->scene_cp) a.rolling = a.rolling || cp.rfric != 0.0;
    a.nscene = s->nscene;
    a.scene_of = s->d_scene_of;
    a.scene_plane_first = s->d_scene_plane_first;
    a.ns_state = s->ns;
    if (s->clusters) {
        mixed_cluster_tab(s, a.cl);
        a.cpos = &s->cpos;
        a.rloc = s->rloc;
    }
    return a;
}

// ---- CUDA graphs of the fused step
void drop_graph(xdem_sim* s)
{
    for (auto& g : s->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = xdem_sim::StepGraph{};
    }
}

void graph_key(const xdem_sim* s, const void* k[8])
{
    k[0] = s->pos; k[1] = s->fs.pos_alt; k[2] = s->ep; k[3] = s->fs.ep_alt;
    k[4] = s->pp_count; k[5] = s->fs.pp_count2; k[6] = s->pp_id; k[7] = s->pp_tsd;
}

int find_graph(const xdem_sim* s)
{
    const void* k[8];
    graph_key(s, k);
    for (int g = 0; g < 2; ++g) {
        if (!s->graphs[g].exec) continue;
        bool same = true;
        for (int i = 0; i < 8; ++i) same = same && k[i] == s->graphs[g].key[i];
        if (same) return g;
    }
    return -1;
}

// The host side of one primed fused step: its buffer swaps (fused_step).
void step_swaps(xdem_sim* s)
{
    std::swap(s->pos, s->fs.pos_alt);
    std::swap(s->ep, s->fs.ep_alt);
    if (s->clusters) std::swap(s->cpos, s->fs.cpos_alt);
    if (s->has_pp) {
        std::swap(s->pp_count, s->fs.pp_count2);
        std::swap(s->pp_id, s->fs.pp_id2);
        std::swap(s->pp_tsd, s->fs.pp_tsd2);
    }
}

// Records one fused step into graph slot `slot`.  Nothing runs during the
// capture, but the host side of the step (its swaps) does: on success the
// caller must launch the graph; on failure the arrangement is restored.
int capture_step_graph(xdem_sim* s, int slot)
{
    xdem_sim::StepGraph& sg = s->graphs[slot];
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    sg = xdem_sim::StepGraph{};
    const void* key[8];
    graph_key(s, key);
    double *pos = s->pos, *pos_alt = s->fs.pos_alt, *ep = s->ep, *ep_alt = s->fs.ep_alt;
    double *cpos = s->cpos, *cpos_alt = s->fs.cpos_alt;
    unsigned int *c0 = s->pp_count, *c1 = s->fs.pp_count2, *i0 = s->pp_id, *i1 = s->fs.pp_id2;
    double *t0 = s->pp_tsd, *t1 = s->fs.pp_tsd2;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return XDEM_ERR_CUDA;
    FusedArgs a = fused_args(s);
    unsigned int nl = 0;
    int r = fused_step(s->fs, a, s->st, nullptr, nullptr, &nl);
    const cudaError_t ec = cudaStreamEndCapture(s->st, &g);
    if (r == XDEM_OK && (ec != cudaSuccess || !g || cudaGraphInstantiate(&sg.exec, g, 0) != cudaSuccess)) {
        sg.exec = nullptr;
        r = XDEM_ERR_CUDA;
    }
    if (g) cudaGraphDestroy(g);
    if (r != XDEM_OK) {
        s->pos = pos; s->fs.pos_alt = pos_alt; s->ep = ep; s->fs.ep_alt = ep_alt;
        s->cpos = cpos; s->fs.cpos_alt = cpos_alt;
        s->pp_count = c0; s->fs.pp_count2 = c1; s->pp_id = i0; s->fs.pp_id2 = i1;
        s->pp_tsd = t0; s->fs.pp_tsd2 = t1;
        cudaGetLastError();
        return r;
    }
    for (int i = 0; i < 8; ++i) sg.key[i] = key[i];
    sg.launches = nl;
    return XDEM_OK;
}

}  // namespace

bool xdem_sim::precision_mixed() const { return cfg.precision == XDEM_MIXED; }

// ============================================================================
extern "C" {

XDEM_API int xdem_sim_create(const xdem_sim_config* cfg, xdem_sim** out)
{
    if (!cfg || !out || cfg->np == 0 || !(cfg->cell_size > 0) || !(cfg->dt > 0)) return XDEM_ERR_ARG;
    if (cfg->precision != XDEM_FP64 && cfg->precision != XDEM_MIXED) return XDEM_ERR_ARG;
    for (int i = 0; i < 3; ++i) {
        const unsigned int g = cfg->grid_size[i];
        if (!g || (g & (g - 1))) return XDEM_ERR_ARG;
    }
    const unsigned long long ncell =
        (unsigned long long)cfg->grid_size[0] * cfg->grid_size[1] * cfg->grid_size[2];
    if (ncell > (1ull << 31)) return XDEM_ERR_ARG;
    xdem_sim* s = new (std::nothrow) xdem_sim();
    if (!s) return XDEM_ERR_ALLOC;
    s->cfg = *cfg;
    s->np = cfg->np;
    s->ns = cfg->ns ? cfg->ns : cfg->np;
    s->clusters = s->ns != s->np;
    device_dem_parameters& p = s->prm;
    std::memset(&p, 0, sizeof(p));
    p.contact_model = cfg->contact_model;
    p.np = s->np;
    p.nCluster = s->clusters ? s->ns : 0;
    p.grid_size = xdem_uint3{cfg->grid_size[0], cfg->grid_size[1], cfg->grid_size[2]};
    p.ncell = (unsigned int)ncell;
    p.dt = cfg->dt;
    p.half2dt = 0.5 * cfg->dt * cfg->dt;
    p.cell_size = cfg->cell_size;
    p.gravity = xdem_double3{cfg->gravity[0], cfg->gravity[1], cfg->gravity[2]};
    p.world_origin = xdem_double3{cfg->world_origin[0], cfg->world_origin[1], cfg->world_origin[2]};
    s->ncell = ncell;
    const size_t n = s->np, ns = s->ns;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto*& q, size_t cnt) {
        if (e == cudaSuccess) e = dalloc(q, cnt);
    };
    A(s->pos, n * 4); A(s->vel, ns * 3); A(s->acc, ns * 3); A(s->ep, ns * 4); A(s->ev, ns * 4); A(s->ea, ns * 4);
    A(s->force, n * 3); A(s->moment, n * 3); A(s->mass, ns); A(s->inertia, ns * 3); A(s->tmax, n * 3);
    A(s->rres, n);
    A(s->pp_count, n); A(s->pp_id, n * MAX_P2P_COUNT); A(s->pp_tsd, n * MAX_P2P_COUNT * 2);
    A(s->pl_count, n); A(s->pl_id, n * MAX_P2PL_COUNT); A(s->pl_tsd, n * MAX_P2PL_COUNT * 2);
    A(s->ms_count, n); A(s->ms_id, n * MAX_P2MS_COUNT); A(s->ms_tsd, n * MAX_P2MS_COUNT * 2);
    A(s->cy_count, n); A(s->cy_id, n * MAX_P2CY_COUNT); A(s->cy_tsd, n * MAX_P2CY_COUNT * 2);
    A(s->cstart, ncell); A(s->cend, ncell);
    A(s->d_status, 1);
    A(s->d_mp, 65);
    A(s->d_body, 64 * 15);
    s->mp_cap = 65;
    s->body_cap = 64;
    if (s->clusters) A(s->cpos, ns * 4);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->own_st, cudaStreamNonBlocking);
    s->st = s->own_st;
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    // zero everything that carries over between steps
    auto Z = [&](void* q, size_t bytes) {
        if (e == cudaSuccess && q) e = cudaMemsetAsync(q, 0, bytes, s->st);
    };
    Z(s->force, n * 24); Z(s->moment, n * 24); Z(s->tmax, n * 24); Z(s->rres, n * 8);
    Z(s->pp_count, n * 4); Z(s->pp_id, n * 4 * MAX_P2P_COUNT); Z(s->pp_tsd, n * 16 * MAX_P2P_COUNT);
    Z(s->pl_count, n * 4); Z(s->pl_id, n * 4 * MAX_P2PL_COUNT); Z(s->pl_tsd, n * 16 * MAX_P2PL_COUNT);
    Z(s->ms_count, n * 4); Z(s->ms_id, n * 4 * MAX_P2MS_COUNT); Z(s->ms_tsd, n * 16 * MAX_P2MS_COUNT);
    Z(s->cy_count, n * 4); Z(s->cy_id, n * 4 * MAX_P2CY_COUNT); Z(s->cy_tsd, n * 16 * MAX_P2CY_COUNT);
    Z(s->d_status, 4);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        xdem_sim_destroy(s);
        return XDEM_ERR_ALLOC;
    }
    *out = s;
    return XDEM_OK;
}

XDEM_API int xdem_sim_destroy(xdem_sim* s)
{
    if (!s) return XDEM_ERR_ARG;
    if (s->st) cudaStreamSynchronize(s->st);
    drop_graph(s);
    fused_free(s->fs);
    double* dp[] = {s->pos, s->cpos, s->vel, s->acc, s->ep, s->ev, s->ea, s->force, s->moment, s->mass,
                    s->inertia, s->tmax, s->rres, s->rloc, s->pp_tsd, s->pl_tsd, s->ms_tsd, s->cy_tsd, s->d_body,
                    s->d_vlist, s->d_dlocal, s->d_sphere, s->bsums, s->wrench, s->d_scene_energy};
    for (double* q : dp)
        if (q) cudaFree(q);
    unsigned int* up[] = {s->k0, s->v0, s->k1, s->v1, s->hist, s->cstart, s->cend, s->sorted_index, s->pp_count,
                          s->pp_id, s->pl_count, s->pl_id, s->ms_count, s->ms_id, s->cy_count, s->cy_id, s->d_status,
                          s->d_scene_of, s->d_scene_first, s->d_scene_plane_first};
    for (unsigned int* q : up)
        if (q) cudaFree(q);
    if (s->xci) cudaFree(s->xci);
    if (s->d_mp) cudaFree(s->d_mp);
    if (s->d_planes) cudaFree(s->d_planes);
    if (s->d_cyl) cudaFree(s->d_cyl);
    if (s->d_tri) cudaFree(s->d_tri);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->pin_ev) cudaEventDestroy(s->pin_ev);
    if (s->h_pin) cudaFreeHost(s->h_pin);
    for (int i = 0; i < xdem_sim::kProfEvents; ++i) {
        if (s->pe0[i]) cudaEventDestroy(s->pe0[i]);
        if (s->pe1[i]) cudaEventDestroy(s->pe1[i]);
    }
    // a stream given by xdem_sim_set_stream belongs to the caller
    if (s->own_st) cudaStreamDestroy(s->own_st);
    delete s;
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_rolling_inertia(xdem_sim* s, int per_sphere)
{
    if (!s) return XDEM_ERR_ARG;
    s->rolling_per_sphere = per_sphere ? 1 : 0;
    s->dirty_bodies = true;  // captured step graphs bake the switch in
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_stream(xdem_sim* s, void* stream)
{
    if (!s) return XDEM_ERR_ARG;
    cudaStreamSynchronize(s->st);
    // NULL returns to the handle's own stream
    s->st = stream ? reinterpret_cast<cudaStream_t>(stream) : s->own_st;
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_state(xdem_sim* s, const double* pos, const double* vel, const double* acc,
                                const double* ep, const double* ev, const double* ea, const double* mass,
                                const double* inertia)
{
    if (!s || !pos || !mass || !inertia) return XDEM_ERR_ARG;
    const size_t n = s->np, ns = s->ns;
    // a state with a NaN or infinite entry is refused before any upload (the
    // handle keeps its previous state); the step's own hash check raises
    // XDEM_ERR_NONFINITE for values that turn non-finite on the device
    auto finite = [](const double* h, size_t cnt) {
        if (!h) return true;
        for (size_t i = 0; i < cnt; ++i)
            if (!std::isfinite(h[i])) return false;
        return true;
    };
    if (!(finite(pos, n * 4) && finite(vel, ns * 3) && finite(acc, ns * 3) && finite(ep, ns * 4) &&
          finite(ev, ns * 4) && finite(ea, ns * 4) && finite(mass, ns) && finite(inertia, ns * 3)))
        return XDEM_ERR_NONFINITE | XDEM_ERR_ARG;
    cudaError_t e = cudaSuccess;
    auto H = [&](double* d, const double* h, size_t cnt, double fill, int every, int off) {
        if (e != cudaSuccess) return;
        if (h) {
            e = cudaMemcpyAsync(d, h, cnt * sizeof(double), cudaMemcpyHostToDevice, s->st);
        } else {
            std::vector<double> z(cnt, 0.0);
            if (every)
                for (size_t i = off; i < cnt; i += every) z[i] = fill;
            e = cudaMemcpyAsync(d, z.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, s->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        }
    };
    H(s->pos, pos, n * 4, 0, 0, 0);
    H(s->vel, vel, ns * 3, 0, 0, 0);
    H(s->acc, acc, ns * 3, 0, 0, 0);
    H(s->ep, ep, ns * 4, 1.0, 4, 0);
    H(s->ev, ev, ns * 4, 0, 0, 0);
    H(s->ea, ea, ns * 4, 0, 0, 0);
    H(s->mass, mass, ns, 0, 0, 0);
    H(s->inertia, inertia, ns * 3, 0, 0, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    fused_state_written(s->fs);
    return cerr(e);
}

XDEM_API int xdem_sim_set_clusters(xdem_sim* s, const double* cpos, const xClusterInformation* xci, unsigned int nco,
                                   const double* rloc, unsigned int nrloc)
{
    if (!s || !s->clusters || !cpos || !xci || !nco || !rloc) return XDEM_ERR_ARG;
    cudaError_t e = cudaMemcpyAsync(s->cpos, cpos, (size_t)s->ns * 4 * sizeof(double), cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = dalloc(s->xci, nco);
    if (e == cudaSuccess) e = dalloc(s->rloc, (size_t)nrloc * 3);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->xci, xci, nco * sizeof(xClusterInformation), cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->rloc, rloc, (size_t)nrloc * 3 * sizeof(double), cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    s->nco = nco;
    s->nrloc = nrloc;
    s->h_xci.assign(xci, xci + nco);
    s->prm.nClusterObject = nco;
    s->dirty_bodies = true;
    fused_invalidate(s->fs);
    return cerr(e);
}

XDEM_API int xdem_sim_set_pp_contact(xdem_sim* s, const device_contact_property* cp)
{
    if (!s || !cp) return XDEM_ERR_ARG;
    s->pp_cp = *cp;
    s->has_pp = true;
    s->dirty_bodies = true;
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_scenes(xdem_sim* s, unsigned int nscene, const unsigned int* first,
                                 const device_contact_property* pp_cp, const unsigned int* plane_first)
{
    if (!s || !nscene || !first || !pp_cp || !plane_first) return XDEM_ERR_ARG;
    if (s->clusters || s->cfg.launcher_path) return XDEM_ERR_ARG;
    if (first[0] != 0 || first[nscene] != s->np || plane_first[0] != 0) return XDEM_ERR_ARG;
    for (unsigned int k = 0; k < nscene; ++k)
        if (first[k] > first[k + 1] || plane_first[k] > plane_first[k + 1]) return XDEM_ERR_ARG;
    std::vector<unsigned int> of(s->np);
    for (unsigned int k = 0; k < nscene; ++k)
        for (unsigned int i = first[k]; i < first[k + 1]; ++i) of[i] = k;
    cudaError_t e = dalloc(s->d_scene_of, s->np);
    if (e == cudaSuccess) e = dalloc(s->d_scene_first, nscene + 1);
    if (e == cudaSuccess) e = dalloc(s->d_scene_plane_first, nscene + 1);
    if (e == cudaSuccess) e = dalloc(s->d_scene_energy, 2 * (size_t)nscene);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->d_scene_of, of.data(), of.size() * sizeof(unsigned int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->d_scene_first, first, (nscene + 1) * sizeof(unsigned int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->d_scene_plane_first, plane_first, (nscene + 1) * sizeof(unsigned int),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return XDEM_ERR_ALLOC;
    s->nscene = nscene;
    s->scene_first.assign(first, first + nscene + 1);
    s->scene_plane_first.assign(plane_first, plane_first + nscene + 1);
    s->scene_cp.assign(pp_cp, pp_cp + nscene);
    s->pp_cp = pp_cp[0];
    s->has_pp = true;
    s->dirty_bodies = true;
    s->dirty_alloc = true;
    return XDEM_OK;
}

XDEM_API int xdem_sim_scene_energy(xdem_sim* s, double* ke, unsigned int* ncontact)
{
    if (!s || s->nscene < 2 || !s->d_scene_first) return XDEM_ERR_ARG;
    if (int r = ensure_tables(s)) return r;
    return fused_scene_energy(s->vel, s->ep, s->ev, s->mass, s->inertia, s->d_scene_first, s->nscene, s->pp_count,
                              s->pl_count, s->d_scene_energy, ke, ncontact, s->st);
}

XDEM_API int xdem_sim_add_plane(xdem_sim* s, const device_plane_info* plane, const double body[15],
                                const device_contact_property* cp, int* body_index)
{
    if (!s || !plane || !body || !cp) return XDEM_ERR_ARG;
    if (s->bodies.size() >= kMaxBodies) return XDEM_ERR_ARG;
    if (!s->meshes.empty() || !s->cylinders.empty()) return XDEM_ERR_ARG;  // planes first, in id order
    SimBody b{};
    b.kind = 0;
    b.index = (int)s->planes.size();
    std::memcpy(b.rec, body, sizeof(b.rec));
    device_plane_info pl = *plane;
    pl.id = (unsigned int)s->planes.size();  // ids in definition order (xParticlePlaneContact.cpp:53)
    s->planes.push_back(pl);
    s->bodies.push_back(b);
    s->body_cp.push_back(*cp);
    s->prm.nplane = (unsigned int)s->planes.size();
    s->dirty_bodies = true;
    s->dirty_alloc = true;
    if (body_index) *body_index = (int)s->bodies.size() - 1;
    return XDEM_OK;
}

XDEM_API int xdem_sim_add_cylinder(xdem_sim* s, const device_cylinder_info* cyl, const double body[15],
                                   const device_contact_property* cp, int* body_index)
{
    if (!s || !cyl || !body || !cp) return XDEM_ERR_ARG;
    if (s->bodies.size() >= kMaxBodies) return XDEM_ERR_ARG;
    if (!s->meshes.empty()) return XDEM_ERR_ARG;  // planes, then cylinders, then meshes
    SimBody b{};
    b.kind = 2;
    b.index = (int)s->cylinders.size();
    std::memcpy(b.rec, body, sizeof(b.rec));
    device_cylinder_info c = *cyl;
    c.id = (unsigned int)s->cylinders.size();  // ids in definition order, as xParticleCylinderContact counts them
    s->cylinders.push_back(c);
    s->bodies.push_back(b);
    s->body_cp.push_back(*cp);
    s->prm.ncylinder = (unsigned int)s->cylinders.size();
    s->dirty_bodies = true;
    s->dirty_alloc = true;
    if (body_index) *body_index = (int)s->bodies.size() - 1;
    return XDEM_OK;
}

XDEM_API int xdem_sim_add_mesh(xdem_sim* s, unsigned int ntri, const double* vlist_local, const double body[15],
                               const device_contact_property* cp, int* body_index)
{
    if (!s || !ntri || !vlist_local || !body || !cp) return XDEM_ERR_ARG;
    if (s->bodies.size() >= kMaxBodies || s->meshes.size() >= kMaxFusedMeshes) return XDEM_ERR_ARG;
    const unsigned int first = s->ntri_total;
    const h3 bp{body[XDEM_PX], body[XDEM_PY], body[XDEM_PZ]};
    h3 R[3];
    hrot(body + XDEM_E0, R);
    for (unsigned int i = 0; i < ntri; ++i) {
        const double* v = vlist_local + 9 * (size_t)i;
        const h3 P = hadd(bp, hglobal(R, h3{v[0], v[1], v[2]}));
        const h3 Q = hadd(bp, hglobal(R, h3{v[3], v[4], v[5]}));
        const h3 Rr = hadd(bp, hglobal(R, h3{v[6], v[7], v[8]}));
        device_triangle_info t{};
        t.id = (int)i;
        t.tid = first + i;
        t.P = xdem_double3{P.x, P.y, P.z};
        t.Q = xdem_double3{Q.x, Q.y, Q.z};
        t.R = xdem_double3{Rr.x, Rr.y, Rr.z};
        s->h_tri.push_back(t);
        double c[4];
        fit_sphere(P, Q, Rr, 0.8, c);
        for (int k = 0; k < 4; ++k) s->h_sphere.push_back(c[k]);
        const h3 loc = hlocal(R, hsub(h3{c[0], c[1], c[2]}, bp));
        s->h_dlocal.push_back(loc.x); s->h_dlocal.push_back(loc.y); s->h_dlocal.push_back(loc.z);
        for (int k = 0; k < 9; ++k) s->h_vlist.push_back(v[k]);
    }
    // bounding sphere of the vertices in the body frame (centroid, reach)
    double cl[3] = {0.0, 0.0, 0.0};
    for (unsigned int i = 0; i < 3 * ntri; ++i)
        for (int k = 0; k < 3; ++k) cl[k] += vlist_local[3 * (size_t)i + k] / (3.0 * ntri);
    double reach = 0.0;
    for (unsigned int i = 0; i < 3 * ntri; ++i) {
        const double* v = vlist_local + 3 * (size_t)i;
        reach = std::max(reach, hlen(hsub(h3{v[0], v[1], v[2]}, h3{cl[0], cl[1], cl[2]})));
    }
    s->ntri_total += ntri;
    const size_t nt = s->ntri_total;
    cudaError_t e = dalloc(s->d_tri, nt);
    if (e == cudaSuccess) e = dalloc(s->d_sphere, nt * 4);
    if (e == cudaSuccess) e = dalloc(s->d_dlocal, nt * 3);
    if (e == cudaSuccess) e = dalloc(s->d_vlist, nt * 9);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_tri, s->h_tri.data(), nt * sizeof(device_triangle_info), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_sphere, s->h_sphere.data(), nt * 4 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_dlocal, s->h_dlocal.data(), nt * 3 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_vlist, s->h_vlist.data(), nt * 9 * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return XDEM_ERR_ALLOC;
    SimBody b{};
    b.kind = 1;
    b.index = (int)s->meshes.size();
    std::memcpy(b.rec, body, sizeof(b.rec));
    s->bodies.push_back(b);
    s->body_cp.push_back(*cp);
    s->meshes.push_back(SimMesh{ntri, first, (int)s->bodies.size() - 1, {cl[0], cl[1], cl[2]}, reach});
    s->dirty_mesh_bs = true;
    s->dirty_bodies = true;
    s->dirty_alloc = true;
    if (body_index) *body_index = (int)s->bodies.size() - 1;
    return XDEM_OK;
}

XDEM_API int xdem_sim_get_mesh(xdem_sim* s, int body_index, device_triangle_info* tri, double* sphere,
                               unsigned int* ntri)
{
    if (!s || body_index < 0 || body_index >= (int)s->bodies.size() || s->bodies[body_index].kind != 1)
        return XDEM_ERR_ARG;
    const SimMesh& m = s->meshes[s->bodies[body_index].index];
    if (ntri) *ntri = m.ntri;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e == cudaSuccess && tri)
        e = cudaMemcpy(tri, s->d_tri + m.first, m.ntri * sizeof(device_triangle_info), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && sphere)
        e = cudaMemcpy(sphere, s->d_sphere + 4 * (size_t)m.first, m.ntri * 4 * sizeof(double), cudaMemcpyDeviceToHost);
    return cerr(e);
}

XDEM_API int xdem_sim_set_body(xdem_sim* s, int body_index, const double body[15], const device_plane_info* plane)
{
    if (!s || body_index < 0 || body_index >= (int)s->bodies.size() || !body) return XDEM_ERR_ARG;
    if (int r = upload_bodies(s)) return r;  // tables sized for every body added so far
    SimBody& b = s->bodies[body_index];
    std::memcpy(b.rec, body, sizeof(b.rec));
    cudaError_t e = cudaMemcpyAsync(s->d_body + 15 * body_index, b.rec, sizeof(b.rec), cudaMemcpyHostToDevice, s->st);
    if (b.kind == 0 && plane) {
        device_plane_info pl = *plane;
        pl.id = s->planes[b.index].id;
        s->planes[b.index] = pl;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_planes + b.index, &s->planes[b.index], sizeof(pl), cudaMemcpyHostToDevice, s->st);
        // the fused step's prefilter and float-pair tables follow the frame
        if (e == cudaSuccess &&
            fused_update_plane(s->fs, (unsigned int)b.index, pl, s->body_cp[body_index].coh != 0.0, s->st) != XDEM_OK)
            e = cudaErrorUnknown;
    }
    if (b.kind == 1 && e == cudaSuccess) {
        // xParticleMeshObjectContact::update -> cu_update_meshObjectData
        const SimMesh& m = s->meshes[b.index];
        e = launch_update_mesh(s->d_body + 15 * body_index, s->d_vlist + 9 * (size_t)m.first,
                               s->d_sphere + 4 * (size_t)m.first, s->d_dlocal + 3 * (size_t)m.first,
                               s->d_tri + m.first, m.ntri, s->st);
        // the fused step: the mesh spheres change cells, so the next step
        // sorts, and the mesh's bounding sphere moves with it
        if (e == cudaSuccess && fused_force_sort(s->fs, s->st) != XDEM_OK) e = cudaErrorUnknown;
        if (e == cudaSuccess && push_mesh_bounds(s, b.index) != XDEM_OK) e = cudaErrorUnknown;
    }
    // the pinned-free host record must stay valid until the copy ran
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    return cerr(e);
}

// Pinned staging of at least `bytes`, with the last upload from it finished.
static int pin_stage(xdem_sim* s, size_t bytes, char** out)
{
    if (!s->pin_ev) {
        if (cudaEventCreateWithFlags(&s->pin_ev, cudaEventDisableTiming) != cudaSuccess) return XDEM_ERR_CUDA;
    } else if (cudaEventSynchronize(s->pin_ev) != cudaSuccess) {
        return XDEM_ERR_CUDA;
    }
    if (bytes > s->h_pin_cap) {
        if (s->h_pin) cudaFreeHost(s->h_pin);
        s->h_pin = nullptr;
        s->h_pin_cap = 0;
        if (cudaHostAlloc(&s->h_pin, bytes, cudaHostAllocDefault) != cudaSuccess) return XDEM_ERR_ALLOC;
        s->h_pin_cap = bytes;
    }
    *out = static_cast<char*>(s->h_pin);
    return XDEM_OK;
}

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

XDEM_API int xdem_sim_set_bodies(xdem_sim* s, int count, const int* body_index, const double* bodies,
                                 const device_plane_info* planes)
{
    if (!s || count < 0 || (count > 0 && (!body_index || !bodies))) return XDEM_ERR_ARG;
    const int nb = (int)s->bodies.size();
    for (int q = 0; q < count; ++q)
        if (body_index[q] < 0 || body_index[q] >= nb) return XDEM_ERR_ARG;
    if (count == 0) return XDEM_OK;
    if (int r = upload_bodies(s)) return r;
    // the host mirrors in list order (a body listed twice keeps its last entry)
    bool moved_plane = false, tables = false;
    for (int q = 0; q < count; ++q) {
        SimBody& b = s->bodies[body_index[q]];
        std::memcpy(b.rec, bodies + 15 * (size_t)q, sizeof(b.rec));
        if (b.kind == 0 && planes) {
            device_plane_info pl = planes[q];
            pl.id = s->planes[b.index].id;
            s->planes[b.index] = pl;
            moved_plane = true;
            tables |= fused_plane_tables_host(s->fs, (unsigned int)b.index, pl, s->body_cp[body_index[q]].coh != 0.0);
        }
    }
    // then every record, and every plane's frame and tables if one moved,
    // in one copy per array
    const size_t npl = s->planes.size(), nft = tables ? s->fs.nplane : 0;
    const size_t ob = 0, op = align16(ob + (size_t)nb * 15 * sizeof(double));
    const size_t of = align16(op + (moved_plane ? npl * sizeof(device_plane_info) : 0));
    const size_t od = align16(of + nft * sizeof(PlaneF));
    const size_t end = od + nft * sizeof(PlaneDF);
    char* h = nullptr;
    if (int r = pin_stage(s, end, &h)) return r;
    for (int i = 0; i < nb; ++i) std::memcpy(h + ob + (size_t)i * 15 * sizeof(double), s->bodies[i].rec, 15 * sizeof(double));
    cudaError_t e = cudaMemcpyAsync(s->d_body, h + ob, (size_t)nb * 15 * sizeof(double), cudaMemcpyHostToDevice, s->st);
    if (moved_plane && npl) {
        std::memcpy(h + op, s->planes.data(), npl * sizeof(device_plane_info));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_planes, h + op, npl * sizeof(device_plane_info), cudaMemcpyHostToDevice, s->st);
    }
    if (nft) {
        std::memcpy(h + of, s->fs.h_planef.data(), nft * sizeof(PlaneF));
        std::memcpy(h + od, s->fs.h_planedf.data(), nft * sizeof(PlaneDF));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->fs.d_planef, h + of, nft * sizeof(PlaneF), cudaMemcpyHostToDevice, s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->fs.d_planedf, h + od, nft * sizeof(PlaneDF), cudaMemcpyHostToDevice, s->st);
    }
    // meshes follow their records as in xdem_sim_set_body
    for (int q = 0; q < count && e == cudaSuccess; ++q) {
        const int bi = body_index[q];
        const SimBody& b = s->bodies[bi];
        if (b.kind != 1) continue;
        const SimMesh& m = s->meshes[b.index];
        e = launch_update_mesh(s->d_body + 15 * bi, s->d_vlist + 9 * (size_t)m.first, s->d_sphere + 4 * (size_t)m.first,
                               s->d_dlocal + 3 * (size_t)m.first, s->d_tri + m.first, m.ntri, s->st);
        if (e == cudaSuccess && fused_force_sort(s->fs, s->st) != XDEM_OK) e = cudaErrorUnknown;
        if (e == cudaSuccess && push_mesh_bounds(s, b.index) != XDEM_OK) e = cudaErrorUnknown;
    }
    if (e == cudaSuccess) e = cudaEventRecord(s->pin_ev, s->st);
    return cerr(e);
}

XDEM_API int xdem_sim_body_wrenches(xdem_sim* s, int count, const int* body_index, double* out)
{
    if (!s || count < 0 || (count > 0 && (!body_index || !out))) return XDEM_ERR_ARG;
    if (s->nscene > 1) return XDEM_ERR_ARG;  // batched handles keep no body wrenches
    const int nb = (int)s->bodies.size();
    for (int q = 0; q < count; ++q)
        if (body_index[q] < 0 || body_index[q] >= nb) return XDEM_ERR_ARG;
    if (count == 0) return XDEM_OK;
    if (!s->wrench || s->dirty_alloc) return XDEM_ERR_ARG;  // no step has run on this body set
    char* h = nullptr;
    if (int r = pin_stage(s, (size_t)nb * 6 * sizeof(double), &h)) return r;
    cudaError_t e = cudaMemcpyAsync(h, s->wrench, (size_t)nb * 6 * sizeof(double), cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return cerr(e);
    for (int q = 0; q < count; ++q)
        std::memcpy(out + 6 * (size_t)q, h + (size_t)body_index[q] * 6 * sizeof(double), 6 * sizeof(double));
    return XDEM_OK;
}

XDEM_API int xdem_sim_step(xdem_sim* s, unsigned int nsteps)
{
    if (!s) return XDEM_ERR_ARG;
    if (s->clusters && !s->xci) return XDEM_ERR_ARG;
    // cylinders in the mixed form: one scene, no cohesion in a cylinder's
    // material (FP64 handles run them on the launcher kernels)
    if (!s->cylinders.empty() && s->precision_mixed()) {
        if (s->nscene > 1) return XDEM_ERR_ARG;
        for (size_t k = 0; k < s->cylinders.size(); ++k)
            if (s->body_cp[s->planes.size() + k].coh != 0.0) return XDEM_ERR_ARG;
    }
    // mixed clusters: the fused step's cluster form (one member count, no
    // rolling resistance or cohesion)
    if (s->clusters && s->precision_mixed()) {
        ClusterTab t;
        if (int r = mixed_cluster_tab(s, t)) return r;
    }
    // a batch needs its planes in place and no meshes (no body wrenches)
    if (s->nscene > 1 && (s->scene_plane_first.back() != s->planes.size() || !s->meshes.empty()))
        return XDEM_ERR_ARG;
    // the graph bakes in the tables' pointers, the body set and the values
    // computed when the step is primed: any of those changing drops it
    if (s->dirty_alloc || s->dirty_bodies || !s->fs.primed) drop_graph(s);
    if (int r = ensure_tables(s)) return r;
    if (int r = upload_bodies(s)) return r;
    if (s->dirty_mesh_bs) {
        for (unsigned int m = 0; m < s->meshes.size(); ++m)
            if (int r = push_mesh_bounds(s, m)) return r;
        s->dirty_mesh_bs = false;
    }
    s->launches = 0;
    if (s->profiling && !s->pe0[0]) {
        for (int i = 0; i < xdem_sim::kProfEvents; ++i) {
            if (cudaEventCreate(&s->pe0[i]) != cudaSuccess || cudaEventCreate(&s->pe1[i]) != cudaSuccess)
                return XDEM_ERR_CUDA;
        }
    }
    unsigned int recorded = 0;
    const bool fused = fused_path(s);
    if (s->use_graph && fused && !s->profiling) {
        // eager steps until the step has been primed, then one graph per
        // arrangement of the double buffers, each replayed with the host
        // side of the step (its swaps) applied by hand
        unsigned int i = 0;
        while (i < nsteps) {
            if (s->fs.primed && s->fs.have_prev) {
                int g = find_graph(s);
                bool captured = false;
                if (g < 0) {
                    g = s->graphs[0].exec ? 1 : 0;
                    if (s->graphs[g].exec) {  // neither arrangement matches: start over
                        drop_graph(s);
                        g = 0;
                    }
                    captured = capture_step_graph(s, g) == XDEM_OK;
                    if (!captured) {
                        if (!s->capture_failed_noted)
                            fprintf(stderr, "xdem_sim_step: the step graph could not be captured; stepping "
                                            "without it\n");
                        s->capture_failed_noted = true;
                        g = -1;
                    }
                }
                if (g >= 0) {
                    const cudaError_t e = cudaGraphLaunch(s->graphs[g].exec, s->st);
                    if (e != cudaSuccess) return cerr(e);
                    // a replay runs no host code: a mixed sphere step wrote
                    // its accelerations to the FP32 copies only
                    if (s->fs.mixed && !s->clusters) s->fs.f64_stale = true;
                    if (!captured) step_swaps(s);
                    s->launches += s->graphs[g].launches;
                    s->cells_clean = true;
                    ++i;
                    continue;
                }
            }
            FusedArgs a = fused_args(s);
            unsigned int nl = 0;
            if (int r = fused_step(s->fs, a, s->st, nullptr, nullptr, &nl)) return r;
            s->launches += nl;
            s->cells_clean = true;
            ++i;
        }
        s->prof_ms = 0.0;
        s->prof_contact_launches = 0;
        s->prof_launches = s->launches;
        return cerr(cudaGetLastError());
    }
    for (unsigned int i = 0; i < nsteps; ++i) {
        int r;
        const bool rec = s->profiling && recorded < (unsigned int)xdem_sim::kProfEvents;
        cudaEvent_t e0 = rec ? s->pe0[recorded] : nullptr, e1 = rec ? s->pe1[recorded] : nullptr;
        if (!fused) {
            r = step_launcher(s, e0, e1);
        } else {
            FusedArgs a = fused_args(s);
            unsigned int nl = 0;
            r = fused_step(s->fs, a, s->st, e0, e1, &nl);
            s->launches += nl;
            s->cells_clean = true;
        }
        if (r) return r;
        if (rec) recorded++;
    }
    double ms_total = 0.0;
    if (recorded) {
        cudaError_t e = cudaEventSynchronize(s->pe1[recorded - 1]);
        for (unsigned int i = 0; e == cudaSuccess && i < recorded; ++i) {
            float ms = 0.f;
            e = cudaEventElapsedTime(&ms, s->pe0[i], s->pe1[i]);
            ms_total += ms;
        }
        if (e != cudaSuccess) return cerr(e);
    }
    s->prof_ms = ms_total;
    s->prof_contact_launches = recorded;
    s->prof_launches = s->launches;
    return cerr(cudaGetLastError());
}

XDEM_API int xdem_sim_body_wrench(xdem_sim* s, int body_index, double out6[6])
{
    if (!s || !out6 || body_index < 0 || body_index >= (int)s->bodies.size()) return XDEM_ERR_ARG;
    if (s->nscene > 1) return XDEM_ERR_ARG;  // batched handles keep no body wrenches
    cudaError_t e = cudaMemcpyAsync(out6, s->wrench + 6 * body_index, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    return cerr(e);
}

XDEM_API int xdem_sim_get_state(xdem_sim* s, double* pos, double* vel, double* acc, double* ep, double* ev,
                                double* ea, double* cpos)
{
    if (!s) return XDEM_ERR_ARG;
    const size_t n = s->np, ns = s->ns;
    // a mixed sphere handle's acc and ea live in FP32 copies between steps
    if (int r = fused_sync_fp64(s->fs, s->acc, s->ea, s->st)) return r;
    cudaError_t e = cudaStreamSynchronize(s->st);
    auto D = [&](double* h, const double* d, size_t cnt) {
        if (e == cudaSuccess && h && d) e = cudaMemcpy(h, d, cnt * sizeof(double), cudaMemcpyDeviceToHost);
    };
    D(pos, s->pos, n * 4); D(vel, s->vel, ns * 3); D(acc, s->acc, ns * 3); D(ep, s->ep, ns * 4);
    D(ev, s->ev, ns * 4); D(ea, s->ea, ns * 4);
    if (s->clusters) D(cpos, s->cpos, ns * 4);
    return cerr(e);
}

XDEM_API int xdem_sim_get_pairs(xdem_sim* s, int kind, unsigned int* count, unsigned int* ids, double* tsd)
{
    if (!s || kind < 0 || kind > 3) return XDEM_ERR_ARG;
    const size_t n = s->np;
    const PairTables t = pair_tables(s, kind);
    const unsigned int cap = t.cap;
    const unsigned int* dc = t.count;
    const unsigned int* di = t.id;
    const double* dt = t.tsd;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e == cudaSuccess && count) e = cudaMemcpy(count, dc, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && ids) e = cudaMemcpy(ids, di, n * 4 * cap, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && tsd) {
        if (kind == 0 && pp_history_f32(s)) {
            std::vector<float> f(n * cap * 2);
            e = cudaMemcpy(f.data(), dt, f.size() * sizeof(float), cudaMemcpyDeviceToHost);
            for (size_t i = 0; i < f.size(); ++i) tsd[i] = (double)f[i];
        } else {
            e = cudaMemcpy(tsd, dt, n * 16 * cap, cudaMemcpyDeviceToHost);
        }
    }
    return cerr(e);
}

// Lists from a file or a caller are checked before anything reaches the
// device: no count above the slot capacity, and every stored id names
// something the handle has -- a particle (kind 0), a plane (1), a triangle
// (2), a cylinder or its inner cap, id + 1000 (3).  Kernels that look a
// partner up by its id (the adjoint's gather) then never index out of range.
int sim_check_pairs(const xdem_sim* s, int kind, const unsigned int* count, const unsigned int* ids)
{
    if (!s || kind < 0 || kind > 3 || !count || !ids) return XDEM_ERR_ARG;
    const unsigned int cap = kind == 0 ? MAX_P2P_COUNT : kind == 1 ? MAX_P2PL_COUNT
                           : kind == 2 ? MAX_P2MS_COUNT : MAX_P2CY_COUNT;
    const unsigned int ncyl = (unsigned int)s->cylinders.size();
    for (size_t i = 0; i < s->np; ++i) {
        if (count[i] > cap) return XDEM_ERR_ARG;
        for (unsigned int k = 0; k < count[i]; ++k) {
            const unsigned int id = ids[i * cap + k];
            bool ok;
            switch (kind) {
            case 0: ok = id < s->np; break;
            case 1: ok = id < s->planes.size(); break;
            case 2: ok = id < s->ntri_total; break;
            default: ok = id < ncyl || (id >= 1000u && id - 1000u < ncyl); break;
            }
            if (!ok) return XDEM_ERR_ARG;
        }
    }
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_pairs(xdem_sim* s, int kind, const unsigned int* count, const unsigned int* ids,
                                const double* tsd)
{
    if (!s || kind < 0 || kind > 3 || !count || !ids || !tsd) return XDEM_ERR_ARG;
    const size_t n = s->np;
    const PairTables t = pair_tables(s, kind);
    const unsigned int cap = t.cap;
    if (int r = sim_check_pairs(s, kind, count, ids)) return r;
    unsigned int* dc = t.count;
    unsigned int* di = t.id;
    double* dt = t.tsd;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e == cudaSuccess) e = cudaMemcpy(dc, count, n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(di, ids, n * 4 * cap, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (kind == 0 && pp_history_f32(s)) {
            // rounded to nearest, as the mixed kernels round a double history
            std::vector<float> f(n * cap * 2);
            for (size_t i = 0; i < f.size(); ++i) f[i] = (float)tsd[i];
            e = cudaMemcpy(dt, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
        } else {
            e = cudaMemcpy(dt, tsd, n * 16 * cap, cudaMemcpyHostToDevice);
        }
    }
    fused_invalidate(s->fs);
    return cerr(e);
}

XDEM_API int xdem_sim_energy(xdem_sim* s, double* ke, unsigned int* ncontact)
{
    if (!s) return XDEM_ERR_ARG;
    double k = 0.0;
    unsigned int c = 0;
    if (int r = ensure_tables(s)) return r;
    int r = fused_energy(s->fs, s->vel, s->ep, s->ev, s->mass, s->inertia, s->ns, s->pp_count, s->pl_count,
                         s->ms_count, s->np, &k, &c, s->st);
    if (ke) *ke = k;
    if (ncontact) *ncontact = c;
    return r;
}

XDEM_API int xdem_sim_status(xdem_sim* s)
{
    if (!s) return XDEM_ERR_ARG;
    unsigned int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, s->d_status, 4, cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_status, 0, 4, s->st);
    if (e != cudaSuccess) return XDEM_ERR_CUDA;
    return (int)h;
}

XDEM_API int xdem_sim_set_profiling(xdem_sim* s, int on)
{
    if (!s) return XDEM_ERR_ARG;
    s->profiling = on != 0;
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_graph(xdem_sim* s, int on)
{
    if (!s) return XDEM_ERR_ARG;
    s->use_graph = on != 0;
    if (!s->use_graph) drop_graph(s);
    return XDEM_OK;
}

XDEM_API int xdem_sim_set_persistent(xdem_sim* s, int on, unsigned long long barrier_limit_ns)
{
    if (!s) return XDEM_ERR_ARG;
    s->fs.persist = on != 0;
    s->fs.persist_limit_ns = barrier_limit_ns ? barrier_limit_ns : 1000000000ull;
    drop_graph(s);  // the captured steps bake in the launches and the limit
    return XDEM_OK;
}

XDEM_API int xdem_sim_profile(xdem_sim* s, unsigned int* launches, double* contact_ms, unsigned int* contact_launches)
{
    if (!s) return XDEM_ERR_ARG;
    if (launches) *launches = s->prof_launches;
    if (contact_ms) *contact_ms = s->prof_ms;
    if (contact_launches) *contact_launches = s->prof_contact_launches;
    return XDEM_OK;
}

}  // extern "C"
