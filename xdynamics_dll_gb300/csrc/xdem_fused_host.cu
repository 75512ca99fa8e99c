// xdem_fused_host.cu -- driver of the fused sorted-order step and its
// small kernels (prologue, reorder + snapshot, per-body wrench sums, energy).
// Compiled with -fmad=false like the other FP64 units: the prologue's
// position update and hash round exactly as impl:135-147 / 290-302 do in the
// CPU oracle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "xdem_device.cuh"
#include "xdem_df.cuh"
#include "xdem_fused.h"
#include "xdem_kernels.h"

namespace xdem {

namespace {

template <class T>
cudaError_t dalloc(T*& p, size_t n)
{
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T));
}

// FP32 snapshot record of one sphere for the mixed contact kernel: offset of
// the centre from its cell corner and radius as float pairs (A + L), packed
// cell, velocity, mass, spin.
__device__ __forceinline__ int3v mixed_record(const device_dem_parameters& p, double inv_cs, d3 x, double r, d3 v,
                                              double m, d3 w, float4& A, float4& L, float4& B, float4& C,
                                              unsigned int& T)
{
    const double rx = x.x - p.world_origin.x, ry = x.y - p.world_origin.y, rz = x.z - p.world_origin.z;
    const double fx = floor(rx * inv_cs), fy = floor(ry * inv_cs), fz = floor(rz * inv_cs);
    const double ox = rx - fx * p.cell_size, oy = ry - fy * p.cell_size, oz = rz - fz * p.cell_size;
    A = make_float4((float)ox, (float)oy, (float)oz, (float)r);
    L = make_float4((float)(ox - (double)A.x), (float)(oy - (double)A.y), (float)(oz - (double)A.z),
                    (float)(r - (double)A.w));
    B = make_float4((float)v.x, (float)v.y, (float)v.z, (float)m);
    C = make_float4((float)w.x, (float)w.y, (float)w.z, 0.f);
    const int3v g{__double2int_rz(fx), __double2int_rz(fy), __double2int_rz(fz)};
    T = pack_cell(g.x, g.y, g.z);
    return g;
}

// Position update of the first step (impl:135-147) into the alternate
// buffers, and the cell hash of the new position (impl:290-302).  For the
// mixed form also the FP32 record of the first step.
__global__ void k_prologue(device_dem_parameters p, const double* pos, const double* ep, const double* vel,
                           const double* ev, const double* acc, const double* ea, const double* mass,
                           double* pos_next, double* ep_next, unsigned int* key, unsigned int* val, unsigned int n,
                           unsigned int* status, float4* rec)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = p.dt, h = p.half2dt;
    const d4 e = (ld4(ep, i) + dt * ld4(ev, i)) + h * ld4(ea, i);
    const double l = sqrt(dot(e, e));
    const d4 en = mk4(e.x / l, e.y / l, e.z / l, e.w / l);
    st4(ep_next, i, en);
    const d3 v = ld3(vel, i);
    const d3 d = dt * v + h * ld3(acc, i);
    const d4 q = ld4(pos, i);
    const d3 x = mk3(q.x + d.x, q.y + d.y, q.z + d.z);
    st4(pos_next, i, mk4(x.x, x.y, x.z, q.w));
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(status, (unsigned int)XDEM_ERR_NONFINITE);
    int3v g;
    if (rec) {
        // mixed form: the key's cell is the cell the FP32 record is relative to
        float4 A, L, B, C;
        unsigned int T;
        g = mixed_record(p, 1.0 / p.cell_size, x, q.w, v, mass[i], ang_vel(en, ld4(ev, i)), A, L, B, C, T);
        C.w = __uint_as_float(T);
        rec[4 * (size_t)i + kRecA] = A;
        rec[4 * (size_t)i + kRecL] = L;
        rec[4 * (size_t)i + kRecB] = B;
        rec[4 * (size_t)i + kRecC] = C;
    } else {
        g = grid_pos(p, x);
    }
    key[i] = grid_hash(p, g.x, g.y, g.z);
    val[i] = i;
}

// Position update of the first step for clusters (impl:149-190): centre and
// Euler parameters into the alternate buffers, member centres x_c + A(e)
// rloc, and the members' FP32 records and cell hashes.  A member's record
// carries its cluster's mass and spin and the cluster's velocity at the
// member's centre, v + w x (x_m - x_c): the velocity of a contact point at
// x is then the record's velocity + w x (x - x_m), as impl:485-611 forms it
// from the cluster centre.
__global__ void k_prologue_cluster(device_dem_parameters p, ClusterTab t, const double* cpos, const double* ep,
                                   const double* vel, const double* ev, const double* acc, const double* ea,
                                   const double* mass, const double* rloc, const double* pos, double* cpos_next,
                                   double* ep_next, double* pos_next, unsigned int* key, unsigned int* val,
                                   unsigned int* status, float4* rec)
{
    const unsigned int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= t.ns) return;
    const double dt = p.dt, h = p.half2dt;
    const d4 cp = ld4(cpos, c);
    const d3 x = (mk3(cp.x, cp.y, cp.z) + dt * ld3(vel, c)) + h * ld3(acc, c);
    st4(cpos_next, c, mk4(x.x, x.y, x.z, cp.w));
    const d4 w = ld4(ev, c);
    const d4 e = (ld4(ep, c) + dt * w) + h * ld4(ea, c);
    const double l = sqrt(dot(e, e));
    const d4 en = mk4(e.x / l, e.y / l, e.z / l, e.w / l);
    st4(ep_next, c, en);
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(status, (unsigned int)XDEM_ERR_NONFINITE);
    const d3 v = ld3(vel, c);
    const d3 om = ang_vel(en, w);
    const double m = mass[c];
    const unsigned int type = cluster_type(t, c);
    for (unsigned int j = 0; j < t.neach; ++j) {
        const size_t i = (size_t)c * t.neach + j;
        const d3 d = to_global(ld3(rloc, (size_t)type * t.neach + j), en);
        const d3 xm = x + d;
        const double r = pos[4 * i + 3];
        st4(pos_next, i, mk4(xm.x, xm.y, xm.z, r));
        float4 A, L, B, C;
        unsigned int T;
        const int3v g = mixed_record(p, 1.0 / p.cell_size, xm, r, v + cross(om, d), m, om, A, L, B, C, T);
        C.w = __uint_as_float(T);
        rec[4 * i + kRecA] = A;
        rec[4 * i + kRecL] = L;
        rec[4 * i + kRecB] = B;
        rec[4 * i + kRecC] = C;
        key[i] = grid_hash(p, g.x, g.y, g.z);
        val[i] = (unsigned int)i;
    }
}

// Bounding box of the positions: block min/max into out[block*6].
__global__ void k_bbox(const double* pos, unsigned int n, double* out)
{
    __shared__ double sm[6][32];
    double v[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const d3 q = ld4xyz(pos, i);
        if (!(isfinite(q.x) && isfinite(q.y) && isfinite(q.z))) continue;
        v[0] = fmin(v[0], q.x); v[1] = fmin(v[1], q.y); v[2] = fmin(v[2], q.z);
        v[3] = fmax(v[3], q.x); v[4] = fmax(v[4], q.y); v[5] = fmax(v[5], q.z);
    }
    for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_down_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? fmin(v[c], w) : fmax(v[c], w);
        }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int c = 0; c < 6; ++c) sm[c][warp] = v[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            for (int c = 0; c < 6; ++c) v[c] = c < 3 ? fmin(v[c], sm[c][w]) : fmax(v[c], sm[c][w]);
        for (int c = 0; c < 6; ++c) out[blockIdx.x * 6 + c] = v[c];
    }
}

// FP64 form: cell ranges of the sorted keys (impl:317-360) and the sorted
// FP64 snapshot, plus an FP32 copy of the position relative to the grid
// origin for the prefilter.
__global__ void k_reorder_fp64(const unsigned int* sk, const unsigned int* sv, unsigned int n, unsigned int np,
                               unsigned int* cstart, unsigned int* cend, unsigned int* sorted_index,
                               unsigned int* skey, const double* pos, const double* ep, const double* vel,
                               const double* ev, const double* mass, double* snap_pos, double* snap_vel,
                               double* snap_om, float* snap_f, double ox, double oy, double oz, double far2)
{
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const unsigned int k = sk[s];
    cell_bounds(sk, s, n, cstart, cend, k);
    const unsigned int oid = sv[s];
    sorted_index[s] = oid;
    skey[s] = k;
    float4 f = make_float4(0.f, 0.f, 0.f, -1.f);
    if (oid < np) {
        const d4 x = ld4(pos, oid);
        const d3 v = ld3(vel, oid);
        const d3 w = ang_vel(ld4(ep, oid), ld4(ev, oid));
        st4(snap_pos, s, x);
        st4(snap_vel, s, mk4(v.x, v.y, v.z, mass[oid]));
        st4(snap_om, s, mk4(w.x, w.y, w.z, 0.0));
        const double dx = x.x - ox, dy = x.y - oy, dz = x.z - oz;
        if (dx * dx + dy * dy + dz * dz < far2) f = make_float4((float)dx, (float)dy, (float)dz, (float)x.w);
    }
    reinterpret_cast<float4*>(snap_f)[s] = f;
}

// Condition of the captured step's IF node around the gated clear, sort and
// reorder: the gate (rebuild this step, or a list overflowed).
__global__ void k_set_sort_cond(cudaGraphConditionalHandle h, const unsigned int* gate)
{
    cudaGraphSetConditional(h, *gate ? 1u : 0u);
}

// Mixed form: cell ranges and the FP32 records permuted into sorted order.
__global__ void k_reorder_mixed(const unsigned int* gate, const unsigned int* sk, const unsigned int* sv,
                                unsigned int n, unsigned int np,
                                unsigned int* cstart, unsigned int* cend, unsigned int* sorted_index,
                                unsigned int* skey, const float4* rec, float4* mA, float4* mL, float4* mB,
                                float4* mC, uint2* mIT)
{
    if (gate && !*gate) return;
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    reorder_mixed_entry(s, sk, sv, n, np, cstart, cend, sorted_index, skey, rec, mA, mL, mB, mC, mIT);
}

// Sum of the contact kernel's per-block wrench partials, kWrenchChunks
// blocks of 256 threads per body: each block sums one contiguous chunk of
// partial rows (6 doubles a row, read whole, so a warp reads contiguous
// memory), the last block of a body to finish adds the chunk sums in chunk
// order.  The order of every addition is fixed: the result does not depend
// on which block finishes last.
__global__ void k_body_sums(const double* bsums, unsigned int nblocks, unsigned int nrow_plane_bodies,
                            unsigned int rows_plane, unsigned int rows_mesh, double* wrench, double* chunk,
                            unsigned int* done)
{
    __shared__ double sm[8 * 6];
    __shared__ bool last;
    const unsigned int b = blockIdx.x / kWrenchChunks, q = blockIdx.x % kWrenchChunks;
    // rows of body b, written by the kernel that does its contacts: the
    // body kernel for planes and cylinders (the first nrow_plane_bodies
    // bodies), the pair kernel for meshes; nblocks is the row stride
    const unsigned int rows = b < nrow_plane_bodies ? rows_plane : rows_mesh;
    const unsigned int per = (rows + kWrenchChunks - 1) / kWrenchChunks;
    const unsigned int i0 = q * per, i1 = min(rows, i0 + per);
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (unsigned int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double* r = bsums + ((size_t)b * nblocks + i) * 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] += r[c];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
        if ((threadIdx.x & 31) == 0) sm[(threadIdx.x >> 5) * 6 + c] = s[c];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += sm[w * 6 + threadIdx.x];
        chunk[((size_t)b * kWrenchChunks + q) * 6 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done + b, 1u) == kWrenchChunks - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (unsigned int k = 0; k < kWrenchChunks; ++k)
            t += __ldcg(chunk + ((size_t)b * kWrenchChunks + k) * 6 + threadIdx.x);
        wrench[b * 6 + threadIdx.x] = t;
    }
    if (threadIdx.x == 0) done[b] = 0u;  // ready for the next step
}

__global__ void k_energy(const double* vel, const double* ep, const double* ev, const double* mass,
                         const double* inertia, unsigned int ns, const unsigned int* c0, const unsigned int* c1,
                         const unsigned int* c2, unsigned int np, double* out_ke, unsigned int* out_c)
{
    double ke = 0.0;
    unsigned int cnt = 0;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const d3 v = ld3(vel, i);
        const d4 e = ld4(ep, i), d = ld4(ev, i);
        // body-frame angular velocity 2 L(e) e_dot (L rows of impl:77-79)
        const double w0 = 2.0 * (-e.y * d.x + e.x * d.y + e.w * d.z - e.z * d.w);
        const double w1 = 2.0 * (-e.z * d.x - e.w * d.y + e.x * d.z + e.y * d.w);
        const double w2 = 2.0 * (-e.w * d.x + e.z * d.y - e.y * d.z + e.x * d.w);
        const d3 J = ld3(inertia, i);
        ke += 0.5 * mass[i] * dot(v, v) + 0.5 * (J.x * w0 * w0 + J.y * w1 * w1 + J.z * w2 * w2);
    }
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
        cnt += c0[i] + c1[i] + c2[i];
    for (int o = 16; o > 0; o >>= 1) {
        ke += __shfl_down_sync(0xffffffffu, ke, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out_ke, ke);
        atomicAdd(out_c, cnt);
    }
}

// Kinetic energy and stored contacts per scene of a batch: one block per
// scene over its particle range [first[s], first[s + 1]) (free spheres).
__global__ void k_scene_energy(const double* vel, const double* ep, const double* ev, const double* mass,
                               const double* inertia, const unsigned int* first, const unsigned int* c0,
                               const unsigned int* c1, double* out)
{
    __shared__ double sk[8];
    __shared__ unsigned int sc[8];
    const unsigned int s = blockIdx.x;
    double ke = 0.0;
    unsigned int cnt = 0;
    for (unsigned int i = first[s] + threadIdx.x; i < first[s + 1]; i += blockDim.x) {
        const d3 v = ld3(vel, i);
        const d4 e = ld4(ep, i), d = ld4(ev, i);
        const double w0 = 2.0 * (-e.y * d.x + e.x * d.y + e.w * d.z - e.z * d.w);
        const double w1 = 2.0 * (-e.z * d.x - e.w * d.y + e.x * d.z + e.y * d.w);
        const double w2 = 2.0 * (-e.w * d.x + e.z * d.y - e.y * d.z + e.x * d.w);
        const d3 J = ld3(inertia, i);
        ke += 0.5 * mass[i] * dot(v, v) + 0.5 * (J.x * w0 * w0 + J.y * w1 * w1 + J.z * w2 * w2);
        cnt += c0[i] + c1[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        ke += __shfl_down_sync(0xffffffffu, ke, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sk[threadIdx.x >> 5] = ke;
        sc[threadIdx.x >> 5] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double k = 0.0;
        unsigned int n = 0;
        for (unsigned int w = 0; w < (blockDim.x >> 5); ++w) {
            k += sk[w];
            n += sc[w];
        }
        out[2 * s] = k;
        out[2 * s + 1] = (double)n;
    }
}

}  // namespace

int fused_scene_energy(const double* vel, const double* ep, const double* ev, const double* mass,
                       const double* inertia, const unsigned int* d_first, unsigned int nscene, const unsigned int* c0,
                       const unsigned int* c1, double* d_out, double* ke, unsigned int* ncontact, cudaStream_t st)
{
    if (!nscene) return XDEM_OK;
    k_scene_energy<<<nscene, 256, 0, st>>>(vel, ep, ev, mass, inertia, d_first, c0, c1, d_out);
    cudaError_t e = cudaGetLastError();
    std::vector<double> h((size_t)nscene * 2);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return XDEM_ERR_CUDA;
    for (unsigned int s = 0; s < nscene; ++s) {
        if (ke) ke[s] = h[2 * s];
        if (ncontact) ncontact[s] = (unsigned int)h[2 * s + 1];
    }
    return XDEM_OK;
}

int fused_alloc(FusedState& fs, unsigned int np, unsigned int nentry, bool mixed, cudaStream_t st, unsigned int ns)
{
    fs.mixed = mixed;
    fs.np = np;
    fs.nentry = nentry;
    cudaError_t e = dalloc(fs.pos_alt, (size_t)np * 4);
    if (e == cudaSuccess) e = dalloc(fs.ep_alt, (size_t)np * 4);
    if (e == cudaSuccess && ns) e = dalloc(fs.cpos_alt, (size_t)ns * 4);
    if (mixed) {
        if (e == cudaSuccess) e = dalloc(fs.mA, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.mL, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.mB, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.mC, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.mIT, (size_t)nentry * 2);
        if (e == cudaSuccess) e = dalloc(fs.rec, (size_t)np * 4);
        if (e == cudaSuccess) e = dalloc(fs.accf, np);
        if (e == cudaSuccess) e = dalloc(fs.eaf, np);
        if (e == cudaSuccess) e = dalloc(fs.jm, np);
        fs.f32_ready = fs.f64_stale = false;
        if (e == cudaSuccess) e = dalloc(fs.fA, (size_t)np * 4);
        if (e == cudaSuccess) e = dalloc(fs.fB, (size_t)np * 4);
        if (e == cudaSuccess) e = dalloc(fs.fC, (size_t)np * 4);

        if (e == cudaSuccess && !fs.side_st) e = cudaStreamCreateWithFlags(&fs.side_st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = dalloc(fs.vl_ids, (size_t)np * kListCap);
        if (e == cudaSuccess) e = dalloc(fs.vl_cnt, np);
        if (e == cudaSuccess) e = dalloc(fs.vl_xb, (size_t)np * 4);
        if (e == cudaSuccess) e = dalloc(fs.vl_flag, kVlWords);
        if (e == cudaSuccess) e = dalloc(fs.d_bar, 2);
        if (e == cudaSuccess) e = cudaMemsetAsync(fs.vl_flag, 0, kVlWords * sizeof(unsigned int), st);
        // until the handle sets them, every mesh is searched by every sphere
        for (unsigned int m = 0; m < kMaxFusedMeshes; ++m) fs.h_mesh_bs[m] = make_float4(0.f, 0.f, 0.f, 1e18f);
        if (e == cudaSuccess) e = dalloc(fs.d_mesh_bs, kMaxFusedMeshes);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(fs.d_mesh_bs, fs.h_mesh_bs, sizeof(fs.h_mesh_bs), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } else {
        if (e == cudaSuccess) e = dalloc(fs.snap_pos, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.snap_vel, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.snap_om, (size_t)nentry * 4);
        if (e == cudaSuccess) e = dalloc(fs.snap_f, (size_t)nentry * 4);
    }
    if (e == cudaSuccess) e = dalloc(fs.pp_count2, np);
    if (e == cudaSuccess) e = dalloc(fs.pp_id2, (size_t)np * MAX_P2P_COUNT);
    if (e == cudaSuccess) e = dalloc(fs.pp_tsd2, (size_t)np * MAX_P2P_COUNT * 2);
    if (e == cudaSuccess) e = dalloc(fs.skey_prev, nentry);
    if (e == cudaSuccess) e = dalloc(fs.d_energy, 2);
    if (e == cudaSuccess) e = dalloc(fs.d_bbox, (size_t)kBboxBlocks * 6);
    if (e == cudaSuccess) e = cudaMemsetAsync(fs.pp_count2, 0, np * sizeof(unsigned int), st);
    fs.primed = false;
    fs.have_prev = false;
    return e == cudaSuccess ? XDEM_OK : XDEM_ERR_ALLOC;
}

void fused_free(FusedState& fs)
{
    void* ps[] = {fs.pos_alt, fs.ep_alt, fs.cpos_alt, fs.snap_pos, fs.snap_vel, fs.snap_om, fs.snap_f, fs.mA, fs.mL, fs.mB,
                  fs.mC, fs.mIT, fs.rec, fs.accf, fs.eaf, fs.jm, fs.fA, fs.fB, fs.fC, fs.pp_count2, fs.pp_id2,
                  fs.pp_tsd2, fs.vl_ids, fs.vl_cnt, fs.vl_xb, fs.vl_flag, fs.d_bar,
                  fs.skey_prev, fs.d_energy, fs.d_bbox, fs.d_planef, fs.d_planedf, fs.d_mpf, fs.wsum, fs.wcnt,
                  fs.d_mesh_bs};
    for (void* q : ps)
        if (q) cudaFree(q);
    if (fs.side_st) cudaStreamDestroy(fs.side_st);
    fs = FusedState{};
}

void fused_invalidate(FusedState& fs) { fs.primed = false; }

void fused_state_written(FusedState& fs)
{
    fs.primed = false;
    fs.f32_ready = false;
    fs.f64_stale = false;
}

namespace {

// FP64 state -> FP32 copies of a mixed sphere handle (d2f_rn, as the body
// kernel rounds them when it reads the FP64 arrays).
__global__ void k_state_to_f32(const double* acc, const double* ea, const double* inertia, const double* mass,
                               float4* accf, float4* eaf, float4* jm, unsigned int n)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    accf[i] = make_float4(d2f_rn(acc[3 * (size_t)i]), d2f_rn(acc[3 * (size_t)i + 1]), d2f_rn(acc[3 * (size_t)i + 2]),
                          0.f);
    eaf[i] = make_float4(d2f_rn(ea[4 * (size_t)i]), d2f_rn(ea[4 * (size_t)i + 1]), d2f_rn(ea[4 * (size_t)i + 2]),
                         d2f_rn(ea[4 * (size_t)i + 3]));
    jm[i] = make_float4(d2f_rn(inertia[3 * (size_t)i]), d2f_rn(inertia[3 * (size_t)i + 1]),
                        d2f_rn(inertia[3 * (size_t)i + 2]), d2f_rn(mass[i]));
}

// FP32 copies -> FP64 acc and ea (exact).
__global__ void k_state_to_f64(const float4* accf, const float4* eaf, double* acc, double* ea, unsigned int n)
{
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = accf[i], q = eaf[i];
    acc[3 * (size_t)i] = f2d(a.x); acc[3 * (size_t)i + 1] = f2d(a.y); acc[3 * (size_t)i + 2] = f2d(a.z);
    ea[4 * (size_t)i] = f2d(q.x); ea[4 * (size_t)i + 1] = f2d(q.y); ea[4 * (size_t)i + 2] = f2d(q.z);
    ea[4 * (size_t)i + 3] = f2d(q.w);
}

// A conversion must not land in a step graph: it is a host decision of one
// step, not part of every replay.
bool capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

}  // namespace

int fused_sync_fp64(FusedState& fs, double* acc, double* ea, cudaStream_t st)
{
    if (!fs.f64_stale) return XDEM_OK;
    if (capturing(st)) return XDEM_ERR_ARG;
    k_state_to_f64<<<blocks_for(fs.np), kThreads, 0, st>>>(fs.accf, fs.eaf, acc, ea, fs.np);
    if (cudaGetLastError() != cudaSuccess) return XDEM_ERR_CUDA;
    fs.f64_stale = false;
    return XDEM_OK;
}

namespace {

void split_host(double x, float& hi, float& lo)
{
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// Prefilter and float-pair tables of one plane.
void plane_tables(const device_plane_info& pl, const double origin[3], bool coh, PlaneF& pf, PlaneDF& pd)
{
    const double xw[3] = {pl.xw.x, pl.xw.y, pl.xw.z};
    const double u1[3] = {pl.u1.x, pl.u1.y, pl.u1.z}, u2[3] = {pl.u2.x, pl.u2.y, pl.u2.z};
    const double uw[3] = {pl.uw.x, pl.uw.y, pl.uw.z};
    const double lw = std::sqrt(uw[0] * uw[0] + uw[1] * uw[1] + uw[2] * uw[2]);
    float* v = pf.v;
    for (int i = 0; i < 3; ++i) {
        v[i] = (float)(xw[i] - origin[i]);
        v[3 + i] = (float)u1[i];
        v[6 + i] = (float)u2[i];
        v[9 + i] = (float)(uw[i] / lw);
    }
    v[12] = (float)pl.l1; v[13] = (float)pl.l2; v[14] = 0.f; v[15] = 0.f;

    pd = PlaneDF{};
    for (int i = 0; i < 3; ++i) {
        split_host(xw[i], pd.xw_hi[i], pd.xw_lo[i]);
        split_host(u1[i], pd.u_hi[i], pd.u_lo[i]);
        split_host(u2[i], pd.u_hi[3 + i], pd.u_lo[3 + i]);
        split_host(uw[i], pd.u_hi[6 + i], pd.u_lo[6 + i]);
    }
    split_host(pl.l1, pd.l1_hi, pd.l1_lo);
    split_host(pl.l2, pd.l2_hi, pd.l2_lo);
    // orthonormal rectangle: the local-coordinate contact test applies
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    const double cr[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2], u1[0] * u2[1] - u1[1] * u2[0]};
    const double tol = 1e-12;
    bool rect = std::fabs(dot(u1, u1) - 1.0) < tol && std::fabs(dot(u2, u2) - 1.0) < tol &&
                std::fabs(dot(uw, uw) - 1.0) < tol && std::fabs(dot(u1, u2)) < tol;
    for (int i = 0; i < 3; ++i) rect = rect && std::fabs(uw[i] - cr[i]) < tol;
    const double w2[3] = {pl.w2.x, pl.w2.y, pl.w2.z}, w3[3] = {pl.w3.x, pl.w3.y, pl.w3.z};
    const double w4[3] = {pl.w4.x, pl.w4.y, pl.w4.z};
    const double scale = std::fabs(xw[0]) + std::fabs(xw[1]) + std::fabs(xw[2]) + pl.l1 + pl.l2 + 1.0;
    for (int i = 0; i < 3; ++i) {
        rect = rect && std::fabs(w2[i] - (xw[i] + pl.l1 * u1[i])) < tol * scale;
        rect = rect && std::fabs(w4[i] - (xw[i] + pl.l2 * u2[i])) < tol * scale;
        rect = rect && std::fabs(w3[i] - (xw[i] + pl.l1 * u1[i] + pl.l2 * u2[i])) < tol * scale;
    }
    pd.rect = rect ? 1 : 0;
    pd.coh = coh ? 1 : 0;
}

}  // namespace

int fused_set_bodies(FusedState& fs, const device_plane_info* planes, unsigned int nplane, const double* body,
                     const mat_pair* mp, const device_plane_info* host_planes, const mat_pair* host_mp,
                     unsigned int nmp, unsigned int nscene, const double origin[3], cudaStream_t st)
{
    fs.planes = planes;
    fs.nplane = nplane;
    fs.body = body;
    fs.mp = mp;
    for (int i = 0; i < 3; ++i) fs.origin[i] = origin[i];
    if (nmp < nscene + nplane) return XDEM_ERR_ARG;
    const unsigned int nbody = nmp - nscene;
    if (nbody > fs.wsum_cap) {
        if (dalloc(fs.wsum, (size_t)nbody * kWrenchChunks * 6) != cudaSuccess || dalloc(fs.wcnt, nbody) != cudaSuccess)
            return XDEM_ERR_ALLOC;
        if (cudaMemsetAsync(fs.wcnt, 0, nbody * sizeof(unsigned int), st) != cudaSuccess) return XDEM_ERR_CUDA;
        fs.wsum_cap = nbody;
    }
    if (nmp > fs.mpf_cap) {
        if (dalloc(fs.d_mpf, nmp) != cudaSuccess) return XDEM_ERR_ALLOC;
        fs.mpf_cap = nmp;
    }
    std::vector<MatF> mf(nmp);
    fs.any_coh = false;
    for (unsigned int i = 0; i < nscene && i < nmp; ++i) fs.any_coh = fs.any_coh || host_mp[i].coh != 0.0;
    for (unsigned int i = 0; i < nmp; ++i) {
        const mat_pair& m = host_mp[i];
        mf[i] = MatF{(float)m.Eeq, (float)m.Seq8, (float)m.beta, (float)m.vs1, (float)m.sratio, (float)m.fric,
                     (float)m.rfric, m.coh != 0.0 ? 1 : 0};
    }
    if (nmp) {
        cudaError_t e = cudaMemcpyAsync(fs.d_mpf, mf.data(), nmp * sizeof(MatF), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return XDEM_ERR_CUDA;
    }
    if (!nplane) return XDEM_OK;
    if (nplane > fs.plane_cap) {
        if (dalloc(fs.d_planef, nplane) != cudaSuccess || dalloc(fs.d_planedf, nplane) != cudaSuccess)
            return XDEM_ERR_ALLOC;
        fs.plane_cap = nplane;
    }
    fs.h_planef.assign(nplane, PlaneF{});
    fs.h_planedf.assign(nplane, PlaneDF{});
    for (unsigned int k = 0; k < nplane; ++k)
        plane_tables(host_planes[k], origin, host_mp[nscene + k].coh != 0.0, fs.h_planef[k], fs.h_planedf[k]);
    cudaError_t e =
        cudaMemcpyAsync(fs.d_planef, fs.h_planef.data(), nplane * sizeof(PlaneF), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(fs.d_planedf, fs.h_planedf.data(), nplane * sizeof(PlaneDF), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? XDEM_OK : XDEM_ERR_CUDA;
}

bool fused_plane_tables_host(FusedState& fs, unsigned int k, const device_plane_info& host_plane, bool coh)
{
    if (k >= fs.nplane || !fs.d_planef || !fs.d_planedf) return false;
    plane_tables(host_plane, fs.origin, coh, fs.h_planef[k], fs.h_planedf[k]);
    return true;
}

int fused_update_plane(FusedState& fs, unsigned int k, const device_plane_info& host_plane, bool coh,
                       cudaStream_t st)
{
    if (k >= fs.nplane || !fs.d_planef || !fs.d_planedf) return XDEM_OK;  // tables not built yet
    plane_tables(host_plane, fs.origin, coh, fs.h_planef[k], fs.h_planedf[k]);
    cudaError_t e = cudaMemcpyAsync(fs.d_planef + k, &fs.h_planef[k], sizeof(PlaneF), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(fs.d_planedf + k, &fs.h_planedf[k], sizeof(PlaneDF), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? XDEM_OK : XDEM_ERR_CUDA;
}

int fused_set_mesh_bounds(FusedState& fs, unsigned int m, float4 b, cudaStream_t st)
{
    if (m >= kMaxFusedMeshes || !fs.d_mesh_bs) return XDEM_OK;  // tables not built yet
    fs.h_mesh_bs[m] = b;
    const cudaError_t e =
        cudaMemcpyAsync(fs.d_mesh_bs + m, &fs.h_mesh_bs[m], sizeof(float4), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? XDEM_OK : XDEM_ERR_CUDA;
}

int fused_force_sort(FusedState& fs, cudaStream_t st)
{
    if (!fs.vl_flag) return XDEM_OK;
    return cudaMemsetAsync(fs.vl_flag + kVlSort, 1, sizeof(unsigned int), st) == cudaSuccess ? XDEM_OK
                                                                                          : XDEM_ERR_CUDA;
}

int fused_step(FusedState& fs, FusedArgs& a, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, unsigned int* nlaunch)
{
    cudaError_t e = cudaSuccess;
    unsigned int nl = 0;
    auto ok = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
        nl++;
    };
    const unsigned int np = a.np, n = a.nentry;
    const double* org = &a.prm.world_origin.x;
    const bool clusters = a.cl.ns != 0;
    // per-body arrays shorter than the sphere count are cluster state: only
    // the cluster form may run on them
    if (a.ns_state != np && (!clusters || a.cl.ns != a.ns_state)) return XDEM_ERR_ARG;
    if (clusters && (!fs.mixed || !fs.cpos_alt || !a.cpos || !a.rloc || !a.cl.neach ||
                     (unsigned long long)a.cl.ns * a.cl.neach != np))
        return XDEM_ERR_ARG;
    // a mixed sphere handle keeps acc and ea in FP32 copies: the first
    // position update reads the FP64 arrays, the body kernel the copies
    const bool f32_state = fs.mixed && !clusters;
    if (f32_state && !fs.primed && fs.f64_stale) {
        if (int r = fused_sync_fp64(fs, a.acc, a.ea, st)) return r;
    }
    if (f32_state && !fs.f32_ready) {
        if (capturing(st)) return XDEM_ERR_ARG;
        k_state_to_f32<<<blocks_for(np), kThreads, 0, st>>>(a.acc, a.ea, a.inertia, a.mass, fs.accf, fs.eaf, fs.jm,
                                                             np);
        ok(cudaGetLastError());
        fs.f32_ready = true;
    }
    if (!fs.primed) {
        // empty cell table, first position update + hash, and the extent of
        // the FP32 frame (grid origin to the far side of the particle cloud)
        ok(launch_fill_u32(a.cstart, 0xffffffffu, a.ncell, st));
        ok(cudaMemsetAsync(a.cend, 0, a.ncell * sizeof(unsigned int), st));
        fs.have_prev = false;
        if (clusters)
            k_prologue_cluster<<<blocks_for(a.cl.ns), kThreads, 0, st>>>(
                a.prm, a.cl, *a.cpos, *a.ep, a.vel, a.ev, a.acc, a.ea, a.mass, a.rloc, *a.pos, fs.cpos_alt,
                fs.ep_alt, fs.pos_alt, a.k0, a.v0, a.status, fs.rec);
        else
            k_prologue<<<blocks_for(np), kThreads, 0, st>>>(a.prm, *a.pos, *a.ep, a.vel, a.ev, a.acc, a.ea, a.mass,
                                                            fs.pos_alt, fs.ep_alt, a.k0, a.v0, np, a.status, fs.rec);
        ok(cudaGetLastError());
        const unsigned int nbb = std::min(kBboxBlocks, std::max(1u, blocks_for(np, 256)));
        k_bbox<<<nbb, 256, 0, st>>>(*a.pos, np, fs.d_bbox);
        ok(cudaGetLastError());
        std::vector<double> bb((size_t)nbb * 6);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(bb.data(), fs.d_bbox, bb.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return XDEM_ERR_CUDA;
        double r2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            double lo = 1e300, hi = -1e300;
            for (unsigned int b = 0; b < nbb; ++b) {
                lo = std::min(lo, bb[b * 6 + c]);
                hi = std::max(hi, bb[b * 6 + 3 + c]);
            }
            if (!(hi >= lo)) { lo = org[c]; hi = org[c]; }
            const double far = std::max(std::fabs(lo - org[c]), std::fabs(hi - org[c]));
            r2 += far * far;
        }
        // particles may drift: the FP32 frame covers the cloud plus 1 m
        const double R = std::sqrt(r2) + 1.0;
        fs.frame_far2 = R * R;
        // rounding of two FP32 coordinates of size <= R, their difference and
        // the sum of squares, with 4x slack; the mixed form rounds the centre
        // and the origin separately, so the origin's size counts too
        const double o_len = std::sqrt(org[0] * org[0] + org[1] * org[1] + org[2] * org[2]);
        fs.frame_margin = (float)(16.0 * (R + o_len) * std::ldexp(1.0, -24) + 1e-9);
        // the first step after priming builds the candidate lists
        if (fs.vl_flag) {
            ok(cudaMemsetAsync(fs.vl_flag + kVlRebuild, 1, sizeof(unsigned int), st));
            ok(cudaMemsetAsync(fs.vl_flag + kVlMoved, 0, sizeof(unsigned int), st));
            ok(cudaMemsetAsync(fs.vl_flag + kVlOverflow, 0, sizeof(unsigned int), st));
            ok(cudaMemsetAsync(fs.vl_flag + kVlSort, 1, sizeof(unsigned int), st));
        }
        fs.primed = true;
    }
    // Between steps *a.pos / *a.ep hold the committed state (x_n) and the
    // alternate buffers the positions of the next step (x_{n+1}, computed by
    // the prologue or by the previous contact kernel).  They become current
    // here; the contact kernel then writes x_{n+2} into the old buffers.
    std::swap(*a.pos, fs.pos_alt);
    std::swap(*a.ep, fs.ep_alt);
    if (clusters) std::swap(*a.cpos, fs.cpos_alt);
    // mesh spheres join the sort at entries np + first (xIntegratorVV.cpp:32-43)
    for (unsigned int m = 0; m < a.nmesh; ++m)
        ok(launch_hash(a.prm, a.k0, a.v0, a.tri_sphere + 4 * (size_t)a.mesh_first[m], np + a.mesh_first[m],
                       a.mesh_ntri[m], a.status, st));
    // With candidate lists the cell sort is only read by the stencil walk of
    // a rebuild step (or of a sphere whose list overflowed at the last
    // build): the device skips the clear, sort and reorder otherwise.
    const bool use_list = fs.mixed && fs.tune.skin_div != 0 && a.has_pp && !fs.any_coh && fs.vl_flag;
    const unsigned int* sort_gate = use_list ? fs.vl_flag + kVlSort : nullptr;
    // a batched list step as one persistent launch: the gated sort runs
    // inside it
    const bool persist = fs.persist && use_list && a.nscene > 1 && a.nmesh == 0 && !clusters && fs.d_bar;
    if (!persist) {
    // Captured into a graph, the gated section becomes the body of an IF
    // node whose condition a one-thread kernel sets from the gate, so that
    // between rebuilds the graph skips it instead of launching kernels that
    // return at once.  The body is captured on a side stream.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (use_list && fs.side_st && cudaStreamIsCapturing(st, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusNone;
    const bool cond = use_list && fs.side_st && cap == cudaStreamCaptureStatusActive;
    cudaStream_t sst = st;
    cudaGraphNode_t cnode = nullptr;
    const unsigned int nl_before = nl;
    if (cond) {
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaGraphConditionalHandle h = 0;
        ok(cudaStreamGetCaptureInfo(st, &cap, nullptr, &g, nullptr, nullptr, nullptr));
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
        if (e == cudaSuccess) {
            k_set_sort_cond<<<1, 1, 0, st>>>(h, sort_gate);
            ok(cudaGetLastError());
        }
        if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(st, &cap, nullptr, &g, &deps, nullptr, &nd);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        if (e == cudaSuccess) e = cudaGraphAddNode(&cnode, g, deps, nullptr, nd, &cp);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(fs.side_st, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return XDEM_ERR_CUDA;
        sst = fs.side_st;
    }
    if (fs.have_prev) ok(launch_clear_cells(fs.skey_prev, n, a.cstart, a.cend, sst, sort_gate));
    unsigned int *sk = nullptr, *sv = nullptr;
    ok(radix_sort_pairs(a.k0, a.v0, a.k1, a.v1, a.hist, n, a.sort_bits, &sk, &sv, sst, sort_gate));
    nl += 3 * ((a.sort_bits + 7) / 8) - 1;
    if (fs.mixed) {
        k_reorder_mixed<<<blocks_for(n), kThreads, 0, sst>>>(
            sort_gate, sk, sv, n, np, a.cstart, a.cend, a.sorted_index, fs.skey_prev,
            fs.rec, reinterpret_cast<float4*>(fs.mA),
            reinterpret_cast<float4*>(fs.mL), reinterpret_cast<float4*>(fs.mB), reinterpret_cast<float4*>(fs.mC),
            reinterpret_cast<uint2*>(fs.mIT));
    } else {
        k_reorder_fp64<<<blocks_for(n), kThreads, 0, st>>>(sk, sv, n, np, a.cstart, a.cend, a.sorted_index,
                                                           fs.skey_prev, *a.pos, *a.ep, a.vel, a.ev, a.mass,
                                                           fs.snap_pos, fs.snap_vel, fs.snap_om, fs.snap_f, org[0],
                                                           org[1], org[2], fs.frame_far2);
    }
    ok(cudaGetLastError());
    if (cond) {
        // the body's kernels run on rebuild steps only: a replayed step
        // counts the condition kernel
        nl = nl_before + 1;
        cudaGraph_t body = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(fs.side_st, &body);
        if (e == cudaSuccess) e = ee;
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) return XDEM_ERR_CUDA;
    }
    }  // !persist
    const bool had_prev = fs.have_prev;
    fs.have_prev = true;

    ContactLaunch c{};
    c.prm = a.prm;
    c.np = np;
    c.nentry = n;
    c.vel_compat = a.vel_compat;
    c.rolling_per_sphere = a.rolling_per_sphere;
    c.rolling = a.rolling;
    c.snap_pos = fs.snap_pos; c.snap_vel = fs.snap_vel; c.snap_om = fs.snap_om; c.snap_f = fs.snap_f;
    c.margin = fs.frame_margin;
    c.mA = fs.mA; c.mL = fs.mL; c.mB = fs.mB; c.mC = fs.mC; c.mIT = fs.mIT;
    c.rec = fs.rec;
    c.fA = fs.fA; c.fB = fs.fB; c.fC = fs.fC;
    c.use_list = use_list;
    c.vl_ids = fs.vl_ids; c.vl_cnt = fs.vl_cnt; c.vl_xb = fs.vl_xb;
    c.vl_flag = fs.vl_flag;
    c.skin_f = fs.tune.skin_div ? (float)(a.prm.cell_size / fs.tune.skin_div) : 0.f;
    c.half_skin2_f = 0.25f * c.skin_f * c.skin_f;
    c.mpf = fs.d_mpf;
    c.planef = fs.d_planef;
    c.planedf = fs.d_planedf;
    c.inv_cs = 1.0 / a.prm.cell_size;
    split_host(a.prm.cell_size, c.cs_f, c.cs_lo);
    c.inv_cs_f = (float)(1.0 / a.prm.cell_size);
    for (int i = 0; i < 3; ++i) split_host(org[i], c.o_hi[i], c.o_lo[i]);
    c.dt_f = (float)a.prm.dt;
    c.hdt_f = (float)(0.5 * a.prm.dt);
    c.h2_f = (float)a.prm.half2dt;
    c.g_f[0] = (float)a.prm.gravity.x; c.g_f[1] = (float)a.prm.gravity.y; c.g_f[2] = (float)a.prm.gravity.z;
    c.sorted_index = a.sorted_index; c.cstart = a.cstart; c.cend = a.cend; c.skey = fs.skey_prev;
    c.pos_cur = *a.pos; c.pos_next = fs.pos_alt; c.ep_cur = *a.ep; c.ep_next = fs.ep_alt;
    c.vel = a.vel; c.acc = a.acc; c.ev = a.ev; c.ea = a.ea; c.mass = a.mass; c.inertia = a.inertia;
    c.accf = f32_state ? fs.accf : nullptr;
    c.eaf = f32_state ? fs.eaf : nullptr;
    c.jm = f32_state ? fs.jm : nullptr;
    c.k_out = a.k0; c.v_out = a.v0;
    c.has_pp = a.has_pp;
    c.pp_count_old = *a.pp_count; c.pp_id_old = *a.pp_id; c.pp_tsd_old = *a.pp_tsd;
    c.pp_count_new = fs.pp_count2; c.pp_id_new = fs.pp_id2; c.pp_tsd_new = fs.pp_tsd2;
    c.planes = fs.planes; c.nplane = a.nplane; c.nmesh = a.nmesh;
    for (unsigned int m = 0; m < a.nmesh && m < kMaxFusedMeshes; ++m) {
        c.mesh_first[m] = a.mesh_first[m];
        c.mesh_ntri[m] = a.mesh_ntri[m];
        c.mesh_body[m] = a.mesh_body[m];
    }
    c.pl_count = a.pl_count; c.pl_id = a.pl_id; c.pl_tsd = a.pl_tsd;
    c.tri = a.tri; c.ms_count = a.ms_count; c.ms_id = a.ms_id; c.ms_tsd = a.ms_tsd;
    c.mesh_bs = fs.d_mesh_bs;
    c.tri_sphere = a.tri_sphere;
    c.ncyl = fs.mixed ? a.ncyl : 0u;
    c.cyl = a.cyl;
    c.cy_count = a.cy_count; c.cy_id = a.cy_id; c.cy_tsd = a.cy_tsd;
    c.body = a.body; c.mp = a.mp;
    // body wrench partials: one row entry per block of the emitting kernel
    // (the mixed pair and body kernels share their block size whenever the
    // handle keeps wrenches)
    c.tune = fs.tune;
    const unsigned int nt_emit = fs.mixed ? fs.tune.nt_bodies : (unsigned int)kFusedThreads;
    c.nblocks = (n + nt_emit - 1) / nt_emit;
    unsigned int rows_plane = c.nblocks, rows_mesh = c.nblocks;
    c.cl = a.cl;
    c.rloc = a.rloc;
    c.cpos_cur = clusters ? *a.cpos : nullptr;
    c.cpos_next = clusters ? fs.cpos_alt : nullptr;
    if (fs.mixed) {
        // rows of partial wrench sums: one per block of the kernel doing the
        // body's contacts -- planes: the body kernel (sorted entries, or
        // clusters); meshes: the pair kernel (sorted entries on the walk,
        // spheres with candidate lists); the row stride covers both
        // (the sphere body kernel writes one row per warp, the cluster body
        // kernel one per block)
        const unsigned int nt_b = fs.tune.nt_bodies, nt_p = fs.tune.nt_pairs;
        rows_plane = clusters ? (a.cl.ns + nt_b - 1) / nt_b : (n + 31) / 32;
        rows_mesh = use_list ? (np + nt_p - 1) / nt_p : (n + nt_p - 1) / nt_p;
        c.nblocks = std::max(rows_plane, rows_mesh);
    }
    c.bsums = a.bsums;
    c.status = a.status;
    c.nscene = a.nscene ? a.nscene : 1;
    c.scene_of = c.nscene > 1 ? a.scene_of : nullptr;
    c.scene_plane_first = c.nscene > 1 ? a.scene_plane_first : nullptr;
    if (e0) cudaEventRecord(e0, st);
    if (persist) {
        BatchSort b{};
        b.gate = sort_gate;
        b.k0 = a.k0; b.v0 = a.v0; b.k1 = a.k1; b.v1 = a.v1; b.hist = a.hist;
        b.n = n; b.np = np; b.bits = (unsigned int)std::max(a.sort_bits, 0);
        b.ntiles = (n + 2047u) / 2048u;  // the sort's tile: 256 threads x 8 keys
        b.have_prev = had_prev ? 1 : 0;
        b.skey_prev = fs.skey_prev; b.cstart = a.cstart; b.cend = a.cend; b.sorted_index = a.sorted_index;
        b.rec = fs.rec;
        b.mA = reinterpret_cast<float4*>(fs.mA); b.mL = reinterpret_cast<float4*>(fs.mL);
        b.mB = reinterpret_cast<float4*>(fs.mB); b.mC = reinterpret_cast<float4*>(fs.mC);
        b.mIT = reinterpret_cast<uint2*>(fs.mIT);
        b.bar = fs.d_bar;
        b.limit_ns = fs.persist_limit_ns;
        ok(launch_batch_step(c, b, fs.tune.occ_pairs, fs.persist_grid, st));
    } else {
        ok(fs.mixed ? launch_fused_contact_mixed(c, st) : launch_fused_contact_fp64(c, st));
    }
    if (f32_state) fs.f64_stale = true;
    // the mixed contact stage is two kernels (pairs, bodies), with candidate
    // lists three (list pairs, bodies, flag roll); the persistent step one
    if (fs.mixed && !persist) nl += c.use_list ? 2 : 1;
    if (e1) cudaEventRecord(e1, st);
    if (a.nbody && c.nscene == 1) {  // batched handles keep no body wrenches
        if (a.nbody > fs.wsum_cap) return XDEM_ERR_ARG;  // fused_set_bodies sizes the chunk sums
        k_body_sums<<<a.nbody * kWrenchChunks, 256, 0, st>>>(a.bsums, c.nblocks, a.nplane + c.ncyl, rows_plane, rows_mesh,
                                                             a.wrench, fs.wsum, fs.wcnt);
        ok(cudaGetLastError());
    }
    if (e != cudaSuccess) return XDEM_ERR_CUDA;
    // state now: x_{n+1}, e_{n+1} and vel/acc/ev/ea of step n+1 committed;
    // x_{n+2}, e_{n+2} in the alternate buffers (input of the next step); the
    // new pair lists in the partner buffers
    if (a.has_pp) {
        std::swap(*a.pp_count, fs.pp_count2);
        std::swap(*a.pp_id, fs.pp_id2);
        std::swap(*a.pp_tsd, fs.pp_tsd2);
    }
    if (nlaunch) *nlaunch = nl;
    return XDEM_OK;
}

int fused_energy(FusedState& fs, const double* vel, const double* ep, const double* ev, const double* mass,
                 const double* inertia, unsigned int ns, const unsigned int* c0, const unsigned int* c1,
                 const unsigned int* c2, unsigned int np, double* ke, unsigned int* ncontact, cudaStream_t st)
{
    double* d = fs.d_energy;
    if (!d) return XDEM_ERR_ARG;
    cudaError_t e = cudaMemsetAsync(d, 0, 16, st);
    if (e == cudaSuccess) {
        k_energy<<<304, 256, 0, st>>>(vel, ep, ev, mass, inertia, ns, c0, c1, c2, np, d,
                                      reinterpret_cast<unsigned int*>(d + 1));
        e = cudaGetLastError();
    }
    double h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return XDEM_ERR_CUDA;
    *ke = h[0];
    unsigned int c;
    std::memcpy(&c, &h[1], sizeof(c));
    *ncontact = c;
    return XDEM_OK;
}

}  // namespace xdem
