// xdem_fused_mixed.cu -- the mixed form's sphere kernels without meshes (the
// candidate-list and stencil-walk pair kernels, the sphere body kernel) and
// the launch of the whole contact stage.  Compiled without implicit FMA
// contraction; the kernels are in xdem_fused_mixed.cuh.
#include "xdem_fused_mixed.cuh"
#include "xdem_sort.cuh"

namespace xdem {
namespace {

template <unsigned int NT, unsigned int STAGE, unsigned int OCC>
cudaError_t launch_pairs(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs<false, NT, STAGE, OCC><<<(c.nentry + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT, unsigned int STAGE>
cudaError_t launch_pairs_occ(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.occ_pairs == 1024 ? launch_pairs<NT, STAGE, 1024>(c, st) : launch_pairs<NT, STAGE, 768>(c, st);
}
template <unsigned int NT>
cudaError_t launch_pairs_stage(const ContactLaunch& c, cudaStream_t st)
{
    return c.tune.stage == 8 ? launch_pairs_occ<NT, 8>(c, st) : launch_pairs_occ<NT, 16>(c, st);
}
cudaError_t launch_pairs_nt(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.nt_pairs) {
    case 64: return launch_pairs_stage<64>(c, st);
    case 256: return launch_pairs_stage<256>(c, st);
    default: return launch_pairs_stage<128>(c, st);
    }
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_list(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_pairs_list<false, NT, OCC><<<(c.np + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
cudaError_t launch_list_nt(const ContactLaunch& c, cudaStream_t st)
{
    const bool hi = c.tune.occ_pairs == 1024;
    switch (c.tune.nt_pairs) {
    case 64: return hi ? launch_list<64, 1024>(c, st) : launch_list<64, 768>(c, st);
    case 256: return hi ? launch_list<256, 1024>(c, st) : launch_list<256, 768>(c, st);
    default: return hi ? launch_list<128, 1024>(c, st) : launch_list<128, 768>(c, st);
    }
}
template <unsigned int NT, unsigned int OCC>
cudaError_t launch_bodies(const ContactLaunch& c, cudaStream_t st)
{
    k_mixed_bodies<NT, OCC><<<(c.nentry + NT - 1) / NT, NT, 0, st>>>(c);
    return cudaGetLastError();
}
template <unsigned int NT>
cudaError_t launch_bodies_occ(const ContactLaunch& c, cudaStream_t st)
{
    switch (c.tune.occ_bodies) {
    case 768: return launch_bodies<NT, 768>(c, st);
    case 1024: return launch_bodies<NT, 1024>(c, st);
    default: return launch_bodies<NT, 512>(c, st);
    }
}

}  // namespace

// The block shapes come from c.tune (the autotuner's choice; by default 128
// threads, stage 16 and 768 threads per SM for the pairs, 128 threads and 512
// per SM for the bodies).  Body wrench partials are written by the kernel
// that owns the body (meshes: pairs, one row per block; planes and
// cylinders: the sphere body kernel, one row per warp; clusters: the cluster
// body kernel, one row per block) into rows of c.nblocks entries.  Scenes
// with meshes and cluster bodies run the kernels of xdem_fused_mixed_mesh.cu.
cudaError_t launch_fused_contact_mixed(const ContactLaunch& c, cudaStream_t st)
{
    if (c.nentry == 0) return cudaSuccess;
    cudaError_t e = c.nmesh ? launch_mixed_mesh_pairs(c, st) : c.use_list ? launch_list_nt(c, st) : launch_pairs_nt(c, st);
    if (e != cudaSuccess) return e;
    if (c.cl.ns) {
        e = launch_mixed_cluster_bodies(c, st);
    } else {
        switch (c.tune.nt_bodies) {
        case 64: e = launch_bodies_occ<64>(c, st); break;
        case 256: e = launch_bodies_occ<256>(c, st); break;
        default: e = launch_bodies_occ<128>(c, st); break;
        }
    }
    if (e != cudaSuccess || !c.use_list) return e;
    k_vl_roll<<<1, 1, 0, st>>>(c.vl_flag);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- persistent batched step
namespace {

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of the persistent step.  bar[0] counts the blocks that have
// arrived, bar[1] is the generation that the last arrival advances (after
// putting the count back to 0, so the barrier can be used again).  A block
// waits at most limit_ns on the global timer; past that it raises
// XDEM_ERR_BARRIER and returns false, and the kernel ends: the step is
// incomplete.  A block goes on only when every block has finished the
// phase before, so no phase reads inputs another block has not written.
// Every thread of the block calls it.
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, unsigned long long limit_ns, unsigned int* status,
                                             int* ok_s)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = bar + 1;
        const unsigned int g = *gen;
        int ok = 1;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1u) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*gen == g) {
                if (global_ns() - t0 > limit_ns) {
                    ok = 0;
                    atomicOr(status, XDEM_ERR_BARRIER);
                    break;
                }
                __nanosleep(100);
            }
            __threadfence();
        }
        *ok_s = ok;
    }
    __syncthreads();
    return *ok_s != 0;
}

constexpr unsigned int kBatchThreads = sortk::kSortThreads;
// shared words: the list phase's per-thread columns, reused by the sort
constexpr unsigned int kBatchWords = (kListCap + MAX_P2P_COUNT) * kBatchThreads;
static_assert(kBatchWords >= (unsigned int)sortk::kScatterWords, "the scatter fits in the list phase's columns");

// The step of xdem_fused_host.cu's fused_step for a batched list step, each
// phase over blocks of 256 threads striding the grid (the same arithmetic
// as the separate kernels: block shapes never change results).
template <unsigned int OCC>
__global__ void __launch_bounds__(kBatchThreads, OCC / kBatchThreads)
k_batch_step(const __grid_constant__ ContactLaunch c, const __grid_constant__ BatchSort b)
{
    constexpr unsigned int NT = kBatchThreads;
    __shared__ __align__(16) unsigned int sm[kBatchWords];
    __shared__ int ok_s;
    const unsigned int nb = gridDim.x;
    unsigned int* bar = b.bar;
    if (*b.gate) {
        // rebuild or overflowed list: clear last step's cells, sort, reorder
        if (b.have_prev) {
            for (unsigned int i = blockIdx.x * NT + threadIdx.x; i < b.n; i += nb * NT) {
                const unsigned int h = b.skey_prev[i];
                b.cstart[h] = 0xffffffffu;
                b.cend[h] = 0u;
            }
            if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
        }
        unsigned int *ki = b.k0, *vi = b.v0, *ko = b.k1, *vo = b.v1;
        if (b.n >= 2) {
            unsigned int* totals = b.hist + (size_t)b.ntiles * sortk::kRadix;
            for (unsigned int shift = 0; shift < b.bits; shift += 8) {
                for (unsigned int t = blockIdx.x; t < b.ntiles; t += nb)
                    sortk::upsweep_tile(ki, b.n, (int)shift, b.hist, b.ntiles, t, sm);
                if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
                for (unsigned int d = blockIdx.x; d < (unsigned int)sortk::kRadix; d += nb)
                    sortk::scan_digit(b.hist, b.ntiles, totals, d, sm);
                if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
                for (unsigned int t = blockIdx.x; t < b.ntiles; t += nb)
                    sortk::scatter_tile(ki, vi, ko, vo, b.n, (int)shift, b.hist, b.ntiles, totals, t, sm);
                if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
                unsigned int* t = ki; ki = ko; ko = t;
                t = vi; vi = vo; vo = t;
            }
        }
        for (unsigned int s = blockIdx.x * NT + threadIdx.x; s < b.n; s += nb * NT)
            reorder_mixed_entry(s, ki, vi, b.n, b.np, b.cstart, b.cend, b.sorted_index, b.skey_prev, b.rec, b.mA,
                                b.mL, b.mB, b.mC, b.mIT);
        if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
    }
    const unsigned int npb = (c.np + NT - 1) / NT;
    for (unsigned int bx = blockIdx.x; bx < npb; bx += nb) pairs_list_block<false, NT>(c, bx, sm, sm + kListCap * NT, nullptr);
    if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
    const unsigned int neb = (c.nentry + NT - 1) / NT;
    for (unsigned int bx = blockIdx.x; bx < neb; bx += nb) bodies_block<NT>(c, bx);
    if (!grid_barrier(bar, b.limit_ns, c.status, &ok_s)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) vl_roll(c.vl_flag);
}

template <unsigned int OCC>
cudaError_t launch_batch_occ(const ContactLaunch& c, const BatchSort& b, unsigned int* grid, cudaStream_t st)
{
    if (*grid == 0) {
        int dev = 0, nsm = 0, per = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<OCC>, kBatchThreads, 0);
        if (e != cudaSuccess) return e;
        if (per < 1 || nsm < 1) return cudaErrorCooperativeLaunchTooLarge;
        *grid = (unsigned int)(per * nsm);
    }
    cudaError_t e = cudaMemsetAsync(b.bar, 0, 2 * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(*grid);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch_step<OCC>, c, b);
}

}  // namespace

cudaError_t launch_batch_step(const ContactLaunch& c, const BatchSort& b, unsigned int occ, unsigned int* grid,
                              cudaStream_t st)
{
    if (c.nentry == 0) return cudaSuccess;
    return occ == 1024 ? launch_batch_occ<1024>(c, b, grid + 1, st) : launch_batch_occ<768>(c, b, grid, st);
}

}  // namespace xdem
