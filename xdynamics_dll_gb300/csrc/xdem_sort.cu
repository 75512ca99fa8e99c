// xdem_sort.cu -- stable LSD radix sort of (cell hash, particle index) pairs.
//
// Replaces thrust::sort_by_key of cu_reorderDataAndFindCellStart
// (source/xdynamics_parallel/xParallelDEM_def.cu:107-109): stable, so entries
// of one cell stay in index order, which fixes the order the contact kernels
// visit candidates in and therefore the order of the pair lists.
//
// Per 8-bit digit: (1) per-tile digit histograms, (2) one exclusive scan of
// the digit-major histogram table, (3) a scatter where each tile ranks its
// keys stably (rounds of 256 consecutive keys; inside a round, warp
// match-any peers + per-warp digit counts) and writes them to their global
// slots.
#include <cuda_runtime.h>

#include "xdem_kernels.h"

namespace xdem {

namespace {
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;

__global__ void __launch_bounds__(kSortThreads)
k_radix_upsweep(const unsigned int* keys, unsigned int n, int shift, unsigned int* hist, unsigned int ntiles,
                const unsigned int* gate)
{
    if (gate && !*gate) return;
    __shared__ unsigned int h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const unsigned int base = blockIdx.x * kTile;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const unsigned int e = base + r * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (256 threads); returns
// the prefix and writes the block total to *total.
__device__ __forceinline__ unsigned int block_exclusive_scan(unsigned int v, unsigned int* sm /* [8] */,
                                                             unsigned int* total)
{
    const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned int)o) x += y;
    }
    if (lane == 31) sm[warp] = x;
    __syncthreads();
    unsigned int woff = 0, tot = 0;
    for (unsigned int w = 0; w < kSortThreads / 32; ++w) {
        const unsigned int c = sm[w];
        woff += w < warp ? c : 0u;
        tot += c;
    }
    __syncthreads();
    *total = tot;
    return woff + x - v;
}

// One block per digit: exclusive scan of that digit's per-tile counts (one
// row of the digit-major table), row total into totals[digit].
__global__ void __launch_bounds__(kSortThreads) k_radix_scan(unsigned int* hist, unsigned int ntiles,
                                                             unsigned int* totals, const unsigned int* gate)
{
    if (gate && !*gate) return;
    __shared__ unsigned int sm[kSortThreads / 32];
    unsigned int* row = hist + (size_t)blockIdx.x * ntiles;
    unsigned int carry = 0;
    for (unsigned int base = 0; base < ntiles; base += kSortThreads) {
        const unsigned int i = base + threadIdx.x;
        const unsigned int v = i < ntiles ? row[i] : 0u;
        unsigned int tot;
        const unsigned int ex = block_exclusive_scan(v, sm, &tot);
        if (i < ntiles) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads)
k_radix_scatter(const unsigned int* kin, const unsigned int* vin, unsigned int* kout, unsigned int* vout,
                unsigned int n, int shift, const unsigned int* hist, unsigned int ntiles, const unsigned int* totals,
                const unsigned int* gate)
{
    if (gate && !*gate) return;
    constexpr int kWarps = kSortThreads / 32;
    __shared__ unsigned int base[kRadix];
    __shared__ unsigned int run[kRadix];
    __shared__ unsigned int wcnt[kWarps][kRadix + 1];
    __shared__ unsigned int scan_sm[kSortThreads / 32];
    const unsigned int tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // start of each digit = exclusive scan of the digit totals, plus this
    // tile's offset within the digit
    unsigned int tot;
    const unsigned int dbase = block_exclusive_scan(totals[tid], scan_sm, &tot);
    base[tid] = dbase + hist[tid * ntiles + blockIdx.x];
    run[tid] = 0;
    const unsigned int lt = (1u << lane) - 1u;
    const unsigned int tile = blockIdx.x * kTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int w = 0; w < kWarps; ++w) wcnt[w][tid] = 0;
        if (tid == 0)
            for (int w = 0; w < kWarps; ++w) wcnt[w][kRadix] = 0;
        __syncthreads();
        const unsigned int e = tile + r * kSortThreads + tid;
        const bool ok = e < n;
        unsigned int k = 0, v = 0, d = kRadix;
        if (ok) { k = kin[e]; v = vin[e]; d = (k >> shift) & 255u; }
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int rank = __popc(peers & lt);
        if (rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            unsigned int acc = run[tid];
            for (int w = 0; w < kWarps; ++w) {
                const unsigned int c = wcnt[w][tid];
                wcnt[w][tid] = acc;
                acc += c;
            }
            run[tid] = acc;
        }
        __syncthreads();
        if (ok) {
            const unsigned int dst = base[d] + wcnt[warp][d] + rank;
            kout[dst] = k;
            vout[dst] = v;
        }
        __syncthreads();
    }
}
}  // namespace

size_t radix_hist_size(unsigned int n)
{
    const size_t ntiles = (n + kTile - 1) / kTile;
    return (ntiles ? ntiles : 1) * kRadix + kRadix;  // table + digit totals
}

cudaError_t radix_sort_pairs(unsigned int* k0, unsigned int* v0, unsigned int* k1, unsigned int* v1,
                             unsigned int* hist, unsigned int n, int bits, unsigned int** out_k,
                             unsigned int** out_v, cudaStream_t st, const unsigned int* gate)
{
    *out_k = k0;
    *out_v = v0;
    if (n < 2) return cudaSuccess;
    const unsigned int ntiles = (n + kTile - 1) / kTile;
    unsigned int* totals = hist + (size_t)ntiles * kRadix;
    unsigned int *ki = k0, *vi = v0, *ko = k1, *vo = v1;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_upsweep<<<ntiles, kSortThreads, 0, st>>>(ki, n, shift, hist, ntiles, gate);
        k_radix_scan<<<kRadix, kSortThreads, 0, st>>>(hist, ntiles, totals, gate);
        k_radix_scatter<<<ntiles, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, shift, hist, ntiles, totals, gate);
        unsigned int* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    *out_k = ki;
    *out_v = vi;
    return cudaGetLastError();
}

}  // namespace xdem
