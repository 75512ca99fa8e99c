// xdem_sort.cuh -- the phases of the stable LSD radix sort of (cell hash,
// particle index) pairs as per-tile device functions: the sort's own kernels
// (xdem_sort.cu) run one tile or digit per block, and the persistent batched
// step (xdem_fused_mixed.cu) runs them over its blocks with grid barriers in
// between.
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
// slots.  Every function is called by all kSortThreads threads of a block.
#pragma once
#include <cuda_runtime.h>

namespace xdem {
namespace sortk {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;

// Shared memory of the scatter (the largest phase), in 32-bit words.
constexpr int kScatterWords = kRadix + kRadix + kWarps * (kRadix + 1) + kWarps;

// Digit histogram of one tile into column `tile` of the digit-major table.
// h: kRadix shared words.
__device__ __forceinline__ void upsweep_tile(const unsigned int* keys, unsigned int n, int shift, unsigned int* hist,
                                             unsigned int ntiles, unsigned int tile, unsigned int* h)
{
    h[threadIdx.x] = 0;
    __syncthreads();
    const unsigned int base = tile * kTile;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const unsigned int e = base + r * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + tile] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (kSortThreads threads);
// returns the prefix and writes the block total to *total.  sm: kWarps words.
__device__ __forceinline__ unsigned int block_exclusive_scan(unsigned int v, unsigned int* sm, unsigned int* total)
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
    for (unsigned int w = 0; w < kWarps; ++w) {
        const unsigned int c = sm[w];
        woff += w < warp ? c : 0u;
        tot += c;
    }
    __syncthreads();
    *total = tot;
    return woff + x - v;
}

// Exclusive scan of one digit's per-tile counts (one row of the
// digit-major table), row total into totals[digit].  sm: kWarps words.
__device__ __forceinline__ void scan_digit(unsigned int* hist, unsigned int ntiles, unsigned int* totals,
                                           unsigned int digit, unsigned int* sm)
{
    unsigned int* row = hist + (size_t)digit * ntiles;
    unsigned int carry = 0;
    for (unsigned int base = 0; base < ntiles; base += kSortThreads) {
        const unsigned int i = base + threadIdx.x;
        const unsigned int v = i < ntiles ? row[i] : 0u;
        unsigned int tot;
        const unsigned int ex = block_exclusive_scan(v, sm, &tot);
        if (i < ntiles) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[digit] = carry;
}

// Stable scatter of one tile.  sm: kScatterWords shared words.
__device__ __forceinline__ void scatter_tile(const unsigned int* kin, const unsigned int* vin, unsigned int* kout,
                                             unsigned int* vout, unsigned int n, int shift, const unsigned int* hist,
                                             unsigned int ntiles, const unsigned int* totals, unsigned int tile,
                                             unsigned int* sm)
{
    unsigned int* base = sm;
    unsigned int* run = sm + kRadix;
    unsigned int* wcnt = sm + 2 * kRadix;                     // [kWarps][kRadix + 1]
    unsigned int* scan_sm = sm + 2 * kRadix + kWarps * (kRadix + 1);
    const unsigned int tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // start of each digit = exclusive scan of the digit totals, plus this
    // tile's offset within the digit
    unsigned int tot;
    const unsigned int dbase = block_exclusive_scan(totals[tid], scan_sm, &tot);
    base[tid] = dbase + hist[tid * ntiles + tile];
    run[tid] = 0;
    const unsigned int lt = (1u << lane) - 1u;
    const unsigned int t0 = tile * kTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int w = 0; w < kWarps; ++w) wcnt[w * (kRadix + 1) + tid] = 0;
        if (tid == 0)
            for (int w = 0; w < kWarps; ++w) wcnt[w * (kRadix + 1) + kRadix] = 0;
        __syncthreads();
        const unsigned int e = t0 + r * kSortThreads + tid;
        const bool ok = e < n;
        unsigned int k = 0, v = 0, d = kRadix;
        if (ok) { k = kin[e]; v = vin[e]; d = (k >> shift) & 255u; }
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int rank = __popc(peers & lt);
        if (rank == 0) wcnt[warp * (kRadix + 1) + d] = __popc(peers);
        __syncthreads();
        {
            unsigned int acc = run[tid];
            for (int w = 0; w < kWarps; ++w) {
                const unsigned int c = wcnt[w * (kRadix + 1) + tid];
                wcnt[w * (kRadix + 1) + tid] = acc;
                acc += c;
            }
            run[tid] = acc;
        }
        __syncthreads();
        if (ok) {
            const unsigned int dst = base[d] + wcnt[warp * (kRadix + 1) + d] + rank;
            kout[dst] = k;
            vout[dst] = v;
        }
        __syncthreads();
    }
}

}  // namespace sortk
}  // namespace xdem
