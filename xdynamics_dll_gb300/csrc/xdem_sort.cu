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
k_radix_upsweep(const unsigned int* keys, unsigned int n, int shift, unsigned int* hist, unsigned int ntiles)
{
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

// Exclusive scan of `len` counters by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_radix_scan(unsigned int* hist, unsigned int len)
{
    __shared__ unsigned int part[1024];
    const unsigned int per = (len + 1023) / 1024;
    const unsigned int b = threadIdx.x * per;
    const unsigned int e = b + per < len ? b + per : len;
    unsigned int s = 0;
    for (unsigned int i = b; i < e; ++i) s += hist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    // Hillis-Steele inclusive scan of the 1024 partial sums
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned int v = threadIdx.x >= (unsigned int)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned int run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (unsigned int i = b; i < e; ++i) {
        const unsigned int v = hist[i];
        hist[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kSortThreads)
k_radix_scatter(const unsigned int* kin, const unsigned int* vin, unsigned int* kout, unsigned int* vout,
                unsigned int n, int shift, const unsigned int* hist, unsigned int ntiles)
{
    constexpr int kWarps = kSortThreads / 32;
    __shared__ unsigned int base[kRadix];
    __shared__ unsigned int run[kRadix];
    __shared__ unsigned int wcnt[kWarps][kRadix + 1];
    const unsigned int tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    base[tid] = hist[tid * ntiles + blockIdx.x];
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
    return (ntiles ? ntiles : 1) * kRadix;
}

cudaError_t radix_sort_pairs(unsigned int* k0, unsigned int* v0, unsigned int* k1, unsigned int* v1,
                             unsigned int* hist, unsigned int n, int bits, unsigned int** out_k,
                             unsigned int** out_v, cudaStream_t st)
{
    *out_k = k0;
    *out_v = v0;
    if (n < 2) return cudaSuccess;
    const unsigned int ntiles = (n + kTile - 1) / kTile;
    unsigned int *ki = k0, *vi = v0, *ko = k1, *vo = v1;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_upsweep<<<ntiles, kSortThreads, 0, st>>>(ki, n, shift, hist, ntiles);
        k_radix_scan<<<1, 1024, 0, st>>>(hist, ntiles * kRadix);
        k_radix_scatter<<<ntiles, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, shift, hist, ntiles);
        unsigned int* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    *out_k = ki;
    *out_v = vi;
    return cudaGetLastError();
}

}  // namespace xdem
