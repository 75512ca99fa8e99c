// xdem_sort.cu -- stable LSD radix sort of (cell hash, particle index) pairs:
// the launches of the phases in xdem_sort.cuh, one tile (or digit) per
// block.
#include <cuda_runtime.h>

#include "xdem_kernels.h"
#include "xdem_sort.cuh"

namespace xdem {

namespace {
using sortk::kRadix;
using sortk::kSortThreads;
using sortk::kTile;

__global__ void __launch_bounds__(kSortThreads)
k_radix_upsweep(const unsigned int* keys, unsigned int n, int shift, unsigned int* hist, unsigned int ntiles,
                const unsigned int* gate)
{
    if (gate && !*gate) return;
    __shared__ unsigned int h[kRadix];
    sortk::upsweep_tile(keys, n, shift, hist, ntiles, blockIdx.x, h);
}

// One block per digit.
__global__ void __launch_bounds__(kSortThreads) k_radix_scan(unsigned int* hist, unsigned int ntiles,
                                                             unsigned int* totals, const unsigned int* gate)
{
    if (gate && !*gate) return;
    __shared__ unsigned int sm[sortk::kWarps];
    sortk::scan_digit(hist, ntiles, totals, blockIdx.x, sm);
}

__global__ void __launch_bounds__(kSortThreads)
k_radix_scatter(const unsigned int* kin, const unsigned int* vin, unsigned int* kout, unsigned int* vout,
                unsigned int n, int shift, const unsigned int* hist, unsigned int ntiles, const unsigned int* totals,
                const unsigned int* gate)
{
    if (gate && !*gate) return;
    __shared__ unsigned int sm[sortk::kScatterWords];
    sortk::scatter_tile(kin, vin, kout, vout, n, shift, hist, ntiles, totals, blockIdx.x, sm);
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
