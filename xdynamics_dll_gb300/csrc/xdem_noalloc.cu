// xdem_noalloc.cu -- cu_reorderDataAndFindCellStart without any device
// allocation.
//
// The regular launcher sorts with scratch the library allocates (and grows)
// on first use with cudaMalloc.  Some callers cannot allow that: real-time
// loops where an allocation's latency or a possible out-of-memory failure in
// mid-run is unacceptable, and hosts whose device memory is owned by an
// external pool that forbids allocations behind its back.  This variant takes
// its sort scratch from a fixed array compiled into the library instead.
// Its first call on a device looks the array's address up
// (cudaGetSymbolAddress); make that first call before any stream capture.
//
// The array lives in device memory of every GPU that loads the library and
// stays there until the process exits; its size is fixed at build time
// (kNoAllocMaxEntries sort entries, about 2.2 MB).  All calls share it: two
// calls whose kernels overlap on the GPU (for instance on two streams) race
// on it and must be serialised by the caller.  Every word of it that a call
// reads is written earlier in the same call, so nothing left by a previous
// call needs clearing.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "xdem_kernels.h"

namespace {

constexpr unsigned int kNoAllocMaxEntries = 262144u;  // 2^18 (particles + mesh spheres)
constexpr unsigned int kSortTile = 2048u;             // entries per sort tile (xdem_sort.cu)
constexpr unsigned int kHistWords = ((kNoAllocMaxEntries + kSortTile - 1) / kSortTile) * 256u + 256u;
constexpr unsigned int kScratchWords = 2u * kNoAllocMaxEntries + kHistWords;

// Sort scratch: keys, values, then the per-tile digit table and digit totals.
static __device__ __align__(256) unsigned int g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
unsigned int* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device.  The host-side
// name g_noalloc_scratch is only a stand-in for the symbol, never a device
// address, so the address is looked up once per device with that device
// current.
int scratch_address(unsigned int** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return XDEM_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "cu_reorderDataAndFindCellStart_noalloc: cudaGetSymbolAddress failed: %s\n",
                    cudaGetErrorString(e));
            return XDEM_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<unsigned int*>(p);
    }
    *out = g_scratch_addr[dev];
    return XDEM_OK;
}

int bits_for_cells(unsigned long long ncell)
{
    int b = 0;
    while (b < 32 && (1ull << b) < ncell) ++b;
    return b == 0 ? 1 : b;
}

}  // namespace

extern "C" XDEM_API int cu_reorderDataAndFindCellStart_noalloc(unsigned int* hash, unsigned int* index,
                                                               unsigned int* cstart, unsigned int* cend,
                                                               unsigned int* sorted_index, unsigned int np,
                                                               unsigned int ncell)
{
    using namespace xdem;
    if (!hash || !index || !cstart || !cend || !sorted_index) return launcher_set_status(XDEM_ERR_ARG);
    if (np > kNoAllocMaxEntries) {
        fprintf(stderr,
                "cu_reorderDataAndFindCellStart_noalloc: %u entries exceed the fixed scratch capacity of %u; "
                "use cu_reorderDataAndFindCellStart\n",
                np, kNoAllocMaxEntries);
        return launcher_set_status(XDEM_ERR_ARG);
    }
    unsigned int* scratch = nullptr;
    if (int s = scratch_address(&scratch)) return launcher_set_status(s);
    const cudaStream_t st = launcher_stream();
    unsigned int* k1 = scratch;
    unsigned int* v1 = scratch + kNoAllocMaxEntries;
    unsigned int* hist = scratch + 2u * kNoAllocMaxEntries;
    // same steps as cu_reorderDataAndFindCellStart (def:94-124): empty the
    // cell tables, stable sort by hash in place, cell ranges + sorted index
    cudaError_t e = launch_fill_u32(cstart, 0xffffffffu, ncell, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cend, 0, (size_t)ncell * sizeof(unsigned int), st);
    unsigned int *sk = hash, *sv = index;
    if (e == cudaSuccess) e = radix_sort_pairs(hash, index, k1, v1, hist, np, bits_for_cells(ncell), &sk, &sv, st);
    if (e == cudaSuccess && sk != hash) {
        e = cudaMemcpyAsync(hash, sk, (size_t)np * sizeof(unsigned int), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(index, sv, (size_t)np * sizeof(unsigned int), cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) e = launch_cell_bounds(hash, index, cstart, cend, sorted_index, np, st);
    if (e != cudaSuccess) {
        fprintf(stderr, "cu_reorderDataAndFindCellStart_noalloc: CUDA error %s\n", cudaGetErrorString(e));
        return launcher_set_status(XDEM_ERR_CUDA);
    }
    return launcher_set_status(XDEM_OK);
}
