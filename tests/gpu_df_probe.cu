// Test probe for xdem_df.cuh: runs the integer-pipe conversions and the
// float-pair helpers over host arrays so tests/test_gpu_df.py can compare
// them with numpy's IEEE conversions and FP64 arithmetic.  Built by that
// test with nvcc into a temporary shared library.
#include <cuda_runtime.h>

#include "../xdynamics_dll_gb300/csrc/xdem_df.cuh"

using namespace xdem;

// The field-by-field form of d2f_rn that the mixed kernels used first: the
// reference the rebias-and-round form is checked against, bit for bit.
__device__ __forceinline__ float d2f_rn_fields(double x)
{
    const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
    const unsigned int sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned int m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned int rest = lo & 0x1fffffffu;
    const int fe = e - 896;
    unsigned int r = ((unsigned int)fe << 23) + m;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    r = fe <= 0 ? 0u : r;
    r = (fe >= 255 || r >= 0x7f800000u) ? 0x7f800000u : r;
    r = e == 0x7ff ? (0x7f800000u | ((m | rest) ? 0x400000u : 0u)) : r;
    return __uint_as_float(sign | r);
}

// Bit patterns where d2f_rn and d2f_rn_fields differ, over n doubles made on
// the device from a counter-based hash of (seed, i): every exponent, random
// mantissas, and the rounding boundaries (dropped bits 0x0fffffff,
// 0x10000000, 0x10000001 with either lowest kept bit).
__global__ void k_d2f_sweep(unsigned long long seed, unsigned long long n, unsigned long long* mismatches)
{
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    unsigned long long b = z;
    const unsigned int kind = (unsigned int)(i & 7u);
    if (kind >= 4) {
        const unsigned long long drop[4] = {0x0fffffffull, 0x10000000ull, 0x10000001ull, 0x1fffffffull};
        b = (b & ~0x1fffffffull) | drop[kind - 4];
    }
    const double x = __longlong_as_double((long long)b);
    if (__float_as_uint(d2f_rn(x)) != __float_as_uint(d2f_rn_fields(x))) atomicAdd(mismatches, 1ull);
}

extern "C" int d2f_sweep(unsigned long long seed, unsigned long long n, unsigned long long* mismatches)
{
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        k_d2f_sweep<<<(unsigned int)((n + 255) / 256), 256>>>(seed, n, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 1;
}

__global__ void k_probe(const double* x, const float* f, const float* a, const float* b, int n, float* d2f,
                        double* f2d_out, float* shi, float* slo, float* sum_hi, float* sum_lo, float* prod_hi,
                        float* prod_lo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d2f[i] = d2f_rn(x[i]);
    f2d_out[i] = f2d(f[i]);
    const df s = split_d(x[i]);
    shi[i] = s.hi;
    slo[i] = s.lo;
    // float-pair sum and product of (a[2i], a[2i+1]) and (b[2i], b[2i+1])
    const df A = df{a[2 * i], a[2 * i + 1]}, B = df{b[2 * i], b[2 * i + 1]};
    const df t = df_add(A, B);
    sum_hi[i] = t.hi;
    sum_lo[i] = t.lo;
    const df p = df_mul(A, B);
    prod_hi[i] = p.hi;
    prod_lo[i] = p.lo;
}

extern "C" int df_probe(const double* x, const float* f, const float* a, const float* b, int n, float* d2f,
                        double* f2d_out, float* shi, float* slo, float* sum_hi, float* sum_lo, float* prod_hi,
                        float* prod_lo)
{
    if (n <= 0) return 0;
    double *dx = nullptr, *dfo = nullptr;
    float *dff = nullptr, *da = nullptr, *db = nullptr, *out = nullptr;
    const size_t N = (size_t)n;
    cudaError_t e = cudaMalloc(&dx, N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dfo, N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dff, N * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&da, 2 * N * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&db, 2 * N * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&out, 7 * N * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, N * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dff, f, N * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(da, a, 2 * N * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, b, 2 * N * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_probe<<<(n + 255) / 256, 256>>>(dx, dff, da, db, n, out, dfo, out + N, out + 2 * N, out + 3 * N,
                                         out + 4 * N, out + 5 * N, out + 6 * N);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    float* outs[7] = {d2f, shi, slo, sum_hi, sum_lo, prod_hi, prod_lo};
    for (int k = 0; k < 7 && e == cudaSuccess; ++k)
        e = cudaMemcpy(outs[k], out + k * N, N * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f2d_out, dfo, N * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dx); cudaFree(dfo); cudaFree(dff); cudaFree(da); cudaFree(db); cudaFree(out);
    return e == cudaSuccess ? 0 : (int)e;
}
