// Test probe for xdem_df.cuh: runs the integer-pipe conversions and the
// float-pair helpers over host arrays so tests/test_gpu_df.py can compare
// them with numpy's IEEE conversions and FP64 arithmetic.  Built by that
// test with nvcc into a temporary shared library.
#include <cuda_runtime.h>

#include "../xdynamics_dll_gb300/csrc/xdem_df.cuh"

using namespace xdem;

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
