// Evaluates the library's FP64 reciprocal and reciprocal square root (rcp_nr, rsqrt_nr in
// adfvm_gb300/csrc/physics.cuh) on the GPU for a host array of arguments, so that a test can
// check them against correctly rounded references. Test helper: compiled by
// tests/test_gpu_rcp.py, never part of the library.
#include <cuda_runtime.h>
#include "physics.cuh"

__global__ void k_probe(const double* x, double* r, double* rs, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    r[i] = afvm::rcp_nr(x[i]);
    rs[i] = afvm::rsqrt_nr(x[i]);
}

extern "C" int rcp_probe(const double* x, double* r, double* rs, int n) {
    if (n <= 0) return 1;
    double* d = nullptr;
    size_t b = sizeof(double) * (size_t)n;
    if (cudaMalloc(&d, 3 * b) != cudaSuccess) return 2;
    int st = 0;
    if (cudaMemcpy(d, x, b, cudaMemcpyHostToDevice) != cudaSuccess) st = 3;
    if (!st) {
        k_probe<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
        if (cudaDeviceSynchronize() != cudaSuccess) st = 4;
    }
    if (!st && cudaMemcpy(r, d + n, b, cudaMemcpyDeviceToHost) != cudaSuccess) st = 5;
    if (!st && cudaMemcpy(rs, d + 2 * (size_t)n, b, cudaMemcpyDeviceToHost) != cudaSuccess) st = 6;
    cudaFree(d);
    return st;
}
