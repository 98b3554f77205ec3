// Sensitivity dot product sum_k <grad_k, pert_k> in FP64 (cmesh.computeSensitivity,
// adFVM/cpp/cmesh.cpp:309-340, an OpenMP reduction in the reference).
//
// Deterministic two-level reduction: for array k, at most SENS_BLOCKS blocks run a
// grid-stride loop, reduce with warp shuffles and write one partial each to
// partials[k * SENS_BLOCKS + b]; one block then adds all partials in a fixed order. The
// result does not depend on timing, and repeated calls give identical bits.
#include <cuda_runtime.h>
#include "ctx.cuh"

namespace afvm {

constexpr int SENS_BLOCKS = 1024;

__device__ __forceinline__ double warp_sum(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

__global__ void __launch_bounds__(BLOCK) k_sens_partial(const double* __restrict__ g, const double* __restrict__ p,
                                                        long long n, double* __restrict__ partials) {
    __shared__ double sh[BLOCK / 32];
    double v = 0.0;
    for (long long i = blockIdx.x * (long long)BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK)
        v += g[i] * p[i];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double r = (threadIdx.x < BLOCK / 32) ? sh[threadIdx.x] : 0.0;
        r = warp_sum(r);
        if (threadIdx.x == 0) partials[blockIdx.x] = r;
    }
}

// partials are laid out [array][SENS_BLOCKS]; nUsed[k] blocks of array k are valid
__global__ void __launch_bounds__(BLOCK) k_sens_finish(const double* __restrict__ partials, const int* nUsed,
                                                       int nArrays, double* out) {
    __shared__ double sh[BLOCK / 32];
    double v = 0.0;
    for (int k = 0; k < nArrays; k++)
        for (int b = threadIdx.x; b < nUsed[k]; b += BLOCK) v += partials[(size_t)k * SENS_BLOCKS + b];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double r = (threadIdx.x < BLOCK / 32) ? sh[threadIdx.x] : 0.0;
        r = warp_sum(r);
        if (threadIdx.x == 0) *out = r;
    }
}

static int sens_blocks(long long n) {
    long long b = (n + BLOCK - 1) / BLOCK;
    return (int)(b < SENS_BLOCKS ? (b < 1 ? 1 : b) : SENS_BLOCKS);
}

// scratch: nArrays * SENS_BLOCKS partials + nArrays block counts + the result
int sensitivity_launch(int nArrays, const double* const* grad, const double* const* pert, const int64_t* n,
                       double* partials, int* nUsedDev, double* resultDev, cudaStream_t s, std::string* err) {
    std::vector<int> used(nArrays);
    for (int k = 0; k < nArrays; k++) {
        if (n[k] < 0 || (n[k] > 0 && (!grad[k] || !pert[k]))) {
            if (err) *err = "afvm_sensitivity: array " + std::to_string(k) + " has a bad size or pointer";
            return AFVM_ERR_BAD_ARG;
        }
        used[k] = n[k] > 0 ? sens_blocks(n[k]) : 0;
    }
    cudaError_t e = cudaMemcpyAsync(nUsedDev, used.data(), sizeof(int) * nArrays, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        if (err) *err = std::string("afvm_sensitivity: ") + cudaGetErrorString(e);
        return AFVM_ERR_CUDA;
    }
    for (int k = 0; k < nArrays; k++)
        if (used[k] > 0)
            k_sens_partial<<<used[k], BLOCK, 0, s>>>(grad[k], pert[k], (long long)n[k], partials + (size_t)k * SENS_BLOCKS);
    k_sens_finish<<<1, BLOCK, 0, s>>>(partials, nUsedDev, nArrays, resultDev);
    // the block counts are read from host memory that lives until the copy is done
    e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (err) *err = std::string("afvm_sensitivity: ") + cudaGetErrorString(e);
        return AFVM_ERR_CUDA;
    }
    return AFVM_OK;
}

int sensitivity_dev(Ctx* c, int nArrays, const double* const* grad, const double* const* pert, const int64_t* n,
                    double* out, cudaStream_t s) {
    if (nArrays <= 0 || !grad || !pert || !n || !out) return fail(c, AFVM_ERR_BAD_ARG, "afvm_sensitivity arguments");
    // scratch sized for this call, kept on the context and grown on demand
    size_t need = sizeof(double) * ((size_t)nArrays * SENS_BLOCKS + 1) + sizeof(int) * (size_t)nArrays;
    if (need > c->sensBytes) {
        if (c->sensScratch) cudaFree(c->sensScratch);
        c->sensScratch = nullptr;
        c->sensBytes = 0;
        if (cudaMalloc(&c->sensScratch, need) != cudaSuccess) {
            cudaGetLastError();
            return fail(c, AFVM_ERR_OOM, "afvm_sensitivity scratch");
        }
        c->sensBytes = need;
    }
    double* partials = (double*)c->sensScratch;
    double* result = partials + (size_t)nArrays * SENS_BLOCKS;
    int* nUsed = (int*)(result + 1);
    ProfScope ps(c, KID_SENS, s);
    int st = sensitivity_launch(nArrays, grad, pert, n, partials, nUsed, result, s, &c->err);
    if (st) return st;
    cudaError_t e = cudaMemcpy(out, result, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "afvm_sensitivity result");
    return AFVM_OK;
}

}  // namespace afvm
