// Sensitivity dot product sum_k <grad_k, pert_k> in FP64 (cmesh.computeSensitivity,
// adFVM/cpp/cmesh.cpp:309-340, an OpenMP reduction in the reference).
//
// Deterministic two-level reduction: for array k, at most SENS_BLOCKS blocks run a
// grid-stride loop, reduce with warp shuffles and write one partial each to
// partials[k * SENS_BLOCKS + b]; one block then adds all partials in a fixed order. The
// result does not depend on timing, and repeated calls give identical bits.
#include <cuda_runtime.h>
#include <mutex>
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

// ---------------------------------------------------------------------------------------
// Allocation-free variant (afvm_sensitivity_noalloc).
//
// Some callers may not allocate device memory: an application that gives this library a
// fixed share of the GPU up front and makes every allocation itself, or a plug-in loaded
// into a host program whose memory pool it must not touch. Such a caller can create no
// context and cannot let afvm_sensitivity grow its scratch. For them the reduction's
// scratch (block partials, per-array block counts and the result) is this file-scope device
// array, sized for at most AFVM_SENSITIVITY_NOALLOC_MAX_ARRAYS arrays. Every GPU that loads
// the library keeps it (~129 KB) until the process exits. All calls share it: two calls
// that overlap on the GPU (different streams, or different host threads without ordering)
// race on it.
// ---------------------------------------------------------------------------------------

constexpr int NOALLOC_MAX_ARRAYS = AFVM_SENSITIVITY_NOALLOC_MAX_ARRAYS;
constexpr size_t NOALLOC_PARTIALS = (size_t)NOALLOC_MAX_ARRAYS * SENS_BLOCKS;
// partials, then the result, then the block counts (as doubles' worth of ints)
constexpr size_t NOALLOC_DOUBLES = NOALLOC_PARTIALS + 1 + (NOALLOC_MAX_ARRAYS + 1) / 2;

static __device__ __align__(256) double g_sens_noalloc_scratch[NOALLOC_DOUBLES];

// Host code must not use the symbol itself as a device address: the device address of the
// array is looked up by the first call on each device, with that device current, and cached
// here (so that first call belongs before any stream capture). cudaDeviceReset unloads the
// module: the cached address is then stale, and calls after a reset are not supported.
static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[256] = {nullptr};

static int noalloc_scratch(int device, double** out) {
    if (device < 0 || device >= 256) return AFVM_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sens_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return AFVM_ERR_CUDA;
        }
        g_noalloc_ptr[device] = (double*)p;
    }
    *out = g_noalloc_ptr[device];
    return AFVM_OK;
}

}  // namespace afvm

extern "C" int afvm_sensitivity_noalloc(int32_t device, int32_t nArrays, const double* const* grad,
                                        const double* const* pert, const int64_t* n, double* out, void* stream) {
    using namespace afvm;
    if (nArrays <= 0 || nArrays > NOALLOC_MAX_ARRAYS || !grad || !pert || !n || !out) return AFVM_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return AFVM_ERR_BAD_ARG;
    }
    // every array must be memory of `device` and the stream a stream of it: a host pointer or
    // another GPU's memory would make the kernels fault or read the wrong memory
    for (int k = 0; k < nArrays; k++) {
        if (n[k] <= 0) continue;
        const void* ptrs[2] = {grad[k], pert[k]};
        for (const void* q : ptrs) {
            cudaPointerAttributes a;
            if (!q || cudaPointerGetAttributes(&a, q) != cudaSuccess ||
                (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != device) {
                cudaGetLastError();
                return AFVM_ERR_BAD_ARG;
            }
        }
    }
    if (stream) {
        int sdev = -1;
        if (cudaStreamGetDevice((cudaStream_t)stream, &sdev) != cudaSuccess || sdev != device) {
            cudaGetLastError();
            return AFVM_ERR_BAD_ARG;
        }
    }
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device && cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return AFVM_ERR_CUDA;
    }
    double* scratch = nullptr;
    int st = noalloc_scratch(device, &scratch);
    if (st == AFVM_OK) {
        double* partials = scratch;
        double* result = scratch + NOALLOC_PARTIALS;
        int* nUsed = (int*)(result + 1);
        cudaStream_t s = (cudaStream_t)stream;
        // every partial and count read below is written earlier in this call, so nothing left by
        // a previous call is used and nothing needs clearing
        st = sensitivity_launch(nArrays, grad, pert, n, partials, nUsed, result, s, nullptr);
        if (st == AFVM_OK && cudaMemcpy(out, result, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            st = AFVM_ERR_CUDA;
        }
    }
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return st;
}
