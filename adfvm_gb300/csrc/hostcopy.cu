// Host <-> device copies of the solver's field arrays from ANY host memory (pageable, pinned),
// with FP64 <-> FP32 conversion on the way when the host and device types differ.
//
// The reference hands its compiled step plain numpy arrays every call (adFVM/solver.py:312-323,
// apps/adjoint.py:268-291): pageable memory. Measured on a GB300 (Grace host, 16 threads, 168 MB
// arrays): a pageable device-to-host cudaMemcpy into a new array runs at about 22 GB/s and a
// precision change costs a further single-threaded pass over the array, while the pageable
// host-to-device copy of equal types already runs at about 180 GB/s, and so does the download
// into pages that are already mapped. So copies of equal types go straight to the CUDA driver (a
// download first touches its destination's pages with all host threads); conversions use a
// ring of two pinned staging chunks per device: the host threads (OpenMP) fill or drain chunk i,
// converting, while the copy engine moves chunk i-1, at the lower of the host's multi-threaded
// rate and the link's DMA rate (156 GB/s of FP64 host data uploaded as FP32, 56 GB/s of FP32
// device data downloaded into a new FP64 array).
#include <cuda_runtime.h>
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "afvm.h"

namespace afvm {
namespace {

constexpr size_t CHUNK = size_t(8) << 20;   // bytes of one staging chunk (device-side element type)
constexpr int MAX_DEVICES = 64;

struct Stager {
    std::mutex mu;
    unsigned char* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool armed[2] = {false, false};   // ev[k] recorded after the last copy that used buf[k]
    bool ready = false;
};
Stager g_stagers[MAX_DEVICES];

int stager_init(Stager& st) {
    if (st.ready) return AFVM_OK;
    for (int k = 0; k < 2; k++) {
        if (!st.buf[k] && cudaHostAlloc((void**)&st.buf[k], CHUNK, cudaHostAllocPortable) != cudaSuccess) {
            cudaGetLastError();
            return AFVM_ERR_OOM;
        }
        if (!st.ev[k] && cudaEventCreateWithFlags(&st.ev[k], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return AFVM_ERR_CUDA;
        }
    }
    st.ready = true;
    return AFVM_OK;
}

// waits until the copy engine no longer reads or writes buf[k]
int stager_wait(Stager& st, int k) {
    if (!st.armed[k]) return AFVM_OK;
    st.armed[k] = false;
    if (cudaEventSynchronize(st.ev[k]) != cudaSuccess) {
        cudaGetLastError();
        return AFVM_ERR_CUDA;
    }
    return AFVM_OK;
}

// n values from src (element size ss) to dst (element size ds), split over the host threads
void host_convert(void* dst, int ds, const void* src, int ss, size_t n) {
    const int nt = omp_get_max_threads();
    const size_t per = (n + (size_t)nt - 1) / (size_t)nt;
#pragma omp parallel num_threads(nt)
    {
        const size_t a = per * (size_t)omp_get_thread_num();
        const size_t b = a + per < n ? a + per : n;
        if (a < b) {
            if (ds == ss) {
                std::memcpy((unsigned char*)dst + a * ds, (const unsigned char*)src + a * ss, (b - a) * ds);
            } else if (ds == 4) {
                const double* s = (const double*)src;
                float* d = (float*)dst;
                for (size_t i = a; i < b; i++) d[i] = (float)s[i];
            } else {
                const float* s = (const float*)src;
                double* d = (double*)dst;
                for (size_t i = a; i < b; i++) d[i] = (double)s[i];
            }
        }
    }
}

bool pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

int to_device(Stager& st, void* dst, int ds, const void* src, int ss, size_t n, cudaStream_t s) {
    // same type: the CUDA driver's own path, pinned or not (on a GB300's Grace host its pageable
    // host-to-device copy runs at about 180 GB/s, against about 100 GB/s through the staging)
    if (ds == ss) {
        if (cudaMemcpyAsync(dst, src, n * (size_t)ds, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            cudaGetLastError();
            return AFVM_ERR_CUDA;
        }
        return AFVM_OK;
    }
    const size_t per = CHUNK / (size_t)ds;
    int k = 0;
    for (size_t off = 0; off < n; off += per, k ^= 1) {
        const size_t m = n - off < per ? n - off : per;
        int e = stager_wait(st, k);
        if (e) return e;
        host_convert(st.buf[k], ds, (const unsigned char*)src + off * ss, ss, m);
        if (cudaMemcpyAsync((unsigned char*)dst + off * ds, st.buf[k], m * (size_t)ds, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaEventRecord(st.ev[k], s) != cudaSuccess) {
            cudaGetLastError();
            return AFVM_ERR_CUDA;
        }
        st.armed[k] = true;
    }
    return AFVM_OK;
}

// writes a zero into every 4 KB page of [p, p + bytes), split over the host threads: a new
// (never touched) array takes its page faults in parallel here instead of one by one inside
// the CUDA driver's copy
void touch_pages(void* p, size_t bytes) {
    if (!bytes) return;
    unsigned char* b = (unsigned char*)p;
    const long long pages = (long long)((bytes + 4095) / 4096);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < pages; i++) b[(size_t)i * 4096] = 0;
    b[bytes - 1] = 0;
}

int to_host(Stager& st, void* dst, int ds, const void* src, int ss, size_t n, cudaStream_t s, bool syncPinned) {
    // same type: the CUDA driver's own path (a pageable device-to-host copy runs at about 185 GB/s
    // into pages that are already mapped but 21 GB/s into a new array; with the parallel touch
    // first, about 48 GB/s - the page faults themselves - and 168 GB/s into mapped pages)
    if (ds == ss) {
        const bool pin = pinned(dst);
        if (!pin) touch_pages(dst, n * (size_t)ds);
        if (cudaMemcpyAsync(dst, src, n * (size_t)ds, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            ((syncPinned || !pin) && cudaStreamSynchronize(s) != cudaSuccess)) {
            cudaGetLastError();
            return AFVM_ERR_CUDA;
        }
        return AFVM_OK;
    }
    // chunk c is copied into buf[c % 2] and drained by the host threads while chunk c+1 moves
    const size_t per = CHUNK / (size_t)ss;
    const size_t nChunks = (n + per - 1) / per;
    for (size_t c = 0; c <= nChunks; c++) {
        if (c < nChunks) {
            const int k = (int)(c & 1);
            const size_t off = c * per, m = n - off < per ? n - off : per;
            int e = stager_wait(st, k);
            if (e) return e;
            if (cudaMemcpyAsync(st.buf[k], (const unsigned char*)src + off * ss, m * (size_t)ss,
                                cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaEventRecord(st.ev[k], s) != cudaSuccess) {
                cudaGetLastError();
                return AFVM_ERR_CUDA;
            }
            st.armed[k] = true;
        }
        if (c > 0) {
            const int k = (int)((c - 1) & 1);
            const size_t off = (c - 1) * per, m = n - off < per ? n - off : per;
            int e = stager_wait(st, k);
            if (e) return e;
            host_convert((unsigned char*)dst + off * ds, ds, st.buf[k], ss, m);
        }
    }
    return AFVM_OK;
}

}  // namespace

int host_copy(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes, int64_t count,
              void* stream, bool toDevice, bool syncPinned) {
    if (count < 0 || (count > 0 && (!dst || !src)) || (dstBytes != 4 && dstBytes != 8) ||
        (srcBytes != 4 && srcBytes != 8) || device < 0 || device >= MAX_DEVICES)
        return AFVM_ERR_BAD_ARG;
    if (count == 0) return AFVM_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
        cudaGetLastError();
        return AFVM_ERR_BAD_ARG;
    }
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device && cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return AFVM_ERR_CUDA;
    }
    Stager& st = g_stagers[device];
    int e;
    {
        std::lock_guard<std::mutex> lock(st.mu);
        e = stager_init(st);
        if (!e)
            e = toDevice ? to_device(st, dst, dstBytes, src, srcBytes, (size_t)count, (cudaStream_t)stream)
                         : to_host(st, dst, dstBytes, src, srcBytes, (size_t)count, (cudaStream_t)stream,
                                   syncPinned);
    }
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return e;
}

}  // namespace afvm

extern "C" int afvm_copy_to_device(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes,
                                   int64_t count, void* stream) {
    return afvm::host_copy(device, dst, dstBytes, src, srcBytes, count, stream, true, true);
}

extern "C" int afvm_copy_to_host(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes,
                                 int64_t count, void* stream) {
    return afvm::host_copy(device, dst, dstBytes, src, srcBytes, count, stream, false, true);
}
