// Device-side loads of the face inputs from the cell records and the mesh tables.
#pragma once
#include "ctx.cuh"
#include "face.cuh"

namespace afvm {

// 16-byte vector loads of n values (n a multiple of 4 floats / 2 doubles; p 16-byte aligned)
__device__ __forceinline__ void load_vec(const double* __restrict__ p, double* o, int n) {
#pragma unroll
    for (int i = 0; i < n; i += 2) {
        double2 v = __ldg(reinterpret_cast<const double2*>(p + i));
        o[i] = v.x; o[i + 1] = v.y;
    }
}
__device__ __forceinline__ void load_vec(const float* __restrict__ p, float* o, int n) {
#pragma unroll
    for (int i = 0; i < n; i += 4) {
        float4 v = __ldg(reinterpret_cast<const float4*>(p + i));
        o[i] = v.x; o[i + 1] = v.y; o[i + 2] = v.z; o[i + 3] = v.w;
    }
}

// the 55 inputs of one face: primitives and gradients of both sides, geometry
template <typename R>
__device__ __forceinline__ void load_face(const MeshDev<R>& m, const R* __restrict__ rec, int f, FaceIn<R>& in) {
    const size_t nF = m.nF;
    int iP = m.own[f], iN = m.nbr[f];
    int iNg = (f < m.nIF) ? iN : m.gsrc[iN - m.nIC];   // ghost gradient = copy of its source
    R rP[REC], rN[REC], rNg[REC];
    load_vec(rec + (size_t)iP * REC, rP, REC);
    load_vec(rec + (size_t)iN * REC, rN, REC);
    if (iNg == iN) {
        for (int k = 0; k < REC; k++) rNg[k] = rN[k];
    } else {
        load_vec(rec + (size_t)iNg * REC, rNg, REC);
    }
    for (int k = 0; k < 3; k++) { in.UP[k] = rP[k]; in.UN[k] = rN[k]; }
    in.TP = rP[R_T]; in.pP = rP[R_P];
    in.TN = rN[R_T]; in.pN = rN[R_P];
    for (int k = 0; k < 9; k++) { in.gUP[k] = rP[R_GU + k]; in.gUN[k] = rNg[R_GU + k]; }
    for (int k = 0; k < 3; k++) {
        in.gTP[k] = rP[R_GT + k]; in.gTN[k] = rNg[R_GT + k];
        in.gpP[k] = rP[R_GP + k]; in.gpN[k] = rNg[R_GP + k];
        in.N[k] = m.nrm[k * nF + f];
        in.D[k] = m.du[k * nF + f];
        in.qw0[k] = m.qw[k * nF + f];
        in.qw1[k] = m.qw[(3 + k) * nF + f];
    }
    in.lw0 = m.lw[f];
    in.lw1 = m.lw[nF + f];
    in.rdelta = m.rdlt[f];
    if constexpr (sizeof(R) == 8) {
        for (int k = 0; k < 3; k++) in.Nt[k] = m.ntd[k * nF + f];
        in.ND = m.ntd[3 * nF + f];
    } else {
        // FP32 face kernels are bound by their loads, not by their (FP32) arithmetic: formed here
        in.ND = dot3(in.N, in.D);
        for (int k = 0; k < 3; k++) in.Nt[k] = in.N[k] - in.ND * in.D[k];
    }
}

// a face's column of a device tape (value k of face f at tape[k nF + f]; p = tape + f)
template <typename R>
struct TapeStore {
    R* p;
    size_t stride;
    __device__ __forceinline__ void put(int k, R x) const { p[(size_t)k * stride] = x; }
};
template <typename R>
struct TapeLoad {
    static constexpr bool kFull = true;
    const R* p;
    size_t stride;
    __device__ __forceinline__ R get(int k) const { return __ldg(p + (size_t)k * stride); }
};

// the geometry inputs of a face only (what the VJP reads besides the tape)
template <typename R>
__device__ __forceinline__ void load_face_geometry(const MeshDev<R>& m, int f, FaceIn<R>& in) {
    const size_t nF = m.nF;
    for (int k = 0; k < 3; k++) {
        in.N[k] = m.nrm[k * nF + f];
        in.D[k] = m.du[k * nF + f];
        in.qw0[k] = m.qw[k * nF + f];
        in.qw1[k] = m.qw[(3 + k) * nF + f];
    }
    in.lw0 = m.lw[f];
    in.lw1 = m.lw[nF + f];
    in.rdelta = m.rdlt[f];
    if constexpr (sizeof(R) == 8) {
        for (int k = 0; k < 3; k++) in.Nt[k] = m.ntd[k * nF + f];
        in.ND = m.ntd[3 * nF + f];
    } else {
        // FP32 face kernels are bound by their loads, not by their (FP32) arithmetic: formed here
        in.ND = dot3(in.N, in.D);
        for (int k = 0; k < 3; k++) in.Nt[k] = in.N[k] - in.ND * in.D[k];
    }
}

}  // namespace afvm
