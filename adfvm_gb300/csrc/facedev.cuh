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

// the 55 inputs of one face: primitives and gradients of both sides, geometry. ownRec: the
// owner's record where the caller staged it (shared memory), else NULL
template <typename R>
__device__ __forceinline__ void load_face(const MeshDev<R>& m, const R* __restrict__ rec, int f, FaceIn<R>& in,
                                          const R* ownRec = nullptr) {
    const size_t nF = m.nF;
    int iP = m.own[f], iN = m.nbr[f];
    int iNg = (f < m.nIF) ? iN : m.gsrc[iN - m.nIC];   // ghost gradient = copy of its source
    R rP[REC], rN[REC], rNg[REC];
    if (ownRec) {
        for (int k = 0; k < REC; k++) rP[k] = ownRec[k];
    } else {
        load_vec(rec + (size_t)iP * REC, rP, REC);
    }
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
}

// FP32 face kernels: the owners of a block's internal faces (faces sorted by owner) are a
// short run of consecutive cells, whose records the block copies into shared memory with
// coalesced 16-byte loads before its threads read them (each record is read by about three
// faces). Returns the staged record of face f's owner, or NULL (face outside the run, a
// boundary face, a mesh whose faces are not sorted by owner) for a global load. All threads
// of the block must call it (it synchronises).
template <typename R>
__device__ __forceinline__ const R* stage_owner_records(const MeshDev<R>& m, const R* __restrict__ rec, int f0,
                                                        int nFaces, int f, R* sOwn) {
    const int fl = min(f0 + nFaces, m.nIF) - 1;        // the block's last internal face
    int o0 = 0, no = 0;
    if (f0 <= fl) {
        o0 = m.own[f0];
        no = m.own[fl] - o0 + 1;
    }
    const bool ok = no > 0 && no <= nFaces;             // uniform over the block
    if (ok) {
        using V = typename Vec16<R>::type;
        const V* src = reinterpret_cast<const V*>(rec + (size_t)o0 * REC);
        V* dst = reinterpret_cast<V*>(sOwn);
        const int nv = no * (REC * (int)sizeof(R) / 16);
        for (int i = threadIdx.x; i < nv; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    __syncthreads();
    if (!ok || f > fl) return nullptr;
    const int o = m.own[f] - o0;
    return (o >= 0 && o < no) ? sOwn + (size_t)o * REC : nullptr;
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
}

}  // namespace afvm
