// Device-side hex-mesh geometry and connectivity: the same arithmetic as the host builder
// (geometry.cpp, which restates adFVM/cpp/cmesh.cpp:3-270 and Mesh.createGhostCells,
// adFVM/mesh.py:758-819), one thread per face or cell, so that a mesh admitted by a serving
// process is built where it is used. This file is compiled with -fmad=false: every product
// and sum is rounded as in the host build (compiled with -ffp-contract=off), so the two
// agree to the last bit; double division and square root are IEEE-rounded on both.
//
// Connectivity without atomics in the result: faces claim slots of their cells with atomic
// counters, then each cell sorts its six faces by (own ? f : nFaces + f) - owned faces in face
// order, then neighbour faces in face order, the host builder's order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <vector>
#include "afvm.h"

namespace {

constexpr int TB = 256;
enum : int { E_COUNT = 1, E_OWNER = 2, E_POINT = 4, E_NEIGHBOUR = 8, E_SLOTS = 16 };

struct DevPatch {
    int startFace, nFaces, kind, nStart;   // nStart: start face of the cyclic partner
};

__global__ void k_check_and_claim(int nFaces, int nIF, int nIC, int nPoints, const int32_t* __restrict__ faces,
                                  const int32_t* __restrict__ owner, const int32_t* __restrict__ nbr,
                                  int* __restrict__ fill, int32_t* __restrict__ slots, int* __restrict__ err) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    const int32_t* fp = faces + 5 * (size_t)f;
    int bad = 0;
    if (fp[0] != 4) bad |= E_COUNT;
    for (int j = 1; j < 5; j++)
        if (fp[j] < 0 || fp[j] >= nPoints) bad |= E_POINT;
    int p = owner[f];
    if (p < 0 || p >= nIC) bad |= E_OWNER;
    int n = -1;
    if (f < nIF) {
        n = nbr[f];
        if (n < 0 || n >= nIC || n <= p) bad |= E_NEIGHBOUR;
    }
    if (bad) {
        atomicOr(err, bad);
        return;
    }
    int s = atomicAdd(fill + p, 1);
    if (s < 6) slots[6 * (size_t)p + s] = f;
    if (n >= 0) {
        s = atomicAdd(fill + n, 1);
        if (s < 6) slots[6 * (size_t)n + s] = f;
    }
}

__global__ void k_cell_faces(int nIC, int nFaces, const int32_t* __restrict__ owner, const int* __restrict__ fill,
                             const int32_t* __restrict__ slots, int32_t* __restrict__ cellFaces, int* __restrict__ err) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC) return;
    if (fill[c] != 6) {
        atomicOr(err, E_SLOTS);
        return;
    }
    long long key[6];
    for (int j = 0; j < 6; j++) {
        int f = slots[6 * (size_t)c + j];
        key[j] = (owner[f] == c) ? (long long)f : (long long)nFaces + f;
    }
    for (int i = 1; i < 6; i++) {          // insertion sort of six keys
        long long k = key[i];
        int j = i - 1;
        while (j >= 0 && key[j] > k) {
            key[j + 1] = key[j];
            j--;
        }
        key[j + 1] = k;
    }
    for (int j = 0; j < 6; j++) cellFaces[6 * (size_t)c + j] = (int32_t)(key[j] >= nFaces ? key[j] - nFaces : key[j]);
}

__device__ __forceinline__ const double* pt(const double* points, int id) { return points + 3 * (size_t)id; }

__global__ void k_face_geometry(int nFaces, const int32_t* __restrict__ faces, const double* __restrict__ points,
                                double* __restrict__ normals, double* __restrict__ faceCentres,
                                double* __restrict__ areas) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    const int32_t* fp = faces + 5 * (size_t)f;
    const double* a = pt(points, fp[1]);
    const double* b = pt(points, fp[2]);
    const double* c = pt(points, fp[3]);
    double v1[3], v2[3];
    for (int i = 0; i < 3; i++) {
        v1[i] = a[i] - b[i];
        v2[i] = b[i] - c[i];
    }
    double normal[3];
    normal[0] = v1[1] * v2[2] - v1[2] * v2[1];
    normal[1] = v1[2] * v2[0] - v1[0] * v2[2];
    normal[2] = v1[0] * v2[1] - v1[1] * v2[0];
    double Ns = sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
    for (int i = 0; i < 3; i++) normals[3 * (size_t)f + i] = normal[i] / Ns;
    double faceCentre[3] = {0, 0, 0};
    double sumCentre[3] = {0, 0, 0};
    double area = 0;
    for (int i = 0; i < 3; i++) {
        for (int j = 1; j < 5; j++) faceCentre[i] += pt(points, fp[j])[i];
        faceCentre[i] /= 4;
    }
    for (int j = 1; j < 5; j++) {
        const double* point = pt(points, fp[j]);
        const double* nextPoint = pt(points, fp[(j % 4) + 1]);
        double avgPoint[3] = {0, 0, 0};
        double N[3], w1[3], w2[3];
        for (int i = 0; i < 3; i++) {
            avgPoint[i] += (point[i] + nextPoint[i] + faceCentre[i]) / 3;
            w1[i] = nextPoint[i] - point[i];
            w2[i] = faceCentre[i] - point[i];
        }
        N[0] = w1[1] * w2[2] - w1[2] * w2[1];
        N[1] = w1[2] * w2[0] - w1[0] * w2[2];
        N[2] = w1[0] * w2[1] - w1[1] * w2[0];
        double s = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        area += s / 2;
        for (int i = 0; i < 3; i++) sumCentre[i] += s * avgPoint[i] / 2;
    }
    areas[f] = area;
    for (int i = 0; i < 3; i++) faceCentres[3 * (size_t)f + i] = sumCentre[i] / area;
}

__global__ void k_cell_geometry(int nIC, const int32_t* __restrict__ cellFaces, const double* __restrict__ normals,
                                const double* __restrict__ faceCentres, const double* __restrict__ areas,
                                double* __restrict__ cellCentres, double* __restrict__ volumes) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC) return;
    const int32_t* cf = cellFaces + 6 * (size_t)c;
    double vol = 0;
    double sumCentre[3] = {0, 0, 0};
    double cellCentre[3] = {0, 0, 0};
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 6; j++) cellCentre[i] += faceCentres[3 * (size_t)cf[j] + i];
        cellCentre[i] /= 6;
    }
    for (int j = 0; j < 6; j++) {
        int f = cf[j];
        const double* faceCentre = faceCentres + 3 * (size_t)f;
        double area = areas[f];
        const double* N = normals + 3 * (size_t)f;
        double v = 0;
        double avgCentre[3];
        for (int i = 0; i < 3; i++) {
            double height = cellCentre[i] - faceCentre[i];
            double areaN = area * N[i];
            v += areaN * height;
            avgCentre[i] = 3. / 4 * faceCentre[i] + 1. / 4 * cellCentre[i];
        }
        v = fabs(v / 3);
        vol += v;
        for (int i = 0; i < 3; i++) sumCentre[i] += v * avgCentre[i];
    }
    volumes[c] = vol;
    for (int i = 0; i < 3; i++) cellCentres[3 * (size_t)c + i] = sumCentre[i] / vol;
}

// ghost cells of the boundary faces (one per face, at cellStartFace = startFace - nIF + nIC)
__global__ void k_ghosts(int nFaces, int nIF, int nIC, int nPatches, const DevPatch* __restrict__ patches,
                         const int32_t* __restrict__ owner, const double* __restrict__ faceCentres,
                         int32_t* __restrict__ neighbour, double* __restrict__ cellCentres) {
    int f = nIF + blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    int ghost = f - nIF + nIC;
    int nb = 0;
    double cc[3] = {0, 0, 0};
    for (int q = 0; q < nPatches; q++) {
        DevPatch P = patches[q];
        if (f < P.startFace || f >= P.startFace + P.nFaces) continue;
        int i = f - P.startFace;
        nb = ghost;
        if (P.kind == AFVM_PATCH_CYCLIC) {
            int src = owner[P.nStart + i];
            for (int k = 0; k < 3; k++) {
                double transform = faceCentres[3 * (size_t)P.startFace + k] - faceCentres[3 * (size_t)P.nStart + k];
                cc[k] = transform + cellCentres[3 * (size_t)src + k];
            }
        } else {
            for (int k = 0; k < 3; k++) cc[k] = faceCentres[3 * (size_t)f + k];
        }
    }
    neighbour[f] = nb;
    for (int k = 0; k < 3; k++) cellCentres[3 * (size_t)ghost + k] = cc[k];
}

__global__ void k_face_weights(int nFaces, const int32_t* __restrict__ owner, const int32_t* __restrict__ neighbour,
                               const double* __restrict__ cellCentres, const double* __restrict__ faceCentres,
                               const double* __restrict__ normals, double* __restrict__ deltas,
                               double* __restrict__ deltasUnit, double* __restrict__ weights,
                               double* __restrict__ linearWeights, double* __restrict__ quadraticWeights) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    int p = owner[f];
    int n = neighbour[f];
    const double* P = cellCentres + 3 * (size_t)p;
    const double* N = cellCentres + 3 * (size_t)n;
    double delta[3];
    for (int i = 0; i < 3; i++) delta[i] = P[i] - N[i];
    double d = sqrt(delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
    deltas[f] = d;
    for (int i = 0; i < 3; i++) deltasUnit[3 * (size_t)f + i] = -delta[i] / d;
    const double* F = faceCentres + 3 * (size_t)f;
    const double* normal = normals + 3 * (size_t)f;
    double nD = 0, pD = 0;
    double nF[3], pF[3];
    for (int i = 0; i < 3; i++) {
        nF[i] = (F[i] - N[i]);
        pF[i] = (F[i] - P[i]);
        nD += nF[i] * normal[i];
        pD += pF[i] * normal[i];
    }
    nD = fabs(nD);
    pD = fabs(pD);
    weights[f] = nD / (nD + pD);
    double w1 = 0, w2 = 0;
    d = 0;
    for (int i = 0; i < 3; i++) {
        w1 += -delta[i] * pF[i];
        w2 += delta[i] * nF[i];
        d += delta[i] * delta[i];
    }
    w1 /= d;
    w2 /= d;
    linearWeights[2 * (size_t)f + 0] = w1 / 3;
    linearWeights[2 * (size_t)f + 1] = w2 / 3;
    for (int i = 0; i < 3; i++) {
        quadraticWeights[6 * (size_t)f + i] = 2. / 3 * pF[i] + 1. / 3 * (pF[i] + w1 * delta[i]);
        quadraticWeights[6 * (size_t)f + 3 + i] = 2. / 3 * nF[i] + 1. / 3 * (nF[i] - w2 * delta[i]);
    }
}

__global__ void k_cell_neighbours(int nIC, const int32_t* __restrict__ cellFaces, const int32_t* __restrict__ owner,
                                  const int32_t* __restrict__ neighbour, int32_t* __restrict__ cellOwner,
                                  int32_t* __restrict__ cellNeighbours, int32_t* __restrict__ matOp) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC) return;
    for (int j = 0; j < 6; j++) {
        size_t k = 6 * (size_t)c + j;
        int f = cellFaces[k];
        int p = owner[f];
        int n = neighbour[f];
        if (p != c) {
            cellOwner[k] = 0;
            cellNeighbours[k] = p;
            if (matOp) matOp[k] = p;
        } else {
            cellOwner[k] = 1;
            cellNeighbours[k] = n;
            if (matOp) matOp[k] = (n < nIC) ? n : -1;
        }
    }
}

__global__ void k_copy_int(int n, const int32_t* __restrict__ a, int32_t* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

inline int nb(long long n) { return (int)((n + TB - 1) / TB); }

}  // namespace

extern "C" int afvm_mesh_build_device(const afvm_mesh_in* in, afvm_mesh_out* out, void* stream) {
    if (!in || !out) return AFVM_ERR_BAD_ARG;
    const int nFaces = in->nFaces, nIF = in->nInternalFaces, nIC = in->nInternalCells;
    if (nFaces <= 0 || nIF < 0 || nIF > nFaces || nIC <= 0 || in->nPoints <= 0) return AFVM_ERR_BAD_ARG;
    if (!in->points || !in->faces || !in->owner || (nIF > 0 && !in->neighbour) || (in->nPatches > 0 && !in->patches))
        return AFVM_ERR_BAD_ARG;
    if (!out->normals || !out->faceCentres || !out->areas || !out->cellCentres || !out->volumes || !out->neighbour ||
        !out->deltas || !out->deltasUnit || !out->weights || !out->linearWeights || !out->quadraticWeights ||
        !out->cellFaces || !out->cellOwner || !out->cellNeighbours)
        return AFVM_ERR_BAD_ARG;
    // the patch table is small and read on the host, as the host builder checks it
    std::vector<DevPatch> pt(in->nPatches > 0 ? in->nPatches : 1);
    int nLocalCells = nIC;
    for (int q = 0; q < in->nPatches; q++) {
        const afvm_patch& P = in->patches[q];
        pt[q] = DevPatch{P.startFace, P.nFaces, P.kind, 0};
        if (P.nFaces == 0) continue;
        if (P.startFace < nIF || P.startFace + P.nFaces > nFaces || P.nFaces < 0) return AFVM_ERR_BAD_ARG;
        if (P.kind == AFVM_PATCH_PROCESSOR) return AFVM_ERR_UNSUPPORTED;
        nLocalCells += P.nFaces;
        if (P.kind == AFVM_PATCH_CYCLIC) {
            int np = P.neighbourPatch;
            if (np < 0 || np >= in->nPatches || in->patches[np].nFaces != P.nFaces) return AFVM_ERR_BAD_ARG;
            pt[q].nStart = in->patches[np].startFace;
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    int* scratch = nullptr;       // fill (nIC) + error flag
    int32_t* slots = nullptr;     // nIC x 6
    DevPatch* dp = nullptr;
    cudaError_t e = cudaMalloc(&scratch, sizeof(int) * ((size_t)nIC + 1));
    if (e == cudaSuccess) e = cudaMalloc(&slots, sizeof(int32_t) * 6 * (size_t)nIC);
    if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(DevPatch) * pt.size());
    int status = AFVM_OK;
    if (e != cudaSuccess) {
        status = AFVM_ERR_OOM;
    } else {
        int* fill = scratch;
        int* err = scratch + nIC;
        cudaMemcpyAsync(dp, pt.data(), sizeof(DevPatch) * pt.size(), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(scratch, 0, sizeof(int) * ((size_t)nIC + 1), s);
        k_check_and_claim<<<nb(nFaces), TB, 0, s>>>(nFaces, nIF, nIC, in->nPoints, in->faces, in->owner,
                                                    in->neighbour, fill, slots, err);
        k_cell_faces<<<nb(nIC), TB, 0, s>>>(nIC, nFaces, in->owner, fill, slots, out->cellFaces, err);
        int herr = 0;
        cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            status = AFVM_ERR_CUDA;
        } else if (herr & (E_OWNER | E_POINT | E_NEIGHBOUR)) {
            status = AFVM_ERR_BAD_ARG;         // an index out of range (its faces claimed no slots)
        } else if (herr) {
            status = AFVM_ERR_UNSUPPORTED;     // not a quad face / not a hex cell
        } else {
            k_face_geometry<<<nb(nFaces), TB, 0, s>>>(nFaces, in->faces, in->points, out->normals,
                                                      out->faceCentres, out->areas);
            k_cell_geometry<<<nb(nIC), TB, 0, s>>>(nIC, out->cellFaces, out->normals, out->faceCentres, out->areas,
                                                   out->cellCentres, out->volumes);
            if (nIF > 0) k_copy_int<<<nb(nIF), TB, 0, s>>>(nIF, in->neighbour, out->neighbour);
            if (nFaces > nIF)
                k_ghosts<<<nb(nFaces - nIF), TB, 0, s>>>(nFaces, nIF, nIC, in->nPatches, dp, in->owner,
                                                         out->faceCentres, out->neighbour, out->cellCentres);
            k_face_weights<<<nb(nFaces), TB, 0, s>>>(nFaces, in->owner, out->neighbour, out->cellCentres,
                                                     out->faceCentres, out->normals, out->deltas, out->deltasUnit,
                                                     out->weights, out->linearWeights, out->quadraticWeights);
            k_cell_neighbours<<<nb(nIC), TB, 0, s>>>(nIC, out->cellFaces, in->owner, out->neighbour, out->cellOwner,
                                                     out->cellNeighbours, out->cellNeighboursMatOp);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) status = AFVM_ERR_CUDA;
            out->nLocalCells = nLocalCells;
        }
    }
    cudaFree(dp);
    cudaFree(slots);
    cudaFree(scratch);
    return status;
}
