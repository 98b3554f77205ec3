// Host-side hex-mesh geometry and connectivity builder.
//
// Restates, operation for operation, the arithmetic of the reference's native mesh
// builder so that connectivity is bit-identical and geometry agrees to the last bit when
// both are compiled without floating-point contraction:
//   cellFaces                  adFVM/cpp/cmesh.cpp:3-19   (Mesh::buildBeforeWrite)
//   normals, centres, areas    adFVM/cpp/cmesh.cpp:70-121
//   cell centres, volumes      adFVM/cpp/cmesh.cpp:128-163
//   ghost cells                adFVM/mesh.py:758-819      (Mesh.createGhostCells, 1 rank)
//   deltas, weights            adFVM/cpp/cmesh.cpp:178-233
//   cellOwner, cellNeighbours  adFVM/cpp/cmesh.cpp:240-269
// This file must be compiled with -ffp-contract=off (the build recipe passes it).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "afvm.h"

namespace {

inline const double* pt(const double* points, int id) { return points + 3 * (size_t)id; }

}  // namespace

extern "C" int afvm_mesh_build(const afvm_mesh_in* in, afvm_mesh_out* out) {
    if (!in || !out) return AFVM_ERR_BAD_ARG;
    const int nFaces = in->nFaces, nIF = in->nInternalFaces, nIC = in->nInternalCells;
    const int nBF = nFaces - nIF;
    const int nCells = nIC + nBF;
    if (nFaces <= 0 || nIF < 0 || nIF > nFaces || nIC <= 0) return AFVM_ERR_BAD_ARG;
    const int* faces = in->faces;
    const int* owner = in->owner;
    const double* points = in->points;
    for (int f = 0; f < nFaces; f++) {
        if (faces[5 * (size_t)f] != 4) return AFVM_ERR_UNSUPPORTED;  // quads only
        if (owner[f] < 0 || owner[f] >= nIC) return AFVM_ERR_BAD_ARG;
        for (int j = 1; j < 5; j++) {
            int p = faces[5 * (size_t)f + j];
            if (p < 0 || p >= in->nPoints) return AFVM_ERR_BAD_ARG;
        }
    }
    for (int f = 0; f < nIF; f++) {
        int n = in->neighbour[f];
        if (n < 0 || n >= nIC || n <= owner[f]) return AFVM_ERR_BAD_ARG;
    }

    // --- cellFaces: owned faces in face order, then neighbour faces in face order.
    int* cellFaces = out->cellFaces;
    std::vector<int> fill(nIC, 0);
    for (int f = 0; f < nFaces; f++) {
        int p = owner[f];
        if (fill[p] >= 6) return AFVM_ERR_UNSUPPORTED;  // hex cells only
        cellFaces[6 * (size_t)p + fill[p]++] = f;
    }
    for (int f = 0; f < nIF; f++) {
        int p = in->neighbour[f];
        if (fill[p] >= 6) return AFVM_ERR_UNSUPPORTED;
        cellFaces[6 * (size_t)p + fill[p]++] = f;
    }
    for (int c = 0; c < nIC; c++)
        if (fill[c] != 6) return AFVM_ERR_UNSUPPORTED;

    // --- face normals, centres, areas
    double* normals = out->normals;
    double* faceCentres = out->faceCentres;
    double* areas = out->areas;
#pragma omp parallel for
    for (int f = 0; f < nFaces; f++) {
        const int* fp = faces + 5 * (size_t)f;
        const double* a = pt(points, fp[1]);
        const double* b = pt(points, fp[2]);
        const double* c = pt(points, fp[3]);
        double v1[3], v2[3];
        for (int i = 0; i < 3; i++) {
            v1[i] = a[i] - b[i];
            v2[i] = b[i] - c[i];
        }
        double* normal = normals + 3 * (size_t)f;
        normal[0] = v1[1] * v2[2] - v1[2] * v2[1];
        normal[1] = v1[2] * v2[0] - v1[0] * v2[2];
        normal[2] = v1[0] * v2[1] - v1[1] * v2[0];
        double Ns = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
        for (int i = 0; i < 3; i++) normal[i] /= Ns;
        double* sumCentre = faceCentres + 3 * (size_t)f;
        double faceCentre[3] = {0, 0, 0};
        double area = 0;
        for (int i = 0; i < 3; i++) {
            sumCentre[i] = 0;
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
            double s = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
            area += s / 2;
            for (int i = 0; i < 3; i++) sumCentre[i] += s * avgPoint[i] / 2;
        }
        areas[f] = area;
        for (int i = 0; i < 3; i++) sumCentre[i] /= area;
    }

    // --- cell centres and volumes (6 pyramids about the face-centre average)
    double* cellCentres = out->cellCentres;   // nCells x 3 (ghost rows filled below)
    double* volumes = out->volumes;
#pragma omp parallel for
    for (int c = 0; c < nIC; c++) {
        double vol = 0;
        double* sumCentre = cellCentres + 3 * (size_t)c;
        double cellCentre[3] = {0, 0, 0};
        for (int i = 0; i < 3; i++) {
            sumCentre[i] = 0;
            for (int j = 0; j < 6; j++) cellCentre[i] += faceCentres[3 * (size_t)cellFaces[6 * (size_t)c + j] + i];
            cellCentre[i] /= 6;
        }
        for (int j = 0; j < 6; j++) {
            int f = cellFaces[6 * (size_t)c + j];
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
            v = std::fabs(v / 3);
            vol += v;
            for (int i = 0; i < 3; i++) sumCentre[i] += v * avgCentre[i];
        }
        volumes[c] = vol;
        for (int i = 0; i < 3; i++) sumCentre[i] /= vol;
    }

    // --- ghost cells: one per boundary face, at cellStartFace = startFace - nIF + nIC
    int* neighbour = out->neighbour;   // nFaces
    for (int f = 0; f < nIF; f++) neighbour[f] = in->neighbour[f];
    for (int f = nIF; f < nFaces; f++) neighbour[f] = 0;
    for (size_t i = 3 * (size_t)nIC; i < 3 * (size_t)nCells; i++) cellCentres[i] = 0;
    int nLocalCells = nIC;
    for (int pi = 0; pi < in->nPatches; pi++) {
        const afvm_patch& patch = in->patches[pi];
        int startFace = patch.startFace, nF = patch.nFaces;
        if (nF == 0) continue;
        if (startFace < nIF || startFace + nF > nFaces) return AFVM_ERR_BAD_ARG;
        if (patch.kind == AFVM_PATCH_PROCESSOR) return AFVM_ERR_UNSUPPORTED;  // one rank
        nLocalCells += nF;
        int cellStart = startFace - nIF + nIC;
        for (int i = 0; i < nF; i++) neighbour[startFace + i] = cellStart + i;
        if (patch.kind == AFVM_PATCH_CYCLIC) {
            int np = patch.neighbourPatch;
            if (np < 0 || np >= in->nPatches || in->patches[np].nFaces != nF) return AFVM_ERR_BAD_ARG;
            int nStart = in->patches[np].startFace;
            double transform[3];
            for (int k = 0; k < 3; k++)
                transform[k] = faceCentres[3 * (size_t)startFace + k] - faceCentres[3 * (size_t)nStart + k];
            for (int i = 0; i < nF; i++) {
                int src = owner[nStart + i];
                for (int k = 0; k < 3; k++)
                    cellCentres[3 * (size_t)(cellStart + i) + k] = transform[k] + cellCentres[3 * (size_t)src + k];
            }
        } else {
            for (int i = 0; i < nF; i++)
                for (int k = 0; k < 3; k++)
                    cellCentres[3 * (size_t)(cellStart + i) + k] = faceCentres[3 * (size_t)(startFace + i) + k];
        }
    }
    out->nLocalCells = nLocalCells;

    // --- deltas and interpolation weights
#pragma omp parallel for
    for (int f = 0; f < nFaces; f++) {
        int p = owner[f];
        int n = neighbour[f];
        const double* P = cellCentres + 3 * (size_t)p;
        const double* N = cellCentres + 3 * (size_t)n;
        double delta[3];
        for (int i = 0; i < 3; i++) delta[i] = P[i] - N[i];
        double d = std::sqrt(delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
        out->deltas[f] = d;
        for (int i = 0; i < 3; i++) out->deltasUnit[3 * (size_t)f + i] = -delta[i] / d;
        const double* F = faceCentres + 3 * (size_t)f;
        double nD = 0, pD = 0;
        const double* normal = normals + 3 * (size_t)f;
        double nF[3], pF[3];
        for (int i = 0; i < 3; i++) {
            nF[i] = (F[i] - N[i]);
            pF[i] = (F[i] - P[i]);
            nD += nF[i] * normal[i];
            pD += pF[i] * normal[i];
        }
        nD = std::fabs(nD);
        pD = std::fabs(pD);
        out->weights[f] = nD / (nD + pD);
        double w1 = 0, w2 = 0;
        d = 0;
        for (int i = 0; i < 3; i++) {
            w1 += -delta[i] * pF[i];
            w2 += delta[i] * nF[i];
            d += delta[i] * delta[i];
        }
        w1 /= d;
        w2 /= d;
        out->linearWeights[2 * (size_t)f + 0] = w1 / 3;
        out->linearWeights[2 * (size_t)f + 1] = w2 / 3;
        for (int i = 0; i < 3; i++) {
            out->quadraticWeights[6 * (size_t)f + i] = 2. / 3 * pF[i] + 1. / 3 * (pF[i] + w1 * delta[i]);
            out->quadraticWeights[6 * (size_t)f + 3 + i] = 2. / 3 * nF[i] + 1. / 3 * (nF[i] - w2 * delta[i]);
        }
    }

    // --- per-cell ownership flags and neighbour cells, in cellFaces order
#pragma omp parallel for
    for (int c = 0; c < nIC; c++) {
        for (int j = 0; j < 6; j++) {
            int f = cellFaces[6 * (size_t)c + j];
            int p = owner[f];
            int n = neighbour[f];
            if (p != c) {
                out->cellOwner[6 * (size_t)c + j] = 0;
                out->cellNeighbours[6 * (size_t)c + j] = p;
                if (out->cellNeighboursMatOp) out->cellNeighboursMatOp[6 * (size_t)c + j] = p;
            } else {
                out->cellOwner[6 * (size_t)c + j] = 1;
                out->cellNeighbours[6 * (size_t)c + j] = n;
                if (out->cellNeighboursMatOp) out->cellNeighboursMatOp[6 * (size_t)c + j] = (n < nIC) ? n : -1;
            }
        }
    }
    return AFVM_OK;
}
