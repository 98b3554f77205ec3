// Device-side loads of the face inputs from the cell records and the mesh tables.
#pragma once
#include "ctx.cuh"
#include "face.cuh"

namespace afvm {

// the 55 inputs of one face: primitives and gradients of both sides, geometry
template <typename R>
__device__ __forceinline__ void load_face(const MeshDev<R>& m, const R* __restrict__ rec, int f, FaceIn<R>& in) {
    const size_t nF = m.nF;
    int iP = m.own[f], iN = m.nbr[f];
    int iNg = (f < m.nIF) ? iN : m.gsrc[iN - m.nIC];   // ghost gradient = copy of its source
    const R* rP = rec + (size_t)iP * REC;
    const R* rN = rec + (size_t)iN * REC;
    const R* rNg = rec + (size_t)iNg * REC;
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
    in.delta = m.dlt[f];
}

}  // namespace afvm
