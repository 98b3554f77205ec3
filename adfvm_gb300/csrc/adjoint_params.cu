// Gradients of one adjoint step with respect to its parameters other than the state and the
// sources: the mesh tensors (the reference's parameters = 'mesh', Mesh.gradFields areas,
// volumesL, volumesR, weights, deltas, normals, deltasUnit, linearWeights, quadraticWeights,
// volumes; apps/adjoint.py:108-110, adFVM/mesh.py:28-31) and one boundary input (parameters =
// ('BCs', field, patch, key), apps/adjoint.py:111-118: a fixedValue 'value', a CBC_UPT U0 / T0 /
// p0, a CBC_TOTAL_PT direction / Tt / pt).
//
// The reference gets them from adpy's reverse mode over the whole step; here, per stage of the
// reverse sweep, two kernels add the stage's share once the stage's face records (fadj) and
// cell sums (cbar) exist:
//   k_param_face  faces: the face flux again and its VJP with the geometry adjoints (face.cuh,
//                 GeoBar), the div weights A/V_L, A/V_R (op.py:12-20), the Green-Gauss terms of
//                 the two adjacent cells (op.py:45-63), the ghost cells whose values depend on
//                 the normals (symmetryPlane, a CBC_TOTAL_PT direction taken from the normals)
//                 or on the boundary input, and the drag objective's face terms;
//   k_param_cell  cells: the 1/V of the Green-Gauss gradient and the kinetic-energy objective.
// Every output element is written by one thread, so the sums are deterministic. FP64 contexts.
#include <cuda_runtime.h>
#include "facedev.cuh"

namespace afvm {

// the adjoint of a ghost's five primitives: its face record's neighbour side plus the owner's
// gradient slot that reads it (as k_adj_cell2 assembles it), plus the drag objective's ghost
// terms on its objective stage
template <typename R>
__device__ __forceinline__ void ghost_bar(const MeshDev<R>& m, const Phys& P, const R* __restrict__ rec,
                                          const R* __restrict__ fadj, const R* __restrict__ cbar, int f, bool drag,
                                          double obja, const double* __restrict__ objSeed, R* gp) {
    const size_t n = m.nIC;
    int g = f - m.nIF;
    int o = m.own[f];
    int s = m.gslot[g];
    const R* r = fadj + (size_t)f * 40;
    for (int k = 0; k < 5; k++) gp[k] = r[20 + k];
    R sn[3] = {m.gsn[(3 * s) * n + o], m.gsn[(3 * s + 1) * n + o], m.gsn[(3 * s + 2) * n + o]};
    R w = m.gw[s * n + o];
    const R* G = cbar + (size_t)o * 20 + 5;
    R rv = m.rvol[o];
    for (int i = 0; i < 5; i++) gp[i] += w * (rv * (G[3 * i] * sn[0] + G[3 * i + 1] * sn[1] + G[3 * i + 2] * sn[2]));
    if (objSeed)
        for (int k = 0; k < 5; k++) gp[k] += (R)(obja * objSeed[(size_t)(m.nIC + g) * 5 + k]);
    if (drag) {
        const R* rg = rec + (size_t)(m.nIC + g) * REC;
        const R* ro = rec + (size_t)o * REC;
        double T0 = rg[R_T], U0 = rg[0], U0i = ro[0];
        double A = m.area[f], dl = m.dlt[f], nx = m.nrm[f];
        double mu = viscosity<double>(P, T0);
        double dmu = (P.muModel == AFVM_MU_SUTHERLAND) ? mu * (1.5 / T0 - 1.0 / (T0 + P.muTs)) : 0.0;
        gp[R_P] += (R)(obja * nx * A);
        gp[R_T] += (R)(-obja * dmu * (U0 - U0i) / dl * A);
        gp[0] += (R)(-obja * mu / dl * A);
    }
}

template <typename R, typename S>
__global__ void __launch_bounds__(FLUX_BLOCK) k_param_face(MeshDev<R> m, Phys P, const R* __restrict__ rec, R coef,
                                                           const S* __restrict__ ar, const S* __restrict__ au,
                                                           const S* __restrict__ ae, const R* __restrict__ fadj,
                                                           const R* __restrict__ cbar, int inviscid, int dragStage,
                                                           int objStart, int objN, double obja,
                                                           const double* __restrict__ objSeed, ParamDev pd) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nF) return;
    const bool internal = f < m.nIF;
    const int kind = internal ? FACE_INTERNAL : (int)m.fkind[f - m.nIF];
    const int iP = m.own[f], iN = m.nbr[f];
    // adjoint of the residual of the two cells (the stage update is u - beta dt (R - S))
    R rbP[5] = {coef * R(ar[iP]), coef * R(au[3 * iP]), coef * R(au[3 * iP + 1]), coef * R(au[3 * iP + 2]),
                coef * R(ae[iP])};
    R rbN[5] = {R(0), R(0), R(0), R(0), R(0)};
    if (internal) {
        rbN[0] = coef * R(ar[iN]);
        for (int k = 0; k < 3; k++) rbN[1 + k] = coef * R(au[3 * iN + k]);
        rbN[4] = coef * R(ae[iN]);
    }
    const R wp = m.wpf[f], wn = internal ? m.wnf[f] : R(0);
    R Fb[5];
    for (int k = 0; k < 5; k++) Fb[k] = rbP[k] * wp - rbN[k] * wn;
    FaceIn<R> in;
    load_face<R>(m, rec, f, in);
    R F[5], maxaF;
    face_flux<R>(P, kind, inviscid != 0, in, F, maxaF);
    FaceBar<R> b;
    zero_bar(b);
    GeoBar<R> geo;
    zero_geo(geo);
    face_vjp<R>(P, kind, inviscid != 0, in, Fb, b, &geo);
    const R A = m.area[f];
    // op.div: + F A/V_L into the owner, - F A/V_R into the internal neighbour (1/V_L, 1/V_R from
    // the weights A/V_L, A/V_R of the volumesL / volumesR inputs)
    R sP = R(0), sN = R(0);
    for (int k = 0; k < 5; k++) { sP += rbP[k] * F[k]; sN += rbN[k] * F[k]; }
    R rA = R(1) / A;
    R areasb = sP * (wp * rA);
    R volLb = -sP * (wp * wp * rA);
    R volRb = R(0);
    if (internal) {
        areasb -= sN * (wn * rA);
        volRb = sN * (wn * wn * rA);
    }
    // the Green-Gauss gradient divides by the cells' volumes
    const R rvP = m.rvol[iP];
    const R rvN = internal ? m.rvol[iN] : R(0);
    // op.gradCell: phiF (x) (A N) / V_P into the owner's gradient, phiF (x) (-A N) / V_N into an
    // internal neighbour's, phiF = w phi_P + (1 - w) phi_N (the face value both slots form)
    R w = m.wts[f];
    R phiP[5] = {in.UP[0], in.UP[1], in.UP[2], in.TP, in.pP};
    R phiN[5] = {in.UN[0], in.UN[1], in.UN[2], in.TN, in.pN};
    R N[3] = {in.N[0], in.N[1], in.N[2]};
    R nb[3] = {R(0), R(0), R(0)};
    R wb = R(0);
    for (int side = 0; side < (internal ? 2 : 1); side++) {
        const R* G = cbar + (size_t)(side == 0 ? iP : iN) * 20 + 5;
        R sc = side == 0 ? rvP : -rvN;          // +1/V_P or -1/V_N
        R Sh[3] = {R(0), R(0), R(0)};
        R dphiGN = R(0);
        for (int i = 0; i < 5; i++) {
            R phiF = w * phiP[i] + (R(1) - w) * phiN[i];
            R GN = G[3 * i] * N[0] + G[3 * i + 1] * N[1] + G[3 * i + 2] * N[2];
            for (int j = 0; j < 3; j++) Sh[j] += phiF * G[3 * i + j];
            dphiGN += (phiP[i] - phiN[i]) * GN;
        }
        areasb += sc * (Sh[0] * N[0] + Sh[1] * N[1] + Sh[2] * N[2]);
        for (int j = 0; j < 3; j++) nb[j] += sc * A * Sh[j];
        wb += sc * A * dphiGN;
    }
    R dltb = -geo.rdelta * m.rdlt[f] * m.rdlt[f];
    // ghost cells: their values as functions of the normals and of the boundary input
    if (!internal) {
        const int g = f - m.nIF;
        const int gk = m.gkind[g];
        const int kU = gk & 7;
        const bool drag = dragStage && f >= objStart && f < objStart + objN;
        const bool dirN = kU == GK_TOTALPT && pd.gdirn && pd.gdirn[g];
        const bool isBC = pd.bcN > 0 && f >= pd.bcStart && f < pd.bcStart + pd.bcN;
        if (kU == GK_SYM || dirN || isBC || drag) {
            R gp[5];
            ghost_bar<R>(m, P, rec, fadj, cbar, f, drag, obja, objSeed, gp);
            const R* rs = rec + (size_t)m.gsrc[g] * REC;     // the ghost's source cell
            R U[3] = {rs[0], rs[1], rs[2]};
            if (kU == GK_SYM) {
                // U_g = U - (U.n) n
                R gun = gp[0] * N[0] + gp[1] * N[1] + gp[2] * N[2];
                R un = U[0] * N[0] + U[1] * N[1] + U[2] * N[2];
                for (int j = 0; j < 3; j++) nb[j] += -U[j] * gun - un * gp[j];
            }
            R d[3] = {m.gval[g], m.gval[(size_t)m.nG + g], m.gval[2 * (size_t)m.nG + g]};
            // CBC_TOTAL_PT: U_g = (U.d) d, T_g = Tt - (U.d)^2 / (2 Cp), p_g = pt (T / Tt)^(g/(g-1))
            R Un = U[0] * d[0] + U[1] * d[1] + U[2] * d[2];
            R gud = gp[0] * d[0] + gp[1] * d[1] + gp[2] * d[2];
            R dirb[3];
            for (int j = 0; j < 3; j++) dirb[j] = U[j] * gud + Un * gp[j] - gp[R_T] * Un * U[j] / consts<R>(P).Cp;
            if (dirN)
                for (int j = 0; j < 3; j++) nb[j] += dirb[j];
            if (isBC) {
                int i = f - pd.bcStart;
                if (kU == GK_TOTALPT) {
                    R Tt = m.gval[3 * (size_t)m.nG + g], pt = m.gval[4 * (size_t)m.nG + g];
                    R kap = consts<R>(P).ggm1;
                    R ratio = pow(rs[R_T] / Tt, kap);
                    if (pd.bcField == 0)
                        for (int j = 0; j < 3; j++) pd.bc[3 * (size_t)i + j] += dirb[j];
                    else if (pd.bcField == 1)
                        pd.bc[i] += gp[R_T] - gp[R_P] * kap * pt * ratio / Tt;
                    else
                        pd.bc[i] += gp[R_P] * ratio;
                } else if (pd.bcField == 0) {
                    for (int j = 0; j < 3; j++) pd.bc[3 * (size_t)i + j] += gp[j];
                } else {
                    pd.bc[i] += gp[pd.bcField == 1 ? R_T : R_P];
                }
            }
            if (drag) {
                // drag = sum (p0 n_x - mu(T0) (U0_x - U0i_x) / delta) A over the objective patch
                const R* rg = rec + (size_t)iN * REC;
                double p0 = rg[R_P], T0 = rg[R_T], U0 = rg[0], U0i = rs[0];
                double mu = viscosity<double>(P, T0);
                double dl = m.dlt[f];
                areasb += (R)(obja * (p0 * (double)N[0] - mu * (U0 - U0i) / dl));
                nb[0] += (R)(obja * p0 * (double)A);
                dltb += (R)(obja * mu * (U0 - U0i) / (dl * dl) * (double)A);
            }
        }
    }
    if (pd.areas) pd.areas[f] += areasb;
    if (pd.volL) pd.volL[f] += volLb;
    if (pd.volR && internal) pd.volR[f] += volRb;
    if (pd.wts) pd.wts[f] += wb;
    if (pd.dlt) pd.dlt[f] += dltb;
    if (pd.nrm)
        for (int j = 0; j < 3; j++) pd.nrm[3 * (size_t)f + j] += nb[j] + geo.N[j];
    if (pd.du)
        for (int j = 0; j < 3; j++) pd.du[3 * (size_t)f + j] += geo.D[j];
    if (pd.lw) { pd.lw[2 * (size_t)f] += geo.lw0; pd.lw[2 * (size_t)f + 1] += geo.lw1; }
    if (pd.qw)
        for (int j = 0; j < 3; j++) { pd.qw[6 * (size_t)f + j] += geo.qw0[j]; pd.qw[6 * (size_t)f + 3 + j] += geo.qw1[j]; }
}

// volumes: the gradient's 1/V (grad = sum / V) and the kinetic-energy objective (sum 0.5 rho |U|^2 V)
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_param_cell(MeshDev<R> m, Phys P, const R* __restrict__ rec,
                                                      const R* __restrict__ cbar, int keStage, double obja,
                                                      double* __restrict__ vol) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.nIC) return;
    const R* G = cbar + (size_t)c * 20 + 5;
    const R* rc = rec + (size_t)c * REC;
    R s = R(0);
    for (int k = 0; k < 15; k++) s += G[k] * rc[R_GU + k];
    double vb = -(double)(s * m.rvol[c]);
    if (keStage) {
        double U[3] = {rc[0], rc[1], rc[2]}, T = rc[R_T], p = rc[R_P];
        double rho = p / ((P.Cv * T) * P.gm1);
        vb += obja * 0.5 * rho * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    }
    vol[c] += vb;
}

template <typename R, typename S>
void launch_param_grads(Ctx* c, const ParamDev& pd, const R* rec, R coef, const S* ar, const S* au, const S* ae,
                        bool objectiveStage, double obja, cudaStream_t s) {
    const MeshDev<R>& m = meshOf<R>(c);
    const Phys& P = c->phys;
    int inviscid = (P.muModel == AFVM_MU_CONSTANT && P.mu0 == 0.0) ? 1 : 0;
    ProfScope ps(c, KID_ADJ_MISC, s);
    int nbF = (m.nF + FLUX_BLOCK - 1) / FLUX_BLOCK;
    int drag = objectiveStage && c->objective == AFVM_OBJ_DRAG;
    const double* seed = objectiveStage ? c->objSeed : nullptr;
    k_param_face<R, S><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, coef, ar, au, ae, (const R*)c->fadj, (const R*)c->cbar,
                                                  inviscid, drag, c->objStart, c->objN, obja, seed, pd);
    if (pd.vol) {
        int ke = objectiveStage && c->objective == AFVM_OBJ_KINETIC_ENERGY;
        k_param_cell<R><<<nblocks(m.nIC), BLOCK, 0, s>>>(m, P, rec, (const R*)c->cbar, ke, obja, pd.vol);
    }
}

template void launch_param_grads<double, double>(Ctx*, const ParamDev&, const double*, double, const double*,
                                                 const double*, const double*, bool, double, cudaStream_t);

}  // namespace afvm
