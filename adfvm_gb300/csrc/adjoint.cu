// Discrete adjoint of one SSP-RK3 step with dt held fixed (the per-step VJP of the reference's
// adjoint sweep, apps/adjoint.py:101-126 and 268-291).
//
// Forward u0 -> u1 -> u2 -> u3 (timestep.py:27-55) is recomputed, then the three stages are
// reversed. For stage i with output adjoint abar_{i+1}, the residual seed is
// Rbar = -beta_ii dt abar_{i+1}, and J_R(u_i)^T Rbar is formed by three kernels, all gathers
// (no atomics, so every result is bitwise reproducible):
//   k_adj_flux   faces: Fbar = Rbar_P A/V_P - Rbar_N A/V_N, then the hand-derived face VJP
//                (face.cuh) -> a 40-value record per face (primitive/gradient adjoints of
//                both sides)
//   k_adj_cell1  cells: sum of the face records of the cell's 6 faces (its own side) and of the
//                gradient adjoints of the ghost cells it is the source of
//   k_adj_cell2  cells: transpose of the Green-Gauss gradient (own slots and, through the
//                back-slot weights, the neighbours'), ghost boundary conditions transposed,
//                objective gradient (stage 1), primitive VJP and the SSP-RK reverse update.
#include <cuda_runtime.h>
#include <type_traits>
#include "facedev.cuh"
#include "vane.cuh"

namespace afvm {

// face adjoint record, one side after the other: owner side [prims 5 | grads 15], then the
// neighbour (ghost) side [prims 5 | grads 15]
constexpr int FADJ = 40;
constexpr int CBAR = 20;   // per cell: primitive adjoint (5) then gradient adjoint (15)

// one face's record of k_adj_flux into row[0..39]; TAPED: the forward values of a
// non-boundary face come from its tape column instead of a re-evaluation of the face flux
template <typename R, typename S, bool TAPED>
__device__ __forceinline__ void adj_face(const MeshDev<R>& m, const Phys& P, const R* __restrict__ rec, R coef,
                                         const S* __restrict__ ar, const S* __restrict__ au,
                                         const S* __restrict__ ae, int inviscid, int f, R* row,
                                         const R* __restrict__ tape) {
    int kind = (f < m.nIF) ? FACE_INTERNAL : (int)m.fkind[f - m.nIF];
    int iP = m.own[f];
    // Fbar = coef (abar_P A/V_L - abar_N A/V_R), coef folded into the two weights
    R wp = coef * m.wpf[f];
    R Fb[5];
    Fb[0] = R(ar[iP]) * wp;
    for (int k = 0; k < 3; k++) Fb[1 + k] = R(au[3 * iP + k]) * wp;
    Fb[4] = R(ae[iP]) * wp;
    if (f < m.nIF) {
        int iN = m.nbr[f];
        R wn = coef * m.wnf[f];
        Fb[0] = Fb[0] - R(ar[iN]) * wn;
        for (int k = 0; k < 3; k++) Fb[1 + k] = Fb[1 + k] - R(au[3 * iN + k]) * wn;
        Fb[4] = Fb[4] - R(ae[iN]) * wn;
    }
    FaceIn<R> in;
    FaceBar<R> b;
    zero_bar(b);
    if (TAPED && kind != FACE_BOUNDARY) {
        load_face_geometry<R>(m, f, in);
        face_vjp_t<R>(P, kind, inviscid != 0, in, TapeLoad<R>{tape + f, (size_t)m.nF}, Fb, b);
    } else {
        load_face<R>(m, rec, f, in);
        if constexpr (kGauge<R>) {
            // the VJP differentiates the absolute-form flux (the same function of the state as
            // the gauge form the forward evaluates)
            in.TP = rec_abs_T<R>(P, in.TP); in.TN = rec_abs_T<R>(P, in.TN);
            in.pP = rec_abs_p<R>(P, in.pP); in.pN = rec_abs_p<R>(P, in.pN);
        }
        face_vjp<R>(P, kind, inviscid != 0, in, Fb, b);
    }
    const R* src = &b.UP[0];
    R v[FADJ];
    for (int k = 0; k < 5; k++) { v[k] = src[k]; v[20 + k] = src[5 + k]; }
    for (int k = 0; k < 15; k++) { v[5 + k] = src[10 + k]; v[25 + k] = src[25 + k]; }
    stage_row<R, FADJ>(row, v);
}

template <typename R, typename S, bool TAPED>
__global__ void __launch_bounds__(FLUX_BLOCK, sizeof(R) == 8 ? 3 : 5) k_adj_flux(MeshDev<R> m, Phys P, const R* __restrict__ rec, R coef,
                                                    const S* __restrict__ ar, const S* __restrict__ au,
                                                    const S* __restrict__ ae, R* __restrict__ fadj, int inviscid,
                                                    const R* __restrict__ tape) {
    // the block's 40-value face records are staged here and written out contiguously: one
    // thread's 40 scalar stores at a 40-value stride would touch a new 32-byte sector each and
    // load L2 with eight partial writes per sector
    __shared__ __align__(16) R stage[FLUX_BLOCK * FADJ];
    const int f0 = blockIdx.x * FLUX_BLOCK;
    const int f = f0 + threadIdx.x;
    if (f < m.nF) adj_face<R, S, TAPED>(m, P, rec, coef, ar, au, ae, inviscid, f, stage + threadIdx.x * FADJ, tape);
    __syncthreads();
    store_staged<R, FADJ, FLUX_BLOCK>(fadj, f0, min(FLUX_BLOCK, m.nF - f0), stage);
}

// one cell's sum of its faces' adjoint records (and of the ghosts whose gradient is its own)
template <typename R>
__device__ __forceinline__ void adj_cell_gather(const MeshDev<R>& m, const R* __restrict__ fadj, int c, R* row) {
    const size_t n = m.nIC;
    // the first slot initialises the sums: adding it to zeros would cost 20 more adds (FP64
    // pipe issues in double) and changes nothing but the sign of a zero
    R acc[CBAR];
    for (int s = 0; s < 6; s++) {
        int e = m.accf[s * n + c];
        bool ownerSide = e >= 0;
        int f = ownerSide ? e : ~e;
        R v[CBAR];
        load_vec(fadj + (size_t)f * FADJ + (ownerSide ? 0 : CBAR), v, CBAR);
        if (s == 0)
            for (int k = 0; k < CBAR; k++) acc[k] = v[k];
        else
            for (int k = 0; k < CBAR; k++) acc[k] += v[k];
    }
    // gradient adjoints of the ghosts whose gradient is a copy of this cell's
    for (int q = m.gsStart[c]; q < m.gsStart[c + 1]; q++) {
        int g = m.gsList[q];
        const R* r = fadj + (size_t)(m.nIF + g) * FADJ;
        for (int k = 0; k < 15; k++) acc[5 + k] += r[25 + k];
    }
    stage_row<R, CBAR>(row, acc);
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_adj_cell1(MeshDev<R> m, const R* __restrict__ fadj, R* __restrict__ cbar) {
    __shared__ __align__(16) R stage[BLOCK * CBAR];
    const int c0 = blockIdx.x * BLOCK;
    const int c = c0 + threadIdx.x;
    if (c < m.nIC) adj_cell_gather<R>(m, fadj, c, stage + threadIdx.x * CBAR);
    __syncthreads();
    if (c0 < m.nIC) store_staged<R, CBAR, BLOCK>(cbar, c0, min(BLOCK, m.nIC - c0), stage);
}


// phiFbar_i = rv * sum_j G[i][j] sn_j  (transpose of grad += phiF (x) S N', scaled by 1/V)
template <typename R>
__device__ __forceinline__ void phi_bar(const R* G, const R* sn, R rv, R* pb) {
    for (int i = 0; i < 5; i++) pb[i] = rv * (G[3 * i] * sn[0] + G[3 * i + 1] * sn[1] + G[3 * i + 2] * sn[2]);
}

template <typename R, typename S, int STAGE>
__global__ void __launch_bounds__(BLOCK) k_adj_cell2(MeshDev<R> m, Phys P, const R* __restrict__ rec,
                                                     const R* __restrict__ fadj, const R* __restrict__ cbar,
                                                     const S* __restrict__ ur, const S* __restrict__ uu,
                                                     const S* __restrict__ ue,
                                                     const S* ainr, const S* ainu, const S* aine,
                                                     S* a1r, S* a1u, S* a1e, S* a0r, S* a0u, S* a0e, S* sb,
                                                     double dt, int objective, int objStart, int objN, double obja,
                                                     VaneDev vane, const double* __restrict__ objSeed) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.nIC) return;
    const size_t n = m.nIC;
    const size_t nF = m.nF;
    // cell adjoint records in 16-byte loads (a record is 80 / 160 bytes, 16-byte aligned)
    R cb[CBAR];
    load_vec(cbar + (size_t)c * CBAR, cb, CBAR);
    R pbar[5];
    for (int k = 0; k < 5; k++) pbar[k] = cb[k];
    const R* G = cb + 5;
    {
        // the cell's own slots at once: sum_s (1 - w'_s) (G . S N'_s) / V = G . gAv
        R A[3] = {m.gAv[c], m.gAv[n + c], m.gAv[2 * n + c]};
        for (int i = 0; i < 5; i++) pbar[i] += G[3 * i] * A[0] + G[3 * i + 1] * A[1] + G[3 * i + 2] * A[2];
    }
    for (int s = 0; s < 6; s++) {
        int nb = m.gnb[s * n + c];
        if (nb < m.nIC) {
            // neighbour's gradient: its slot for this face has S N'' = -S N' and weight gwb;
            // gbs_s = -gwb_s S N'_s / V_nb
            R b[3] = {m.gbs[(3 * s) * n + c], m.gbs[(3 * s + 1) * n + c], m.gbs[(3 * s + 2) * n + c]};
            R cn[CBAR];
            load_vec(cbar + (size_t)nb * CBAR, cn, CBAR);
            const R* Gn = cn + 5;
            for (int i = 0; i < 5; i++) pbar[i] += Gn[3 * i] * b[0] + Gn[3 * i + 1] * b[1] + Gn[3 * i + 2] * b[2];
        }
    }
    // ghost cells whose boundary value comes from this cell: transpose of the BC
    for (int q = m.gsStart[c]; q < m.gsStart[c + 1]; q++) {
        int g = m.gsList[q];
        int f = m.nIF + g;
        int o = m.own[f];
        int s = m.gslot[g];
        R gp[5];
        const R* r = fadj + (size_t)f * FADJ;
        for (int k = 0; k < 5; k++) gp[k] = r[20 + k];
        R sn[3] = {m.gsn[(3 * s) * n + o], m.gsn[(3 * s + 1) * n + o], m.gsn[(3 * s + 2) * n + o]};
        R w = m.gw[s * n + o];
        R pb[5];
        phi_bar<R>(cbar + (size_t)o * CBAR + 5, sn, m.rvol[o], pb);
        for (int k = 0; k < 5; k++) gp[k] += w * pb[k];
        if (STAGE == 1 && objective == AFVM_OBJ_DRAG && f >= objStart && f < objStart + objN) {
            // drag = sum (p0 nx - mu(T0) (U0 - U0i)/delta) A, ghost values p0, T0, U0
            const R* rg = rec + (size_t)(m.nIC + g) * REC;
            const R* ro = rec + (size_t)o * REC;
            double T0 = rec_T<R>(P, rg[R_T]), U0 = rg[0], U0i = ro[0];
            double A = m.area[f], dl = m.dlt[f], nx = m.nrm[f];
            double mu = viscosity<double>(P, T0);
            double dmu = (P.muModel == AFVM_MU_SUTHERLAND) ? mu * (1.5 / T0 - 1.0 / (T0 + P.muTs)) : 0.0;
            gp[R_P] += (R)(obja * nx * A);
            gp[R_T] += (R)(-obja * dmu * (U0 - U0i) / dl * A);
            gp[0] += (R)(-obja * mu / dl * A);
        }
        if (STAGE == 1 && objSeed)
            for (int k = 0; k < 5; k++) gp[k] += (R)(obja * objSeed[(size_t)(m.nIC + g) * 5 + k]);
        int kind = m.gkind[g];
        int kU = kind & 7, kT = (kind >> 3) & 7, kp = (kind >> 6) & 7;
        if (kU == GK_TOTALPT) {
            // transpose of Ub = (U.d) d, Tb = Tt - (U.d)^2/(2 Cp), pb = pt (T/Tt)^kappa
            const R* rs = rec + (size_t)c * REC;      // this cell is the ghost's source (owner)
            R d[3] = {m.gval[g], m.gval[(size_t)m.nG + g], m.gval[2 * (size_t)m.nG + g]};
            R Tt = m.gval[3 * (size_t)m.nG + g], pt = m.gval[4 * (size_t)m.nG + g];
            R Un = rs[0] * d[0] + rs[1] * d[1] + rs[2] * d[2];
            R kap = consts<R>(P).ggm1;
            R Unb = dot3(gp, d) - gp[R_T] * Un / consts<R>(P).Cp;
            for (int k = 0; k < 3; k++) pbar[k] += Unb * d[k];
            pbar[R_T] += gp[R_P] * pt * kap * pow(rec_abs_T<R>(P, rs[R_T]) / Tt, kap - R(1)) / Tt;
            continue;
        }
        if (kU == GK_COPY) {
            for (int k = 0; k < 3; k++) pbar[k] += gp[k];
        } else if (kU == GK_SYM) {
            R nr[3] = {m.nrm[f], m.nrm[nF + f], m.nrm[2 * nF + f]};
            R un = dot3(gp, nr);
            for (int k = 0; k < 3; k++) pbar[k] += gp[k] - un * nr[k];
        }
        if (kT != GK_FIXED) pbar[R_T] += gp[R_T];
        if (kp != GK_FIXED) pbar[R_P] += gp[R_P];
    }
    // an objective evaluated by the caller: its gradient with respect to this cell's primitives
    if (STAGE == 1 && objSeed)
        for (int k = 0; k < 5; k++) pbar[k] += (R)(obja * objSeed[(size_t)c * 5 + k]);
    // objective on the stage-1 primitives
    if (STAGE == 1 && objective != AFVM_OBJ_NONE) {
        const R* rc = rec + (size_t)c * REC;
        if (objective == AFVM_OBJ_KINETIC_ENERGY) {
            double U[3] = {rc[0], rc[1], rc[2]}, T = rec_T<R>(P, rc[R_T]), p = rec_p<R>(P, rc[R_P]), V = m.vol[c];
            double d = (P.Cv * T) * P.gm1;
            double rd = rcp(d);           // (Newton reciprocals: no IEEE divisions on the FP64 pipe)
            double rho = p * rd;
            double q = U[0] * U[0] + U[1] * U[1] + U[2] * U[2];
            for (int k = 0; k < 3; k++) pbar[k] += (R)(obja * rho * U[k] * V);
            pbar[R_P] += (R)(obja * 0.5 * q * V * rd);
            pbar[R_T] += (R)(-obja * 0.5 * q * V * rho * rcp(T));
        } else if (objective == AFVM_OBJ_SUM_T) {
            pbar[R_T] += (R)obja;
        } else if (objective == AFVM_OBJ_VANE) {
            int q = vane.cellPlane[c];
            if (q >= 0) {
                double g5[5] = {0, 0, 0, 0, 0};
                double U[3] = {rc[0], rc[1], rc[2]};
                vane_cell_grad(P, vane, U, rec_T<R>(P, rc[R_T]), rec_p<R>(P, rc[R_P]), vane.planeArea[q], vane.sums[0],
                               vane.sums[1], obja, g5);
                for (int k = 0; k < 5; k++) pbar[k] += (R)g5[k];
            }
            if (vane.b != 0.0) {
                for (int s = 0; s < 6; s++) {
                    int e = m.accf[s * n + c];
                    if (e < m.nIF) continue;          // owner-side boundary faces only
                    double k = vane.bHeatCoef[e - m.nIF];
                    if (k != 0.0) pbar[R_T] += (R)(-obja * vane.b * vane.rw2 * k);
                }
            }
        } else if (objective == AFVM_OBJ_DRAG) {
            for (int s = 0; s < 6; s++) {
                int e = m.accf[s * n + c];
                if (e < objStart || e >= objStart + objN) continue;   // owner-side faces of the patch
                const R* rg = rec + (size_t)m.nbr[e] * REC;
                double T0 = rec_T<R>(P, rg[R_T]);
                double mu = viscosity<double>(P, T0);
                pbar[0] += (R)(obja * mu / (double)m.dlt[e] * (double)m.area[e]);
            }
        }
    }
    // primitive VJP (density.py:162-171)
    S J[5];
    if constexpr (sizeof(S) == 4) {
        // float state: the density row without the low-Mach cancellation of the form below
        // (rhob and eb E/rho both hold pbar_p (g-1) E): with q = |U|^2/2 and e = E - q,
        //   J_rho = pbar_p (g-1) q - (pbar_U . U)/rho + (pbar_T/Cv) (q - e)/rho,
        // which float evaluates to its own rounding, so the FP32 context needs no FP64 here
        const PhysR<float>& Q = consts<float>(P);
        float rho = ur[c], rr = rcp(rho);
        float U[3] = {uu[3 * c] * rr, uu[3 * c + 1] * rr, uu[3 * c + 2] * rr};
        float E = ue[c] * rr;
        float q = 0.5f * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
        float e = E - q;
        float pT = pbar[R_T] * Q.rCv, pp = pbar[R_P] * Q.gm1;
        float eb = pT + pp * rho;
        for (int k = 0; k < 3; k++) J[1 + k] = (pbar[k] - eb * U[k]) * rr;
        J[4] = eb * rr;
        J[0] = pp * q - (pbar[0] * U[0] + pbar[1] * U[1] + pbar[2] * U[2]) * rr + pT * (q - e) * rr;
    } else {
        double rho = ur[c], rU[3] = {uu[3 * c], uu[3 * c + 1], uu[3 * c + 2]}, rE = ue[c];
        double rr = rcp(rho);
        double U[3] = {rU[0] * rr, rU[1] * rr, rU[2] * rr};
        double E = rE * rr;
        double e = E - 0.5 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
        double eb = (double)pbar[R_T] * P.rCv + (double)pbar[R_P] * P.gm1 * rho;
        double rhob = (double)pbar[R_P] * P.gm1 * e;
        double Ubt[3];
        for (int k = 0; k < 3; k++) Ubt[k] = (double)pbar[k] - eb * U[k];
        for (int k = 0; k < 3; k++) J[1 + k] = Ubt[k] * rr;
        J[4] = eb * rr;
        J[0] = rhob - (Ubt[0] * U[0] + Ubt[1] * U[1] + Ubt[2] * U[2]) * rr - eb * E * rr;
    }
    // SSP-RK reverse (timestep.py:35-45 transposed), in the state's type S
    S ain[5] = {ainr[c], ainu[3 * c], ainu[3 * c + 1], ainu[3 * c + 2], aine[c]};
    S out[5];
    if (STAGE == 2) {
        for (int k = 0; k < 5; k++) out[k] = S(2. / 3) * ain[k] + (S)J[k];
        S z[5];
        for (int k = 0; k < 5; k++) { z[k] = S(1. / 3) * ain[k]; sb[k * n + c] = S(2. / 3) * S(dt) * ain[k]; }
        a0r[c] = z[0]; a0u[3 * c] = z[1]; a0u[3 * c + 1] = z[2]; a0u[3 * c + 2] = z[3]; a0e[c] = z[4];
        a1r[c] = out[0]; a1u[3 * c] = out[1]; a1u[3 * c + 1] = out[2]; a1u[3 * c + 2] = out[3]; a1e[c] = out[4];
    } else if (STAGE == 1) {
        for (int k = 0; k < 5; k++) out[k] = S(1. / 4) * ain[k] + (S)J[k];
        S z[5] = {a0r[c], a0u[3 * c], a0u[3 * c + 1], a0u[3 * c + 2], a0e[c]};
        for (int k = 0; k < 5; k++) { z[k] += S(3. / 4) * ain[k]; sb[k * n + c] += S(1. / 4) * S(dt) * ain[k]; }
        a0r[c] = z[0]; a0u[3 * c] = z[1]; a0u[3 * c + 1] = z[2]; a0u[3 * c + 2] = z[3]; a0e[c] = z[4];
        a1r[c] = out[0]; a1u[3 * c] = out[1]; a1u[3 * c + 1] = out[2]; a1u[3 * c + 2] = out[3]; a1e[c] = out[4];
    } else {
        S z[5] = {a0r[c], a0u[3 * c], a0u[3 * c + 1], a0u[3 * c + 2], a0e[c]};
        for (int k = 0; k < 5; k++) { z[k] += ain[k] + (S)J[k]; sb[k * n + c] += S(dt) * ain[k]; }
        a0r[c] = z[0]; a0u[3 * c] = z[1]; a0u[3 * c + 1] = z[2]; a0u[3 * c + 2] = z[3]; a0e[c] = z[4];
    }
}

// the source adjoint (5 x nIC, one coalesced row per component) into the reference layout
template <typename R>
__global__ void k_split5(int n, const R* __restrict__ sb, R* r, R* u, R* e) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const size_t m = n;
    if (r) r[c] = sb[c];
    if (u) { u[3 * c] = sb[m + c]; u[3 * c + 1] = sb[2 * m + c]; u[3 * c + 2] = sb[3 * m + c]; }
    if (e) e[c] = sb[4 * m + c];
}

template <typename R, typename S>
int adjoint_step_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, double dt, const S* Srho, const S* SrhoU,
                     const S* SrhoE, const S* rhoNa, const S* rhoUNa, const S* rhoENa, double obja, S* rhoa,
                     S* rhoUa, S* rhoEa, S* Srhoa, S* SrhoUa, S* SrhoEa, cudaStream_t s, const S* stages,
                     const R* tape, const ParamDev* params) {
    const MeshDev<R>& m = meshOf<R>(c);
    const Phys& P = c->phys;
    default_sources<S>(c, Srho, SrhoU, SrhoE);
    int inviscid = (P.muModel == AFVM_MU_CONSTANT && P.mu0 == 0.0) ? 1 : 0;
    S* u1[3] = {(S*)c->u1[0], (S*)c->u1[1], (S*)c->u1[2]};
    S* u2[3] = {(S*)c->u2[0], (S*)c->u2[1], (S*)c->u2[2]};
    const S* u0c[3] = {rho, rhoU, rhoE};
    const S* u1c[3] = {u1[0], u1[1], u1[2]};
    const S* u2c[3] = {u2[0], u2[1], u2[2]};
    if (stages) {
        // the stage states the primal step kept (afvm_primal_step_stages)
        stage_views<S, const S>(stages, m.nIC, u1c, u2c);
    } else {
        // forward recompute of the stage states
        cudaMemsetAsync(c->dtcBits, 0, sizeof(unsigned long long), s);
        launch_prim_grad<R, S>(c, rho, rhoU, rhoE, s);
        launch_flux_update<R, S>(c, 0, dt, nullptr, u0c, u1c, u2c, Srho, SrhoU, SrhoE, u1, s);
        launch_prim_grad<R, S>(c, u1[0], u1[1], u1[2], s);
        launch_flux_update<R, S>(c, 1, dt, nullptr, u0c, u1c, u2c, Srho, SrhoU, SrhoE, u2, s);
    }
    // reverse sweep
    S* A1[3] = {(S*)c->a1[0], (S*)c->a1[1], (S*)c->a1[2]};
    S* A2[3] = {(S*)c->a2[0], (S*)c->a2[1], (S*)c->a2[2]};
    R* fadj = (R*)c->fadj;
    R* cbar = (R*)c->cbar;
    S* sb = (S*)c->sbar;
    int nbC = nblocks(m.nIC);
    const double beta[3] = {1.0, 1. / 4, 2. / 3};
    // a tape holds the stage's cell records the primal step built (no primitive or gradient
    // launches here) and, in FP64, its face tape
    const R* faceTape = nullptr;
    const R* recTape = nullptr;
    split_tape<const R>(c, tape, faceTape, recTape);
    for (int st = 2; st >= 0; st--) {
        const S* const* u = st == 0 ? u0c : (st == 1 ? u1c : u2c);
        const R* rec = recTape ? recTape + (size_t)st * m.nC * REC : (const R*)c->rec;
        if (!recTape) launch_prim_grad<R, S>(c, u[0], u[1], u[2], s);
        if (st == 1 && c->objective == AFVM_OBJ_VANE) launch_vane_sums<R>(c, s, nullptr, nullptr, rec);
        // adjoint of this stage's output: a3 = seeds, a2 = A2, a1 = A1
        const S* ain[3];
        if (st == 2) { ain[0] = rhoNa; ain[1] = rhoUNa; ain[2] = rhoENa; }
        else if (st == 1) { ain[0] = A2[0]; ain[1] = A2[1]; ain[2] = A2[2]; }
        else { ain[0] = A1[0]; ain[1] = A1[1]; ain[2] = A1[2]; }
        R coef = (R)(-beta[st] * dt);
        {
            ProfScope ps(c, KID_ADJ_FLUX, s);
            int nbF = (m.nF + FLUX_BLOCK - 1) / FLUX_BLOCK;
            if (faceTape)
                k_adj_flux<R, S, true><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, coef, ain[0], ain[1], ain[2], fadj,
                                                                  inviscid, faceTape + (size_t)st * TAPE * m.nF);
            else
                k_adj_flux<R, S, false><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, coef, ain[0], ain[1], ain[2], fadj,
                                                                   inviscid, nullptr);
        }
        {
            ProfScope ps(c, KID_ADJ_GATHER, s);
            k_adj_cell1<R><<<nbC, BLOCK, 0, s>>>(m, fadj, cbar);
        }
        // the stage's share of the mesh / boundary-input gradients (before the cell kernel: the
        // adjoint outputs it writes may alias this stage's input adjoints)
        if constexpr (std::is_same<R, double>::value && std::is_same<S, double>::value)
            if (params) launch_param_grads<R, S>(c, *params, rec, coef, ain[0], ain[1], ain[2], st == 1, obja, s);
        ProfScope ps(c, KID_ADJ_GRAD, s);
        if (st == 2)
            k_adj_cell2<R, S, 2><<<nbC, BLOCK, 0, s>>>(m, P, rec, fadj, cbar, u[0], u[1], u[2], ain[0], ain[1], ain[2],
                                                    A2[0], A2[1], A2[2], rhoa, rhoUa, rhoEa, sb, dt, c->objective,
                                                    c->objStart, c->objN, obja, c->vane, c->objSeed);
        else if (st == 1)
            k_adj_cell2<R, S, 1><<<nbC, BLOCK, 0, s>>>(m, P, rec, fadj, cbar, u[0], u[1], u[2], ain[0], ain[1], ain[2],
                                                    A1[0], A1[1], A1[2], rhoa, rhoUa, rhoEa, sb, dt, c->objective,
                                                    c->objStart, c->objN, obja, c->vane, c->objSeed);
        else
            k_adj_cell2<R, S, 0><<<nbC, BLOCK, 0, s>>>(m, P, rec, fadj, cbar, u[0], u[1], u[2], ain[0], ain[1], ain[2],
                                                    nullptr, nullptr, nullptr, rhoa, rhoUa, rhoEa, sb, dt,
                                                    c->objective, c->objStart, c->objN, obja, c->vane, c->objSeed);
    }
    if (Srhoa || SrhoUa || SrhoEa) {
        ProfScope ps(c, KID_ADJ_MISC, s);
        k_split5<S><<<nbC, BLOCK, 0, s>>>(m.nIC, sb, Srhoa, SrhoUa, SrhoEa);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint step launch");
    return AFVM_OK;
}

#define AFVM_ADJ_INST(R, S)                                                                                    \
    template int adjoint_step_dev<R, S>(Ctx*, const S*, const S*, const S*, double, const S*, const S*, const S*, \
                                        const S*, const S*, const S*, double, S*, S*, S*, S*, S*, S*,             \
                                        cudaStream_t, const S*, const R*, const ParamDev*);
AFVM_ADJ_INST(double, double)
AFVM_ADJ_INST(float, float)
AFVM_ADJ_INST(float, double)

}  // namespace afvm
