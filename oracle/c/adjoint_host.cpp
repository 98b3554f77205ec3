/*
 * Host (CPU, OpenMP) FP64 adjoint of one SSP-RK3 step - TEST INFRASTRUCTURE ONLY: the timed
 * CPU baseline of the adjoint step in bench.py, checked against torch autograd of the oracle
 * by tests/test_oracle_adjoint_host.py. The product never links it.
 *
 * The reference's adjoint is adpy's reverse mode over the whole step (apps/adjoint.py:101-126),
 * and adpy is absent, so no CPU adjoint of the reference can run. This baseline is what such a
 * CPU adjoint computes, at CPU speed: the forward (stage states and cell records) by the C
 * oracle (oracle/c/afvm_oracle.c), the face VJP of adfvm_gb300/csrc/face.cuh compiled for the
 * host, and the rest of the reverse sweep restated here:
 *   per stage i = 2, 1, 0 with output adjoint a (a3 = the seeds), coefficient -beta_i dt:
 *   faces   Fbar = coef (a_P A/V_L - a_N A/V_R), the face VJP -> 40 input adjoints a face;
 *   cells   the cell's share of its faces' records (op.py:45-63 and 12-20 transposed), the
 *           Green-Gauss gradient transposed through the cell's own slots and its neighbours',
 *           the ghost cells' boundary conditions transposed (BCs.py:86-184), the objective's
 *           gradient on stage 1 (density.py:354-357, 412-413), the primitive VJP
 *           (density.py:162-171) and the SSP-RK update transposed (timestep.py:17-55).
 * Compile with -ffp-contract=off like the rest of the oracle (oracle/build.py).
 */
#include <cmath>
#include <cstring>
#include <vector>
#include "afvm_oracle.h"
#include "face.cuh"

using namespace afvm;

namespace {

Phys phys_of(const oracle_mesh* M) {
    Phys P;
    P.gamma = M->gamma;
    P.gm1 = M->gamma - 1;
    P.Cp = M->Cp;
    P.Cv = M->Cp / M->gamma;
    P.rCv = 1. / P.Cv;
    P.kFac = M->Cp / M->Pr;
    P.muModel = M->muModel;
    P.mu0 = M->mu0;
    P.muAs = M->muAs;
    P.muTs = M->muTs;
    P.riemann = M->riemann;
    P.briemann = M->briemann;
    P.small = 1e-30;
    finish_phys(P);
    return P;
}

inline void face_in(const oracle_mesh* M, const double* rec, int f, FaceIn<double>& in) {
    int iP = M->own[f], iN = M->nbr[f];
    int iG = f < M->nIF ? iN : M->gsrc[iN - M->nIC];
    const double *rP = rec + 20 * (size_t)iP, *rN = rec + 20 * (size_t)iN, *rG = rec + 20 * (size_t)iG;
    for (int k = 0; k < 3; k++) { in.UP[k] = rP[k]; in.UN[k] = rN[k]; }
    in.TP = rP[3]; in.pP = rP[4]; in.TN = rN[3]; in.pN = rN[4];
    for (int k = 0; k < 9; k++) { in.gUP[k] = rP[5 + k]; in.gUN[k] = rG[5 + k]; }
    for (int k = 0; k < 3; k++) {
        in.gTP[k] = rP[14 + k]; in.gTN[k] = rG[14 + k];
        in.gpP[k] = rP[17 + k]; in.gpN[k] = rG[17 + k];
        in.N[k] = M->nrm[3 * (size_t)f + k];
        in.D[k] = M->du[3 * (size_t)f + k];
        in.qw0[k] = M->qw[6 * (size_t)f + k];
        in.qw1[k] = M->qw[6 * (size_t)f + 3 + k];
    }
    in.lw0 = M->lw[2 * (size_t)f];
    in.lw1 = M->lw[2 * (size_t)f + 1];
    in.rdelta = 1.0 / M->dlt[f];
    face_derived(in);
}

// w' and S N' of a gradient slot (op.py:45-63): O = 1 when the cell owns the face
inline void slot_geometry(const oracle_mesh* M, int f, int O, double& wp, double* sn) {
    double w = M->wts[f], S = M->area[f], Od = (double)O;
    wp = (w + Od) - (2 * w) * Od;
    for (int k = 0; k < 3; k++) {
        double n = M->nrm[3 * (size_t)f + k];
        sn[k] = S * ((2 * n) * Od - n);
    }
}

inline double phi_bar(const double* G, const double* sn, double rv, int i) {
    return rv * (G[3 * i] * sn[0] + G[3 * i + 1] * sn[1] + G[3 * i + 2] * sn[2]);
}

}  // namespace

extern "C" size_t oracle_adjoint_work_doubles(const oracle_mesh* M) {
    // the forward's work, the face records (40 a face), the cell adjoints (20 a cell), three
    // stage adjoints (5 a cell each) and the ghost lists (as doubles' worth of ints)
    return oracle_work_doubles(M) + 40 * (size_t)M->nF + 20 * (size_t)M->nIC + 15 * (size_t)M->nIC +
           (size_t)M->nIC + (size_t)M->nG + 2;
}

/* the VJP of one step (dt held fixed, the CFL sum unseeded): seeds aN = (rhoNa, rUNa, rENa),
 * objective seed obja; outputs the state adjoint (rhoa, rUa, rEa) and, if Sa is not NULL, the
 * source adjoint (nIC x 5). S: nIC x 5 sources or NULL. Supported objectives: none, kinetic
 * energy, drag, sum of T. */
extern "C" int oracle_adjoint_step(const oracle_mesh* M, const double* rho, const double* rU, const double* rE,
                                   double dt, const double* S, const double* rhoNa, const double* rUNa,
                                   const double* rENa, double obja, double* rhoa, double* rUa, double* rEa,
                                   double* Sa, double* work) {
    if (M->objective == 4) return 1;
    const int nIC = M->nIC, nIF = M->nIF, nF = M->nF, nG = M->nG;
    const Phys P = phys_of(M);
    const bool inviscid = M->muModel == 0 && M->mu0 == 0.0;
    double* fwork = work;
    double* fadj = fwork + oracle_work_doubles(M);
    double* cbar = fadj + 40 * (size_t)nF;
    double* A2 = cbar + 20 * (size_t)nIC;
    double* A1 = A2 + 5 * (size_t)nIC;
    double* a0 = A1 + 5 * (size_t)nIC;
    int* gStart = reinterpret_cast<int*>(a0 + 5 * (size_t)nIC);
    int* gList = gStart + (nIC + 1);
    // ghosts by source cell (CSR)
    for (int c = 0; c <= nIC; c++) gStart[c] = 0;
    for (int g = 0; g < nG; g++) gStart[M->gsrc[g] + 1]++;
    for (int c = 0; c < nIC; c++) gStart[c + 1] += gStart[c];
    {
        std::vector<int> fill(gStart, gStart + nIC);
        for (int g = 0; g < nG; g++) gList[fill[M->gsrc[g]]++] = g;
    }
    // forward: the step's stage states u1, u2 (and its output, unused)
    std::vector<double> out(5 * (size_t)nIC);
    double dtcMax, obj;
    oracle_step(M, rho, rU, rE, dt, S, out.data(), out.data() + nIC, out.data() + 4 * (size_t)nIC, &dtcMax, &obj,
                fwork);
    const double* st1 = oracle_work_stage(M, fwork, 1);
    const double* st2 = oracle_work_stage(M, fwork, 2);
    const double* ur[3] = {rho, st1, st2};
    const double* uu[3] = {rU, st1 + nIC, st2 + nIC};
    const double* ue[3] = {rE, st1 + 4 * (size_t)nIC, st2 + 4 * (size_t)nIC};
    const double beta[3] = {1.0, 1. / 4, 2. / 3};
    const double* rec = fwork;
    for (int st = 2; st >= 0; st--) {
        oracle_records(M, ur[st], uu[st], ue[st], fwork);
        // the adjoint of this stage's output, as (rho | rhoU | rhoE) per cell
        auto ain = [&](int c, int k) -> double {
            if (st == 2) return k == 0 ? rhoNa[c] : (k < 4 ? rUNa[3 * (size_t)c + k - 1] : rENa[c]);
            return (st == 1 ? A2 : A1)[5 * (size_t)c + k];
        };
        const double coef = -beta[st] * dt;
#pragma omp parallel for schedule(static)
        for (int f = 0; f < nF; f++) {
            int kind = f < nIF ? FACE_INTERNAL : (int)M->fkind[f - nIF];
            int iP = M->own[f];
            double wp = M->area[f] / M->vol[iP];
            double Fb[5];
            for (int k = 0; k < 5; k++) Fb[k] = (coef * ain(iP, k)) * wp;
            if (f < nIF) {
                int iN = M->nbr[f];
                double wn = M->area[f] / M->vol[iN];
                for (int k = 0; k < 5; k++) Fb[k] = Fb[k] - (coef * ain(iN, k)) * wn;
            }
            FaceIn<double> in;
            face_in(M, rec, f, in);
            FaceBar<double> b;
            zero_bar(b);
            face_vjp<double>(P, kind, inviscid, in, Fb, b);
            std::memcpy(fadj + 40 * (size_t)f, &b, sizeof(b));
        }
        // per cell: its faces' primitive and gradient adjoints (FaceBar order: UP TP pP UN TN pN,
        // gUP gTP gpP, gUN gTN gpN), and the gradient adjoints of the ghosts it is the source of
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nIC; c++) {
            double acc[20] = {0};
            for (int s = 0; s < 6; s++) {
                int e = M->accf[6 * (size_t)c + s];
                bool own = e >= 0;
                int f = own ? e : ~e;
                const double* b = fadj + 40 * (size_t)f;
                for (int k = 0; k < 5; k++) acc[k] += b[(own ? 0 : 5) + k];
                for (int k = 0; k < 15; k++) acc[5 + k] += b[(own ? 10 : 25) + k];
            }
            for (int q = gStart[c]; q < gStart[c + 1]; q++) {
                const double* b = fadj + 40 * (size_t)(nIF + gList[q]);
                for (int k = 0; k < 15; k++) acc[5 + k] += b[25 + k];
            }
            std::memcpy(cbar + 20 * (size_t)c, acc, sizeof(acc));
        }
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nIC; c++) {
            double pbar[5];
            for (int k = 0; k < 5; k++) pbar[k] = cbar[20 * (size_t)c + k];
            const double* G = cbar + 20 * (size_t)c + 5;
            double rv = 1.0 / M->vol[c];
            for (int s = 0; s < 6; s++) {
                int f = M->cellFaces[6 * (size_t)c + s];
                int O = M->cellOwn[6 * (size_t)c + s];
                int nb = M->cellNbr[6 * (size_t)c + s];
                double w1, sn[3];
                slot_geometry(M, f, O, w1, sn);
                // this cell's own gradient: phiF = phi_c (1 - w') + phi_nb w'
                for (int i = 0; i < 5; i++) pbar[i] += (1 - w1) * phi_bar(G, sn, rv, i);
                if (nb < nIC) {
                    // the neighbour's gradient reads this cell through its slot of the same face
                    double w2, sn2[3];
                    slot_geometry(M, f, 1 - O, w2, sn2);
                    const double* Gn = cbar + 20 * (size_t)nb + 5;
                    double rvn = 1.0 / M->vol[nb];
                    for (int i = 0; i < 5; i++) pbar[i] += w2 * phi_bar(Gn, sn2, rvn, i);
                }
            }
            // ghost cells whose values come from this cell
            for (int q = gStart[c]; q < gStart[c + 1]; q++) {
                int g = gList[q];
                int f = nIF + g;
                int o = M->own[f];
                const double* b = fadj + 40 * (size_t)f;
                double gp[5];
                for (int k = 0; k < 5; k++) gp[k] = b[5 + k];
                // the owner's gradient slot that reads the ghost (the owner owns the face)
                double w1, sn[3];
                slot_geometry(M, f, 1, w1, sn);
                const double* Go = cbar + 20 * (size_t)o + 5;
                for (int i = 0; i < 5; i++) gp[i] += w1 * phi_bar(Go, sn, 1.0 / M->vol[o], i);
                if (st == 1 && M->objective == 2 && f >= M->objStart && f < M->objStart + M->objN) {
                    // drag = sum (p0 n_x - mu(T0) (U0 - U0i) / delta) A
                    const double* rg = rec + 20 * (size_t)(nIC + g);
                    const double* ro = rec + 20 * (size_t)o;
                    double T0 = rg[3], U0 = rg[0], U0i = ro[0];
                    double A = M->area[f], dl = M->dlt[f], nx = M->nrm[3 * (size_t)f];
                    double mu = viscosity<double>(P, T0);
                    double dmu = M->muModel == 1 ? mu * (1.5 / T0 - 1.0 / (T0 + M->muTs)) : 0.0;
                    gp[4] += obja * nx * A;
                    gp[3] += -obja * dmu * (U0 - U0i) / dl * A;
                    gp[0] += -obja * mu / dl * A;
                }
                int kind = M->gkind[g];
                int kU = kind & 7, kT = (kind >> 3) & 7, kp = (kind >> 6) & 7;
                const double* rs = rec + 20 * (size_t)c;
                if (kU == K_TOTALPT) {
                    const double* d = M->gval + 5 * (size_t)g;
                    double Tt = d[3], pt = d[4];
                    double Un = rs[0] * d[0] + rs[1] * d[1] + rs[2] * d[2];
                    double kap = M->gamma / (M->gamma - 1);
                    double Unb = gp[0] * d[0] + gp[1] * d[1] + gp[2] * d[2] - gp[3] * Un / M->Cp;
                    for (int k = 0; k < 3; k++) pbar[k] += Unb * d[k];
                    pbar[3] += gp[4] * pt * kap * std::pow(rs[3] / Tt, kap - 1) / Tt;
                    continue;
                }
                if (kU == K_COPY) {
                    for (int k = 0; k < 3; k++) pbar[k] += gp[k];
                } else if (kU == K_SYM) {
                    const double* n = M->nrm + 3 * (size_t)f;
                    double un = gp[0] * n[0] + gp[1] * n[1] + gp[2] * n[2];
                    for (int k = 0; k < 3; k++) pbar[k] += gp[k] - un * n[k];
                }
                if (kT != K_FIXED) pbar[3] += gp[3];
                if (kp != K_FIXED) pbar[4] += gp[4];
            }
            // the objective on the stage-1 primitives
            if (st == 1) {
                const double* r = rec + 20 * (size_t)c;
                if (M->objective == 1) {
                    double V = M->vol[c], T = r[3], p = r[4];
                    double d = (P.Cv * T) * P.gm1;
                    double rh = p / d;
                    double q = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
                    for (int k = 0; k < 3; k++) pbar[k] += obja * rh * r[k] * V;
                    pbar[4] += obja * 0.5 * q * V / d;
                    pbar[3] += -obja * 0.5 * q * V * rh / T;
                } else if (M->objective == 3) {
                    pbar[3] += obja;
                } else if (M->objective == 2) {
                    for (int s = 0; s < 6; s++) {
                        int e = M->accf[6 * (size_t)c + s];
                        if (e < M->objStart || e >= M->objStart + M->objN) continue;
                        double T0 = rec[20 * (size_t)M->nbr[e] + 3];
                        pbar[0] += obja * viscosity<double>(P, T0) / M->dlt[e] * M->area[e];
                    }
                }
            }
            // primitive VJP (density.py:162-171)
            double rh = ur[st][c], rr = 1.0 / rh;
            double U[3] = {uu[st][3 * (size_t)c] * rr, uu[st][3 * (size_t)c + 1] * rr, uu[st][3 * (size_t)c + 2] * rr};
            double E = ue[st][c] * rr;
            double e = E - 0.5 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
            double eb = pbar[3] * P.rCv + pbar[4] * P.gm1 * rh;
            double rhob = pbar[4] * P.gm1 * e;
            double Ubt[3], J[5];
            for (int k = 0; k < 3; k++) Ubt[k] = pbar[k] - eb * U[k];
            for (int k = 0; k < 3; k++) J[1 + k] = Ubt[k] * rr;
            J[4] = eb * rr;
            J[0] = rhob - (Ubt[0] * U[0] + Ubt[1] * U[1] + Ubt[2] * U[2]) * rr - eb * E * rr;
            // SSP-RK reverse (timestep.py:35-45 transposed)
            double* sb = Sa ? Sa + 5 * (size_t)c : nullptr;
            for (int k = 0; k < 5; k++) {
                double a = ain(c, k);
                if (st == 2) {
                    A2[5 * (size_t)c + k] = 2. / 3 * a + J[k];
                    a0[5 * (size_t)c + k] = 1. / 3 * a;
                    if (sb) sb[k] = 2. / 3 * dt * a;
                } else if (st == 1) {
                    A1[5 * (size_t)c + k] = 1. / 4 * a + J[k];
                    a0[5 * (size_t)c + k] += 3. / 4 * a;
                    if (sb) sb[k] += 1. / 4 * dt * a;
                } else {
                    a0[5 * (size_t)c + k] += a + J[k];
                    if (sb) sb[k] += dt * a;
                }
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nIC; c++) {
        rhoa[c] = a0[5 * (size_t)c];
        for (int k = 0; k < 3; k++) rUa[3 * (size_t)c + k] = a0[5 * (size_t)c + 1 + k];
        rEa[c] = a0[5 * (size_t)c + 4];
    }
    return 0;
}
