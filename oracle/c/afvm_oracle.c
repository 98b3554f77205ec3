/*
 * Oracle (TEST INFRASTRUCTURE ONLY): C99 + OpenMP restatement of the reference's FP64 time
 * step, used as the timed CPU baseline of bench.py and cross-checked against the torch
 * oracle by tests/test_oracle_c.py. The product never links it.
 *
 * Follows the reference expression by expression:
 *   primitive            adFVM/density.py:162-171
 *   conservative         adFVM/density.py:173-181
 *   ghost BCs            adFVM/BCs.py:86-161, density.py:333-337
 *   gradCell             adFVM/op.py:45-63
 *   secondOrder          adFVM/interp.py:20-28
 *   eulerRoe / LF        adFVM/riemann.py:6-70
 *   viscousFlux          adFVM/density.py:192-222
 *   flux / boundaryFlux  adFVM/density.py:253-331
 *   div / absDiv collate adFVM/op.py:12-29 in the order of density.py:390-402 (per cell, the
 *                        contributions of its faces in collate order: a gather, so the OpenMP
 *                        loop over cells keeps the reference's summation order)
 *   SSP-RK3              adFVM/timestep.py:17-55, stage-1 dtc/objective density.py:405-413
 * Compile with -ffp-contract=off (oracle/build.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "afvm_oracle.h"

#define SMALL 1e-30

static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static double mu_of(const oracle_mesh* M, double T) {
    if (M->muModel == 1) return 1.4792e-06 * pow(T, 1.5) / (T + 116.);
    return M->mu0;
}

static void primitive(const oracle_mesh* M, double rho, const double* rU, double rE, double* U, double* T, double* p) {
    double Cv = M->Cp / M->gamma;
    for (int k = 0; k < 3; k++) U[k] = rU[k] / rho;
    double E = rE / rho;
    double e = E - 0.5 * dot3(U, U);
    *p = (M->gamma - 1) * rho * e;
    *T = e * (1. / Cv);
}

static void conservative(const oracle_mesh* M, const double* U, double T, double p, double* rho, double* rU, double* rE) {
    double Cv = M->Cp / M->gamma;
    double e = Cv * T;
    *rho = p / (e * (M->gamma - 1));
    *rE = *rho * (e + 0.5 * dot3(U, U));
    for (int k = 0; k < 3; k++) rU[k] = U[k] * *rho;
}

static double recon(double phiC, double phiD, const double* g, double lw, const double* qw) {
    double phiF = phiC + (phiD - phiC) * lw;
    return phiF + (qw[0] * g[0] + qw[1] * g[1] + qw[2] * g[2]);
}

static void roe(const oracle_mesh* M, double pL, double pR, const double* UL, const double* UR, double rhoL,
                double rhoR, const double* N, double* F) {
    double g = M->gamma;
    double rhoUnL = rhoL * dot3(UL, N), rhoUnR = rhoR * dot3(UR, N);
    double hL = g * pL / ((g - 1) * rhoL) + 0.5 * dot3(UL, UL);
    double hR = g * pR / ((g - 1) * rhoR) + 0.5 * dot3(UR, UR);
    double fr = 0.5 * (rhoUnL + rhoUnR), fu[3], UF[3], dU[3];
    for (int k = 0; k < 3; k++) fu[k] = 0.5 * (rhoUnL * UL[k] + rhoUnR * UR[k] + (pL + pR) * N[k]);
    double fe = 0.5 * (rhoUnL * hL + rhoUnR * hR);
    double sL = sqrt(rhoL), sR = sqrt(rhoR);
    double D = sL + sR;
    for (int k = 0; k < 3; k++) UF[k] = (UL[k] * sL + UR[k] * sR) / D;
    double hF = (hL * sL + hR * sR) / D;
    double qF = 0.5 * dot3(UF, UF);
    double a2F = (g - 1) * (hF - qF);
    double aF = sqrt(a2F);
    double UnF = dot3(UF, N);
    double drho = rhoR - rhoL;
    for (int k = 0; k < 3; k++) dU[k] = rhoR * UR[k] - rhoL * UL[k];
    double drhoE = (hR * rhoR - pR) - (hL * rhoL - pL);
    double l1 = fabs(UnF), l2 = fabs(UnF + aF), l3 = fabs(UnF - aF);
    double eps = 0.5 * fabs(rhoUnL / rhoL - rhoUnR / rhoR);
    eps = eps + 0.5 * fabs(sqrt(g * pL / rhoL) - sqrt(g * pR / rhoR));
    eps = (eps < 0) ? eps - SMALL : eps + SMALL;
    if (l1 < 2. * eps) l1 = .25 * l1 * l1 / eps + eps;
    if (l2 < 2. * eps) l2 = .25 * l2 * l2 / eps + eps;
    if (l3 < 2. * eps) l3 = .25 * l3 * l3 / eps + eps;
    double abv1 = 0.5 * (l2 + l3), abv2 = 0.5 * (l2 - l3), abv3 = abv1 - l1;
    double abv4 = (g - 1) * (qF * drho - dot3(UF, dU) + drhoE);
    double abv5 = UnF * drho - dot3(dU, N);
    double abv6 = abv3 * abv4 / a2F - abv2 * abv5 / aF;
    double abv7 = abv3 * abv5 - abv2 * abv4 / aF;
    F[0] = fr - 0.5 * (l1 * drho + abv6);
    for (int k = 0; k < 3; k++) F[1 + k] = fu[k] - 0.5 * (l1 * dU[k] + UF[k] * abv6 - abv7 * N[k]);
    F[4] = fe - 0.5 * (l1 * drhoE + hF * abv6 - UnF * abv7);
}

static void laxf(const oracle_mesh* M, double pL, double pR, const double* UL, const double* UR, double rhoL,
                 double rhoR, const double* rUL, const double* rUR, double rEL, double rER, const double* N, double* F) {
    double g = M->gamma;
    double UnL = dot3(UL, N), UnR = dot3(UR, N);
    double cL = sqrt(g * pL / rhoL), cR = sqrt(g * pR / rhoR);
    double A = fabs(UnL) + cL, B = fabs(UnR) + cR;
    double aF = A > B ? A : B;
    F[0] = 0.5 * (rhoL * UnL + rhoR * UnR) - 0.5 * aF * (rhoR - rhoL);
    for (int k = 0; k < 3; k++)
        F[1 + k] = 0.5 * (rUL[k] * UnL + rUR[k] * UnR + (pL + pR) * N[k]) - 0.5 * aF * (rUR[k] - rUL[k]);
    F[4] = 0.5 * ((rEL + pL) * UnL + (rER + pR) * UnR) - 0.5 * aF * (rER - rEL);
}

static void viscous(const oracle_mesh* M, double TL, double TR, const double* UL, const double* UR, double TF,
                    const double* UF, const double* gTF, const double* gUF, const double* D, const double* N,
                    double delta, double* F) {
    double mu = mu_of(M, TF);
    double kappa = mu * (M->Cp / M->Pr);
    double snT = (TR - TL) / delta;
    double gTD = dot3(gTF, D), gT[3], gU[9];
    for (int k = 0; k < 3; k++) gT[k] = gTF[k] + snT * D[k] - gTD * D[k];
    for (int i = 0; i < 3; i++) {
        double snU = (UR[i] - UL[i]) / delta;
        double gUD = gUF[3 * i] * D[0] + gUF[3 * i + 1] * D[1] + gUF[3 * i + 2] * D[2];
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUF[3 * i + k] + snU * D[k] - gUD * D[k];
    }
    double qF = kappa * dot3(gT, N);
    double tmp3 = gU[0] + gU[4] + gU[8], sigma[3];
    for (int i = 0; i < 3; i++) {
        double tmp2 = (gU[3 * i] + gU[i]) * N[0] + (gU[3 * i + 1] + gU[3 + i]) * N[1] + (gU[3 * i + 2] + gU[6 + i]) * N[2];
        sigma[i] = mu * (tmp2 - 2. / 3 * tmp3 * N[i]);
    }
    for (int i = 0; i < 3; i++) F[1 + i] = F[1 + i] + (-sigma[i]);
    F[4] = F[4] + (-(qF + dot3(sigma, UF)));
}

/* rec: nCells x 20 (U3 T p gU9 gT3 gp3); face fluxes: nF x 6 */
static void face_flux(const oracle_mesh* M, const double* rec, int f, double* out) {
    int kind = f < M->nIF ? F_INTERNAL : M->fkind[f - M->nIF];
    int P = M->own[f], Nn = M->nbr[f];
    int Ng = f < M->nIF ? Nn : M->gsrc[Nn - M->nIC];
    const double *rP = rec + 20 * (size_t)P, *rN = rec + 20 * (size_t)Nn, *rG = rec + 20 * (size_t)Ng;
    const double* N = M->nrm + 3 * (size_t)f;
    double F[5], TF, UF[3], gTF[3], gUF[9];
    if (kind == F_BOUNDARY) {
        double rho, rU[3], rE;
        conservative(M, rN, rN[3], rN[4], &rho, rU, &rE);
        double Un = dot3(rN, N);
        F[0] = rho * Un;
        for (int k = 0; k < 3; k++) F[1 + k] = rU[k] * Un + rN[4] * N[k];
        F[4] = (rE + rN[4]) * Un;
        TF = rN[3];
        for (int k = 0; k < 3; k++) { UF[k] = rN[k]; gTF[k] = rG[14 + k]; }
        for (int k = 0; k < 9; k++) gUF[k] = rG[5 + k];
    } else {
        const double* qw0 = M->qw + 6 * (size_t)f;
        const double* qw1 = qw0 + 3;
        double lw0 = M->lw[2 * (size_t)f], lw1 = M->lw[2 * (size_t)f + 1];
        double ULF[3], URF[3], TLF, TRF, pLF, pRF;
        for (int k = 0; k < 3; k++) ULF[k] = recon(rP[k], rN[k], rP + 5 + 3 * k, lw0, qw0);
        TLF = recon(rP[3], rN[3], rP + 14, lw0, qw0);
        pLF = recon(rP[4], rN[4], rP + 17, lw0, qw0);
        double rhoL, rUL[3], rEL, rhoR, rUR[3], rER;
        conservative(M, ULF, TLF, pLF, &rhoL, rUL, &rEL);
        int solver;
        if (kind == F_CHAR) {
            for (int k = 0; k < 3; k++) URF[k] = rN[k];
            TRF = rN[3]; pRF = rN[4];
            solver = M->briemann;
        } else {
            for (int k = 0; k < 3; k++) URF[k] = recon(rN[k], rP[k], rG + 5 + 3 * k, lw1, qw1);
            TRF = recon(rN[3], rP[3], rG + 14, lw1, qw1);
            pRF = recon(rN[4], rP[4], rG + 17, lw1, qw1);
            solver = M->riemann;
        }
        conservative(M, URF, TRF, pRF, &rhoR, rUR, &rER);
        if (solver == 0) roe(M, pLF, pRF, ULF, URF, rhoL, rhoR, N, F);
        else laxf(M, pLF, pRF, ULF, URF, rhoL, rhoR, rUL, rUR, rEL, rER, N, F);
        if (kind == F_CHAR) {
            TF = rN[3];
            for (int k = 0; k < 3; k++) { UF[k] = rN[k]; gTF[k] = rG[14 + k]; }
            for (int k = 0; k < 9; k++) gUF[k] = rG[5 + k];
        } else {
            TF = 0.5 * (TLF + TRF);
            for (int k = 0; k < 3; k++) { UF[k] = 0.5 * (ULF[k] + URF[k]); gTF[k] = 0.5 * (rP[14 + k] + rG[14 + k]); }
            for (int k = 0; k < 9; k++) gUF[k] = 0.5 * (rP[5 + k] + rG[5 + k]);
        }
    }
    if (!(M->muModel == 0 && M->mu0 == 0.0))
        viscous(M, rP[3], rN[3], rP, rN, TF, UF, gTF, gUF, M->du + 3 * (size_t)f, N, M->dlt[f], F);
    double aF = sqrt(M->Cp * TF * (M->gamma - 1));
    for (int k = 0; k < 5; k++) out[k] = F[k];
    out[5] = fabs(dot3(UF, N)) + aF;
}

static void gradients(const oracle_mesh* M, double* rec);
static void prims_ghosts(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double* rec);

/* residual of state (rho, rU, rE) into R (nIC x 5) and the CFL sums; objective if want */
static void equation(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double* rec,
                     double* ff, double* R, double* dtc, double* obj) {
    int nIC = M->nIC;
    prims_ghosts(M, rho, rU, rE, rec);
    if (obj) {
        double v = 0.0;
        if (M->objective == 1) {
            double Cv = M->Cp / M->gamma;
            for (int c = 0; c < nIC; c++) {
                const double* r = rec + 20 * (size_t)c;
                double rh = r[4] / ((Cv * r[3]) * (M->gamma - 1));
                v = v + 0.5 * rh * dot3(r, r) * M->vol[c];
            }
        } else if (M->objective == 3) {
            for (int c = 0; c < nIC; c++) v = v + rec[20 * (size_t)c + 3] * 1;
        } else if (M->objective == 2) {
            for (int i = 0; i < M->objN; i++) {
                int f = M->objStart + i;
                const double *rN = rec + 20 * (size_t)M->nbr[f], *rP = rec + 20 * (size_t)M->own[f];
                double mung = mu_of(M, rN[3]) * (rN[0] - rP[0]) / M->dlt[f];
                v = v + (rN[4] * M->nrm[3 * (size_t)f] - mung) * M->area[f];
            }
        } else if (M->objective == 4) {
            /* pressure loss over the plane cells, normalised by the mass flux through them */
            double g = M->gamma, Cv = M->Cp / M->gamma, w = 0.0, pl = 0.0, w2 = 0.0, ht = 0.0;
            for (int q = 0; q < M->nPlane; q++) {
                const double* r = rec + 20 * (size_t)M->planeCells[q];
                double rh = r[4] / (Cv * r[3] * (g - 1));
                double rUn = 0.0 + rh * r[0] * M->vn[0] + rh * r[1] * M->vn[1] + rh * r[2] * M->vn[2];
                w = w + rUn * M->planeAreas[q];
            }
            for (int q = 0; q < M->nPlane; q++) {
                const double* r = rec + 20 * (size_t)M->planeCells[q];
                double rh = r[4] / (Cv * r[3] * (g - 1));
                double c = sqrt(g * r[4] / rh);
                double rUn = 0.0 + rh * r[0] * M->vn[0] + rh * r[1] * M->vn[1] + rh * r[2] * M->vn[2];
                double Mi = sqrt(dot3(r, r)) / c;
                double pt = r[4] * pow(1 + 0.5 * (g - 1) * Mi * Mi, g / (g - 1));
                pl = pl + (M->ptin - pt) * rUn * M->planeAreas[q] / M->ptin / w;
            }
            /* weighted wall heat transfer k (Tw - T_owner)/delta A w / sum A w */
            double k = M->Cp * mu_of(M, M->Tw) / M->Pr;
            for (int q = 0; q < M->nHeat; q++) w2 = w2 + M->area[M->heatFaces[q]] * M->heatW[q];
            for (int q = 0; q < M->nHeat; q++) {
                int f = M->heatFaces[q];
                double dtdn = (M->Tw - rec[20 * (size_t)M->own[f] + 3]) / M->dlt[f];
                ht = ht + k * dtdn * M->area[f] * M->heatW[q] / w2;
            }
            v = M->va * pl + M->vb * ht;
        }
        *obj = v;
    }
    gradients(M, rec);
#pragma omp parallel for schedule(static)
    for (int f = 0; f < M->nF; f++) face_flux(M, rec, f, ff + 6 * (size_t)f);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nIC; c++) {
        double acc[5] = {0, 0, 0, 0, 0}, d = 0;
        for (int s = 0; s < 6; s++) {
            int e = M->accf[6 * (size_t)c + s];
            int own = e >= 0, f = own ? e : ~e;
            double w = own ? M->area[f] / M->vol[M->own[f]] : M->area[f] / M->vol[M->nbr[f]];
            const double* F = ff + 6 * (size_t)f;
            for (int q = 0; q < 5; q++) {
                double t = F[q] * w;
                acc[q] = acc[q] + (own ? t : -t);
            }
            d = d + F[5] * w;
        }
        for (int q = 0; q < 5; q++) R[5 * (size_t)c + q] = acc[q];
        dtc[c] = d;
    }
}

/* gradCell, cellFaces order (op.py:45-63), into the records' gradient part */
static void prims_ghosts(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double* rec) {
    int nIC = M->nIC, nG = M->nG;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nIC; c++) {
        double* r = rec + 20 * (size_t)c;
        primitive(M, rho[c], rU + 3 * (size_t)c, rE[c], r, r + 3, r + 4);
    }
#pragma omp parallel for schedule(static)
    for (int g = 0; g < nG; g++) {
        const double* s = rec + 20 * (size_t)M->gsrc[g];
        double* r = rec + 20 * (size_t)(nIC + g);
        for (int k = 0; k < 5; k++) r[k] = s[k];
        int kind = M->gkind[g];
        int kU = kind & 7, kT = (kind >> 3) & 7, kp = (kind >> 6) & 7;
        const double* n = M->nrm + 3 * (size_t)(M->nIF + g);
        if (kU == K_TOTALPT) {
            /* CBC_TOTAL_PT, BCs.py:178-184 */
            const double* d = M->gval + 5 * (size_t)g;
            double Tt = d[3], pt = d[4], T = r[3];
            double Un = dot3(r, d);
            for (int k = 0; k < 3; k++) r[k] = Un * d[k];
            r[3] = Tt - 0.5 * Un * Un / M->Cp;
            r[4] = pt * pow(T / Tt, M->gamma / (M->gamma - 1));
            continue;
        }
        if (kU == K_FIXED) for (int k = 0; k < 3; k++) r[k] = M->gval[5 * (size_t)g + k] * 1;
        else if (kU == K_SYM) {
            double un = dot3(r, n);
            for (int k = 0; k < 3; k++) r[k] = r[k] - un * n[k];
        }
        if (kT == K_FIXED) r[3] = M->gval[5 * (size_t)g + 3] * 1;
        if (kp == K_FIXED) r[4] = M->gval[5 * (size_t)g + 4] * 1;
    }
}

static void gradients(const oracle_mesh* M, double* rec) {
    int nIC = M->nIC;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nIC; c++) {
        double g[15];
        const double* rc = rec + 20 * (size_t)c;
        for (int s = 0; s < 6; s++) {
            int f = M->cellFaces[6 * (size_t)c + s];
            double S = M->area[f], O = (double)M->cellOwn[6 * (size_t)c + s];
            const double* N0 = M->nrm + 3 * (size_t)f;
            double N[3], w = M->wts[f];
            for (int k = 0; k < 3; k++) N[k] = 2 * N0[k] * O - N0[k];
            w = w + O - 2 * w * O;
            const double* rn = rec + 20 * (size_t)M->cellNbr[6 * (size_t)c + s];
            double phiF[5];
            for (int k = 0; k < 5; k++) phiF[k] = rc[k] * (-w + 1) + rn[k] * w;
            double SN[3] = {S * N[0], S * N[1], S * N[2]};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    double t = phiF[i] * SN[j];
                    g[3 * i + j] = s == 0 ? t : g[3 * i + j] + t;
                }
            for (int i = 3; i < 5; i++)
                for (int j = 0; j < 3; j++) {
                    double t = phiF[i] * S * N[j];
                    g[3 * i + j] = s == 0 ? t : g[3 * i + j] + t;
                }
        }
        double* out = rec + 20 * (size_t)c + 5;
        for (int k = 0; k < 15; k++) out[k] = g[k] / M->vol[c];
    }
}

/* one SSP-RK3 step. work: oracle_work_doubles(M) doubles. S: nIC x 5 or NULL. */
void oracle_step(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double dt,
                 const double* S, double* rhoN, double* rUN, double* rEN, double* dtcMax, double* obj,
                 double* work) {
    int nIC = M->nIC;
    double* rec = work;
    double* ff = rec + 20 * (size_t)(nIC + M->nG);
    double* R = ff + 6 * (size_t)M->nF;
    double* dtc = R + 5 * (size_t)nIC;
    /* stage states in the reference layout: rho (n), rhoU (n x 3), rhoE (n) */
    double* st1 = dtc + nIC;
    double* st2 = st1 + 5 * (size_t)nIC;
    const double* sr[3] = {rho, st1, st2};
    const double* su[3] = {rU, st1 + nIC, st2 + nIC};
    const double* se[3] = {rE, st1 + 4 * (size_t)nIC, st2 + 4 * (size_t)nIC};
    double* orr[3] = {st1, st2, rhoN};
    double* ou[3] = {st1 + nIC, st2 + nIC, rUN};
    double* oe[3] = {st1 + 4 * (size_t)nIC, st2 + 4 * (size_t)nIC, rEN};
    const double alpha[3][3] = {{1, 0, 0}, {3. / 4, 1. / 4, 0}, {1. / 3, 0, 2. / 3}};
    const double beta[3] = {1, 1. / 4, 2. / 3};
    for (int i = 0; i < 3; i++) {
        double o = 0.0;
        equation(M, sr[i], su[i], se[i], rec, ff, R, dtc, i == 1 ? &o : NULL);
        if (i == 1) {
            double mx = 0;
            for (int c = 0; c < nIC; c++) mx = dtc[c] > mx ? dtc[c] : mx;
            *dtcMax = mx;
            *obj = M->objective ? o : 0.0;
        }
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nIC; c++) {
            for (int q = 0; q < 5; q++) {
                double cur = 0;
                for (int j = 0; j <= i; j++) {
                    double fj = q == 0 ? sr[j][c] : (q < 4 ? su[j][3 * (size_t)c + q - 1] : se[j][c]);
                    cur = cur + alpha[i][j] * fj;
                }
                double Sq = S ? S[5 * (size_t)c + q] : 0.0;
                cur = cur + (-beta[i] * (R[5 * (size_t)c + q] - Sq)) * dt;
                if (q == 0) orr[i][c] = cur;
                else if (q < 4) ou[i][3 * (size_t)c + q - 1] = cur;
                else oe[i][c] = cur;
            }
        }
    }
}

size_t oracle_work_doubles(const oracle_mesh* M) {
    return 20 * (size_t)(M->nIC + M->nG) + 6 * (size_t)M->nF + 5 * (size_t)M->nIC + (size_t)M->nIC +
           10 * (size_t)M->nIC;
}

/* the cell records (primitives with ghost rows, then gradients; 20 values a cell) of a state:
 * what the residual reads, for the host adjoint (oracle/c/adjoint_host.cpp). work: as for
 * oracle_step (its first 20 (nIC + nG) values are the records). */
void oracle_records(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double* work) {
    prims_ghosts(M, rho, rU, rE, work);
    gradients(M, work);
}

/* the RK stage states u1 (k = 1) and u2 (k = 2) a finished oracle_step left in its work */
double* oracle_work_stage(const oracle_mesh* M, double* work, int k) {
    double* st1 = work + 20 * (size_t)(M->nIC + M->nG) + 6 * (size_t)M->nF + 5 * (size_t)M->nIC + (size_t)M->nIC;
    return k == 1 ? st1 : st1 + 5 * (size_t)M->nIC;
}
