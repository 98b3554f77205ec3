// Device-side physics of the compressible finite-volume residual.
//
// Each function states the reference expression it evaluates; operands are combined in the
// reference's order (left to right). FMA contraction is allowed, so results agree with the
// reference to rounding, not bit for bit.
#pragma once
#include <stdint.h>
#include "afvm.h"

// The face physics is written once for the device and, for the unit tests of the hand-derived
// adjoint, also compiles as plain host C++.
#ifdef __CUDACC__
#include <cuda_runtime.h>
#define AFVM_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define AFVM_HD inline
using std::fabs;
using std::fmax;
using std::sqrt;
#endif

namespace afvm {

// per-cell record: primitive state then its gradients (reference layouts: U (3), T, p,
// gradU [component][direction] (3x3), gradT (1x3), gradp (1x3))
constexpr int REC = 20;
constexpr int R_U = 0, R_T = 3, R_P = 4, R_GU = 5, R_GT = 14, R_GP = 17;
// per-face flux record: rho, rhoU (3), rhoE fluxes and the CFL term (|U.n| + a)
constexpr int FREC = 6;

// kinds of faces
constexpr int FACE_INTERNAL = 0, FACE_COUPLED = 1, FACE_CHARACTERISTIC = 2, FACE_BOUNDARY = 3;

struct Phys {
    double gamma, gm1, Cp, Cv, rCv, kFac, mu0, muAs, muTs, small;
    int muModel, riemann, briemann;
};

template <typename R>
AFVM_HD R dot3(const R* a, const R* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// mu(T): constant, or Sutherland 1.4792e-06*T**1.5/(T+116.) (adFVM/density.py:27)
template <typename R>
AFVM_HD R viscosity(const Phys& P, R T) {
    if (P.muModel == AFVM_MU_SUTHERLAND) return (R(P.muAs) * (T * sqrt(T))) / (T + R(P.muTs));
    return R(P.mu0);
}

// RCF.conservative (adFVM/density.py:173-181)
template <typename R>
AFVM_HD void conservative(const Phys& P, const R* U, R T, R p, R& rho, R* rhoU, R& rhoE) {
    R e = R(P.Cv) * T;
    rho = p / (e * R(P.gm1));
    rhoE = rho * (e + R(0.5) * dot3(U, U));
    rhoU[0] = U[0] * rho; rhoU[1] = U[1] * rho; rhoU[2] = U[2] * rho;
}

// interp.secondOrder for one side (adFVM/interp.py:20-28): phiC + (phiD-phiC)*lw + qw.grad
template <typename R>
AFVM_HD R recon(R phiC, R phiD, const R* g, R lw, const R* qw) {
    R phiF = phiC + (phiD - phiC) * lw;
    return phiF + (qw[0] * g[0] + qw[1] * g[1] + qw[2] * g[2]);
}

// riemann.eulerRoe (adFVM/riemann.py:21-70)
template <typename R>
AFVM_HD void roe(const Phys& P, R pL, R pR, const R* UL, const R* UR, R rhoL, R rhoR,
                                    const R* N, R* F) {
    const R g = R(P.gamma), gm1 = R(P.gm1);
    R rhoUnL = rhoL * dot3(UL, N), rhoUnR = rhoR * dot3(UR, N);
    R hL = g * pL / (gm1 * rhoL) + R(0.5) * dot3(UL, UL);
    R hR = g * pR / (gm1 * rhoR) + R(0.5) * dot3(UR, UR);
    R fr = R(0.5) * (rhoUnL + rhoUnR);
    R fu[3], UF[3], dU[3];
    for (int k = 0; k < 3; k++) fu[k] = R(0.5) * (rhoUnL * UL[k] + rhoUnR * UR[k] + (pL + pR) * N[k]);
    R fe = R(0.5) * (rhoUnL * hL + rhoUnR * hR);
    R sL = sqrt(rhoL), sR = sqrt(rhoR);
    R divRho = sL + sR;
    for (int k = 0; k < 3; k++) UF[k] = (UL[k] * sL + UR[k] * sR) / divRho;
    R hF = (hL * sL + hR * sR) / divRho;
    R qF = R(0.5) * dot3(UF, UF);
    R a2F = gm1 * (hF - qF);
    R aF = sqrt(a2F);
    R UnF = dot3(UF, N);
    R drho = rhoR - rhoL;
    for (int k = 0; k < 3; k++) dU[k] = rhoR * UR[k] - rhoL * UL[k];
    R drhoE = (hR * rhoR - pR) - (hL * rhoL - pL);
    R lam1 = fabs(UnF), lam2 = fabs(UnF + aF), lam3 = fabs(UnF - aF);
    R eps = R(0.5) * fabs(rhoUnL / rhoL - rhoUnR / rhoR);
    eps = eps + R(0.5) * fabs(sqrt(g * pL / rhoL) - sqrt(g * pR / rhoR));
    eps = (eps < R(0)) ? eps - R(P.small) : eps + R(P.small);
    if (lam1 < R(2) * eps) lam1 = R(0.25) * lam1 * lam1 / eps + eps;
    if (lam2 < R(2) * eps) lam2 = R(0.25) * lam2 * lam2 / eps + eps;
    if (lam3 < R(2) * eps) lam3 = R(0.25) * lam3 * lam3 / eps + eps;
    R abv1 = R(0.5) * (lam2 + lam3);
    R abv2 = R(0.5) * (lam2 - lam3);
    R abv3 = abv1 - lam1;
    R abv4 = gm1 * (qF * drho - dot3(UF, dU) + drhoE);
    R abv5 = UnF * drho - dot3(dU, N);
    R abv6 = abv3 * abv4 / a2F - abv2 * abv5 / aF;
    R abv7 = abv3 * abv5 - abv2 * abv4 / aF;
    F[0] = fr - R(0.5) * (lam1 * drho + abv6);
    for (int k = 0; k < 3; k++) F[1 + k] = fu[k] - R(0.5) * (lam1 * dU[k] + UF[k] * abv6 - abv7 * N[k]);
    F[4] = fe - R(0.5) * (lam1 * drhoE + hF * abv6 - UnF * abv7);
}

// riemann.eulerLaxFriedrichs (adFVM/riemann.py:6-18)
template <typename R>
AFVM_HD void laxf(const Phys& P, R pL, R pR, const R* UL, const R* UR, R rhoL, R rhoR,
                                     const R* rhoUL, const R* rhoUR, R rhoEL, R rhoER, const R* N, R* F) {
    const R g = R(P.gamma);
    R UnL = dot3(UL, N), UnR = dot3(UR, N);
    R cL = sqrt(g * pL / rhoL);
    R cR = sqrt(g * pR / rhoR);
    R aF = fmax(fabs(UnL) + cL, fabs(UnR) + cR);
    R ha = R(0.5) * aF;
    F[0] = R(0.5) * (rhoL * UnL + rhoR * UnR) - ha * (rhoR - rhoL);
    for (int k = 0; k < 3; k++)
        F[1 + k] = R(0.5) * (rhoUL[k] * UnL + rhoUR[k] * UnR + (pL + pR) * N[k]) - ha * (rhoUR[k] - rhoUL[k]);
    F[4] = R(0.5) * ((rhoEL + pL) * UnL + (rhoER + pR) * UnR) - ha * (rhoER - rhoEL);
}

// RCF.viscousFlux (adFVM/density.py:192-222): adds -sigma to F[1..3] and -(q + sigma.UF) to F[4]
template <typename R>
AFVM_HD void viscous(const Phys& P, R TL, R TR, const R* UL, const R* UR, R TF, const R* UF,
                                        const R* gTF, const R* gUF, const R* D, const R* N, R delta, R* F) {
    R mu = viscosity<R>(P, TF);
    R kappa = mu * R(P.kFac);
    R snT = (TR - TL) / delta;
    R gTD = dot3(gTF, D);
    R gT[3];
    for (int k = 0; k < 3; k++) gT[k] = gTF[k] + snT * D[k] - gTD * D[k];
    R gU[9];
    for (int i = 0; i < 3; i++) {
        R snU = (UR[i] - UL[i]) / delta;
        R gUD = gUF[3 * i] * D[0] + gUF[3 * i + 1] * D[1] + gUF[3 * i + 2] * D[2];
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUF[3 * i + k] + snU * D[k] - gUD * D[k];
    }
    R qF = kappa * dot3(gT, N);
    R tmp3 = gU[0] + gU[4] + gU[8];
    R sigma[3];
    for (int i = 0; i < 3; i++) {
        R tmp2 = (gU[3 * i] + gU[i]) * N[0] + (gU[3 * i + 1] + gU[3 + i]) * N[1] + (gU[3 * i + 2] + gU[6 + i]) * N[2];
        sigma[i] = mu * (tmp2 - R(2.0 / 3) * tmp3 * N[i]);
    }
    F[1] = F[1] + (-sigma[0]);
    F[2] = F[2] + (-sigma[1]);
    F[3] = F[3] + (-sigma[2]);
    F[4] = F[4] + (-(qF + dot3(sigma, UF)));
}

}  // namespace afvm
