// The flux through one face and its hand-derived vector-Jacobian product.
//
// face_flux evaluates RCF.flux / RCF.boundaryFlux (adFVM/density.py:253-331) for one face;
// face_vjp returns the gradient of <Fbar, F> with respect to every input of the face (the
// primitives and gradients of the two adjacent cells). The reference differentiates the
// same arithmetic with adpy's reverse mode (apps/adjoint.py:101); here each forward
// expression is differentiated by hand, in reverse order. At the kinks of |x| the derivative
// taken is sign(x) with sign(0) = 0; at max(a, b) with a == b the whole derivative goes to a.
#pragma once
#include <type_traits>
#include "physics.cuh"

namespace afvm {

template <typename R>
struct FaceIn {
    R UP[3], TP, pP, UN[3], TN, pN;                    // owner cell and neighbour (or ghost) primitives
    R gUP[9], gTP[3], gpP[3], gUN[9], gTN[3], gpN[3];  // gradients ([component][direction])
    R N[3], D[3], lw0, lw1, qw0[3], qw1[3], rdelta;    // normals, deltasUnit, weights, 1/deltas
    R Nt[3], ND;                                       // derived: N - (N.D) D and N.D (face_derived)
};

// the derived geometry of a face from its normal and deltasUnit, formed in double (the device
// reads the same values from mesh tables built this way)
template <typename R>
AFVM_HD void face_derived(FaceIn<R>& in) {
    double nd = (double)in.N[0] * in.D[0] + (double)in.N[1] * in.D[1] + (double)in.N[2] * in.D[2];
    in.ND = R(nd);
    for (int k = 0; k < 3; k++) in.Nt[k] = R((double)in.N[k] - nd * (double)in.D[k]);
}

template <typename R>
struct FaceBar {
    R UP[3], TP, pP, UN[3], TN, pN;
    R gUP[9], gTP[3], gpP[3], gUN[9], gTN[3], gpN[3];
};

// The start of a sum that the compiler may drop: -0 + x is x for every x (IEEE 754), while
// +0 + x turns x = -0 into +0, so a sum started at +0 costs one add (in double an FP64 pipe
// issue) for its first term. The adjoint accumulators start at -0; one that receives no term
// ends as -0.
template <typename R>
AFVM_HD constexpr R acc0() { return R(-0.0); }

template <typename R>
AFVM_HD void zero_bar(FaceBar<R>& b) {
    R* p = &b.UP[0];
    for (int k = 0; k < 40; k++) p[k] = acc0<R>();
}

// Adjoint of a face's geometry inputs (FaceIn's N, D, lw0, lw1, qw0, qw1, 1/deltas), for the
// gradient with respect to the mesh tensors (the reference's parameters = 'mesh',
// apps/adjoint.py:108-110). The VJP functions take an optional GeoBar; with none (GeoNone, the
// default) the geometry terms are not compiled at all.
template <typename R>
struct GeoBar {
    R N[3], D[3], lw0, lw1, qw0[3], qw1[3], rdelta;
};
struct GeoNone {};
template <typename G>
constexpr bool kGeo = !std::is_same<G, GeoNone>::value;

template <typename R>
AFVM_HD void zero_geo(GeoBar<R>& g) {
    R* p = &g.N[0];
    for (int k = 0; k < 15; k++) p[k] = acc0<R>();
}


// the gauge-form face flux: as face_flux below, from gauge offsets of p and T (the viscous
// terms use T only through differences and mu(T_F), T_F absolute)
template <typename R>
AFVM_HD void face_flux_gauge(const Phys& P, int kind, bool inviscid, const FaceIn<R>& in, R* F, R& maxaF) {
    const PhysR<R>& Q = consts<R>(P);
    R TF, Us[3], gTs[3], gUs[9];
    if (kind == FACE_BOUNDARY) {
        // RCF.boundaryFlux: (rho Un, rho U Un + p N, rho h Un) less gP N and gH rho Un
        R rho, rhoU[3], rhoE;
        conservative<R>(P, in.UN, in.TN + Q.gT, in.pN + Q.gP, rho, rhoU, rhoE);
        R Un = dot3(in.UN, in.N);
        R hg = Q.Cp * in.TN + (R(0.5) * dot3(in.UN, in.UN) - Q.gK);
        F[0] = rho * Un;
        for (int k = 0; k < 3; k++) F[1 + k] = rhoU[k] * Un + in.pN * in.N[k];
        F[4] = rho * hg * Un;
        TF = in.TN + Q.gT;
        for (int k = 0; k < 3; k++) { Us[k] = in.UN[k]; gTs[k] = in.gTN[k]; }
        for (int k = 0; k < 9; k++) gUs[k] = in.gUN[k];
    } else {
        R ULF[3], TLF, pLF, URF[3], TRF, pRF;
        // the jumps neighbour - owner, shared by the two sides' reconstructions
        R dU[3], dT = in.TN - in.TP, dp = in.pN - in.pP;
        for (int k = 0; k < 3; k++) dU[k] = in.UN[k] - in.UP[k];
        for (int k = 0; k < 3; k++) ULF[k] = recon<R>(in.UP[k], dU[k], in.gUP + 3 * k, in.lw0, in.qw0);
        TLF = recon<R>(in.TP, dT, in.gTP, in.lw0, in.qw0);
        pLF = recon<R>(in.pP, dp, in.gpP, in.lw0, in.qw0);
        R rhoL, rhoUL[3], rhoEL, rdL, rdR;
        conservative<R>(P, ULF, TLF + Q.gT, pLF + Q.gP, rhoL, rhoUL, rhoEL, &rdL);
        int solver;
        if (kind == FACE_CHARACTERISTIC) {
            for (int k = 0; k < 3; k++) URF[k] = in.UN[k];
            TRF = in.TN; pRF = in.pN;
            solver = P.briemann;
        } else {
            for (int k = 0; k < 3; k++) URF[k] = recon<R>(in.UN[k], -dU[k], in.gUN + 3 * k, in.lw1, in.qw1);
            TRF = recon<R>(in.TN, -dT, in.gTN, in.lw1, in.qw1);
            pRF = recon<R>(in.pN, -dp, in.gpN, in.lw1, in.qw1);
            solver = P.riemann;
        }
        R rhoR, rhoUR[3], rhoER;
        conservative<R>(P, URF, TRF + Q.gT, pRF + Q.gP, rhoR, rhoUR, rhoER, &rdR);
        if (solver == AFVM_RIEMANN_ROE)
            roe_gauge<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, rdL, rdR, in.N, F);
        else
            laxf_gauge<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, rdL, rdR, in.N, F);
        if (kind == FACE_CHARACTERISTIC) {
            TF = in.TN + Q.gT;
            for (int k = 0; k < 3; k++) { Us[k] = in.UN[k]; gTs[k] = in.gTN[k]; }
            for (int k = 0; k < 9; k++) gUs[k] = in.gUN[k];
        } else {
            // the face averages themselves (scale 1 below: the float kernel, capped at 64
            // registers, spills less than with the sums and a runtime scale)
            TF = R(0.5) * (TLF + TRF) + Q.gT;
            for (int k = 0; k < 3; k++) { Us[k] = R(0.5) * (ULF[k] + URF[k]); gTs[k] = R(0.5) * (in.gTP[k] + in.gTN[k]); }
            for (int k = 0; k < 9; k++) gUs[k] = R(0.5) * (in.gUP[k] + in.gUN[k]);
        }
    }
    if (!inviscid) {
        R Fv[4];
        viscous<R>(P, in.TP, in.TN, in.UP, in.UN, TF, Us, gTs, gUs, R(1), false, in.D, in.N, in.Nt, in.ND, in.rdelta,
                   Fv);
        for (int k = 0; k < 3; k++) F[1 + k] = F[1 + k] - Fv[k];
        F[4] = F[4] - Fv[3];
    }
    R aF = sqrt_(Q.Cp * TF * Q.gm1);
    maxaF = fabs(dot3(Us, in.N)) + aF;
}

// flux (rho, rhoU, rhoE) through the face and the CFL term |U.n| + a; the tape values of a
// non-boundary face go to tp. GAUGE: the pressures and temperatures of `in` are gauge offsets
// (FP32 records) and F is the gauge-form flux (physics.cuh: roe_gauge); never taped.
template <typename R, bool GAUGE = false, typename Sink = TapeNone>
AFVM_HD void face_flux(const Phys& P, int kind, bool inviscid, const FaceIn<R>& in, R* F, R& maxaF,
                       Sink&& tp = Sink()) {
    if constexpr (GAUGE) {
        face_flux_gauge<R>(P, kind, inviscid, in, F, maxaF);
        return;
    }
    R TF, Us[3], gTs[3], gUs[9], hs;
    bool sums;
    // the viscous terms (sigma and q + sigma.U_F), subtracted from the inviscid flux
    R Fv[4] = {R(0), R(0), R(0), R(0)};
    if (kind == FACE_BOUNDARY) {
        // RCF.boundaryFlux (density.py:307-331) with RCF.getFlux (density.py:184-190)
        R rho, rhoU[3], rhoE;
        conservative<R>(P, in.UN, in.TN, in.pN, rho, rhoU, rhoE);
        R Un = dot3(in.UN, in.N);
        F[0] = rho * Un;
        for (int k = 0; k < 3; k++) F[1 + k] = rhoU[k] * Un + in.pN * in.N[k];
        F[4] = (rhoE + in.pN) * Un;
        TF = in.TN;
        for (int k = 0; k < 3; k++) { Us[k] = in.UN[k]; gTs[k] = in.gTN[k]; }
        for (int k = 0; k < 9; k++) gUs[k] = in.gUN[k];
        hs = R(1); sums = false;
        if (!inviscid) {
            viscous<R>(P, in.TP, in.TN, in.UP, in.UN, TF, Us, gTs, gUs, hs, sums, in.D, in.N, in.Nt, in.ND, in.rdelta,
                       Fv, tp);
            for (int k = 0; k < 3; k++) F[1 + k] = F[1 + k] - Fv[k];
            F[4] = F[4] - Fv[3];
        }
    } else {
        R ULF[3], TLF, pLF, URF[3], TRF, pRF;
        // the jumps neighbour - owner, shared by the two sides' reconstructions
        R dU[3], dT = in.TN - in.TP, dp = in.pN - in.pP;
        for (int k = 0; k < 3; k++) dU[k] = in.UN[k] - in.UP[k];
        for (int k = 0; k < 3; k++) ULF[k] = recon<R>(in.UP[k], dU[k], in.gUP + 3 * k, in.lw0, in.qw0);
        TLF = recon<R>(in.TP, dT, in.gTP, in.lw0, in.qw0);
        pLF = recon<R>(in.pP, dp, in.gpP, in.lw0, in.qw0);
        R rhoL, rhoUL[3], rhoEL, rdL, rdR;
        conservative<R>(P, ULF, TLF, pLF, rhoL, rhoUL, rhoEL, &rdL);
        int solver;
        if (kind == FACE_CHARACTERISTIC) {
            for (int k = 0; k < 3; k++) URF[k] = in.UN[k];
            TRF = in.TN; pRF = in.pN;
            solver = P.briemann;
        } else {
            for (int k = 0; k < 3; k++) URF[k] = recon<R>(in.UN[k], -dU[k], in.gUN + 3 * k, in.lw1, in.qw1);
            TRF = recon<R>(in.TN, -dT, in.gTN, in.lw1, in.qw1);
            pRF = recon<R>(in.pN, -dp, in.gpN, in.lw1, in.qw1);
            solver = P.riemann;
        }
        R rhoR, rhoUR[3], rhoER;
        conservative<R>(P, URF, TRF, pRF, rhoR, rhoUR, rhoER, &rdR);
        for (int k = 0; k < 3; k++) { tp.put(T_ULF + k, ULF[k]); tp.put(T_URF + k, URF[k]); }
        tp.put(T_TLF, TLF); tp.put(T_PLF, pLF); tp.put(T_TRF, TRF); tp.put(T_PRF, pRF);
        tp.put(T_RDL, rdL); tp.put(T_RDR, rdR);
        if (kind == FACE_CHARACTERISTIC) {
            TF = in.TN;
            for (int k = 0; k < 3; k++) { Us[k] = in.UN[k]; gTs[k] = in.gTN[k]; }
            for (int k = 0; k < 9; k++) gUs[k] = in.gUN[k];
            hs = R(1); sums = false;
        } else {
            // the face averages (density.py:290-291) as hs = 1/2 times the two sides' sums
            TF = R(0.5) * (TLF + TRF);
            for (int k = 0; k < 3; k++) { Us[k] = ULF[k] + URF[k]; gTs[k] = in.gTP[k] + in.gTN[k]; }
            for (int k = 0; k < 9; k++) gUs[k] = in.gUP[k] + in.gUN[k];
            hs = R(0.5); sums = true;
        }
        if (!inviscid)
            viscous<R>(P, in.TP, in.TN, in.UP, in.UN, TF, Us, gTs, gUs, hs, sums, in.D, in.N, in.Nt, in.ND, in.rdelta,
                       Fv, tp);
        if (solver == AFVM_RIEMANN_ROE) {
            roe<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, in.N, Fv, F, tp);
        } else {
            laxf<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, rhoUL, rhoUR, rhoEL, rhoER, in.N, F, tp);
            for (int k = 0; k < 3; k++) F[1 + k] = F[1 + k] - Fv[k];
            F[4] = F[4] - Fv[3];
        }
    }
    R aF = sqrt_(consts<R>(P).Cp * TF * consts<R>(P).gm1);
    maxaF = fabs(hs * dot3(Us, in.N)) + aF;
}

// ---------------------------------------------------------------------------- adjoints

// RCF.conservative: rho = p/(Cv T (g-1)), rhoU = U rho, rhoE = rho (Cv T + |U|^2/2)
// (rd = 1/(e (g-1)), the forward's reciprocal)
template <typename R>
AFVM_HD void conservative_vjp_t(const Phys& P, const R* U, R T, R p, R rd, R rhob, const R* rhoUb, R rhoEb,
                                R* Ub, R& Tb, R& pb) {
    R e = consts<R>(P).Cv * T;
    R rho = p * rd;
    R q = dot3(U, U);
    for (int k = 0; k < 3; k++) Ub[k] += rhoUb[k] * rho + rhoEb * rho * U[k];
    R rhot = rhob + dot3(rhoUb, U) + rhoEb * (e + R(0.5) * q);
    pb += rhot * rd;
    R eb = -rhot * rho * (rd * consts<R>(P).gm1) + rhoEb * rho;    // 1/e = rd (g-1)
    Tb += eb * consts<R>(P).Cv;
}

template <typename R>
AFVM_HD void conservative_vjp(const Phys& P, const R* U, R T, R p, R rhob, const R* rhoUb, R rhoEb, R* Ub,
                              R& Tb, R& pb) {
    R rd = rcp(T * consts<R>(P).Rg);          // as conservative()
    conservative_vjp_t<R>(P, U, T, p, rd, rhob, rhoUb, rhoEb, Ub, Tb, pb);
}

// interp.secondOrder: phiC + (phiD - phiC) lw + qw.g
template <typename R>
AFVM_HD void recon_vjp(R b, R lw, const R* qw, R& phiCb, R& phiDb, R* gb) {
    phiCb += b * (R(1) - lw);
    phiDb += b * lw;
    for (int j = 0; j < 3; j++) gb[j] += b * qw[j];
}

// riemann.eulerRoe; the forward's reciprocals and reciprocal square roots come from the tape
template <typename R, typename Src, typename G = GeoNone>
AFVM_HD void roe_vjp(const Phys& P, R pL, R pR, R TL, R TR, const R* UL, const R* UR, R rhoL, R rhoR, const R* N,
                     const R* Fb, const Src& t, R& pLb, R& pRb, R& TLb, R& TRb, R* ULb, R* URb, R& rhoLb, R& rhoRb,
                     G* geo = nullptr) {
    const R gm1 = consts<R>(P).gm1, gRg = consts<R>(P).gRg, Cp = consts<R>(P).Cp, h = R(0.5);
    // ---- forward values: those dear to recompute from the tape, the cheap ones again (as roe());
    // a lean tape (Src::kFull false) holds only the reciprocals and the normal velocities, and
    // the Roe intermediates are re-evaluated here
    R UnL = t.get(T_UNL), UnR = t.get(T_UNR);
    R rsL = t.get(T_RSL), rsR = t.get(T_RSR);
    R rD = t.get(T_RD);
    R raF = t.get(T_RAF);
    R rcL = t.get(T_RCL), rcR = t.get(T_RCR);
    R re = t.get(T_RE);
    R rhoUnL, rhoUnR, wL, wR, cL, cR;
    if constexpr (Src::kFull) {
        rhoUnL = t.get(T_RUNL); rhoUnR = t.get(T_RUNR);
        wL = t.get(T_WL); wR = t.get(T_WR);
        cL = t.get(T_CL); cR = t.get(T_CR);
    } else {
        rhoUnL = rhoL * UnL; rhoUnR = rhoR * UnR;
        wL = (rhoL * rsL) * rD; wR = (rhoR * rsR) * rD;
        R c2L = gRg * TL, c2R = gRg * TR;
        cL = c2L > R(0) ? c2L * rcL : R(0); cR = c2R > R(0) ? c2R * rcR : R(0);
    }
    R eb_ = cL - cR;
    R ea = UnL - UnR;
    R drho = rhoR - rhoL;
    R hL, hR, UF[3], dU[3], hF, qF, UnF, drhoE, eps, L1, L2, L3, abv4, abv5, abv6, abv7;
    if constexpr (Src::kFull) {
        hL = t.get(T_HL);
        hR = t.get(T_HR);
        for (int k = 0; k < 3; k++) { UF[k] = t.get(T_UFR + k); dU[k] = t.get(T_DU + k); }
        hF = t.get(T_HF);
        qF = t.get(T_QF);
        UnF = t.get(T_UNF);
        drhoE = t.get(T_DRHOE);
        eps = t.get(T_EPS);
        L1 = t.get(T_L1); L2 = t.get(T_L2); L3 = t.get(T_L3);
        abv4 = t.get(T_ABV4); abv5 = t.get(T_ABV5); abv6 = t.get(T_ABV6); abv7 = t.get(T_ABV7);
    }
    if constexpr (!Src::kFull) {
        hL = Cp * TL + h * dot3(UL, UL);
        hR = Cp * TR + h * dot3(UR, UR);
        for (int k = 0; k < 3; k++) UF[k] = UL[k] * wL + UR[k] * wR;
        hF = hL * wL + hR * wR;
        qF = h * dot3(UF, UF);
        UnF = dot3(UF, N);
        for (int k = 0; k < 3; k++) dU[k] = rhoR * UR[k] - rhoL * UL[k];
        drhoE = (hR * rhoR - pR) - (hL * rhoL - pL);
        eps = h * (fabs(ea) + fabs(eb_)) + consts<R>(P).small;      // eps >= 0 (roe())
    }
    R aF, ra2F;
    if constexpr (Src::kFull) {
        aF = t.get(T_AF);
        ra2F = t.get(T_RA2F);
    } else {
        aF = (gm1 * (hF - qF)) * raF;
        ra2F = raF * raF;
    }
    R l1 = fabs(UnF), l2 = fabs(UnF + aF), l3 = fabs(UnF - aF);
    bool s1 = lt_twice(l1, eps), s2 = lt_twice(l2, eps), s3 = lt_twice(l3, eps);
    if constexpr (!Src::kFull) {
        L1 = s1 ? R(0.25) * l1 * l1 * re + eps : l1;
        L2 = s2 ? R(0.25) * l2 * l2 * re + eps : l2;
        L3 = s3 ? R(0.25) * l3 * l3 * re + eps : l3;
    }
    R abv2, abv3;
    if constexpr (Src::kFull) {
        abv2 = t.get(T_ABV2);
        abv3 = t.get(T_ABV3);
    } else {
        abv2 = h * (L2 - L3);
        abv3 = h * (L2 + L3) - L1;
    }
    if constexpr (!Src::kFull) {
        abv4 = gm1 * (qF * drho - dot3(UF, dU) + drhoE);
        abv5 = UnF * drho - dot3(dU, N);
        abv6 = abv3 * abv4 * ra2F - abv2 * abv5 * raF;
        abv7 = abv3 * abv5 - abv2 * abv4 * raF;
    }
    // ---- reverse (every flux component carries a factor 1/2: G = Fbar / 2)
    const R G0 = h * Fb[0], G4 = h * Fb[4];
    const R Gu[3] = {h * Fb[1], h * Fb[2], h * Fb[3]};
    R L1b = -(G0 * drho + dot3(Gu, dU) + G4 * drhoE);
    R drhob = -G0 * L1;
    R dUb[3], UFb[3];
    for (int k = 0; k < 3; k++) { dUb[k] = -Gu[k] * L1; UFb[k] = -Gu[k] * abv6; }
    R drhoEb = -G4 * L1;
    R abv6b = -(G0 + dot3(Gu, UF) + G4 * hF);
    R abv7b = dot3(Gu, N) + G4 * UnF;
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += Gu[k] * abv7;     // - (-abv7 N)/2 in F[1..3]
    R hFb = -G4 * abv6;
    R UnFb = G4 * abv7;
    // abv7 = abv3*abv5 - abv2*abv4/aF
    R b7r = abv7b * raF;
    R abv3b = abv7b * abv5, abv5b = abv7b * abv3, abv2b = -b7r * abv4, abv4b = -b7r * abv2;
    // abv6 = abv3*abv4/a2F - abv2*abv5/aF
    R b6q = abv6b * ra2F, b6r = abv6b * raF;
    abv3b += b6q * abv4;
    abv4b += b6q * abv3;
    R a2Fb = -(b6q * ra2F) * (abv3 * abv4);
    abv2b += -b6r * abv5;
    abv5b += -b6r * abv2;
    // both terms' d/daF (abv2 b7r abv4 + abv2 b6r abv5)/aF are -abv2 abv2b/aF
    R aFb = -(raF * abv2) * abv2b;
    // abv5 = UnF*drho - dU.N
    UnFb += abv5b * drho;
    drhob += abv5b * UnF;
    for (int k = 0; k < 3; k++) dUb[k] += -abv5b * N[k];
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += -abv5b * dU[k];
    // abv4 = gm1*(qF*drho - UF.dU + drhoE)
    R tb = gm1 * abv4b;
    R qFb = tb * drho;
    drhob += tb * qF;
    for (int k = 0; k < 3; k++) { UFb[k] += -tb * dU[k]; dUb[k] += -tb * UF[k]; }
    drhoEb += tb;
    // abv1..3
    R abv1b = abv3b;
    L1b += -abv3b;
    R L2b = h * (abv1b + abv2b), L3b = h * (abv1b - abv2b);
    // entropy fix L = l^2/(4 eps) + eps: dL/dl = t and dL/deps = 1 - t^2 with t = l/(2 eps). A
    // warp runs a branch when any of its faces takes it (most warps do for the first
    // eigenvalue), so the branches are kept short.
    R epsb = acc0<R>(), l1b, l2b, l3b;
    const R hre = h * re;
    if (s1) { R t = hre * l1; l1b = L1b * t; epsb += L1b * (R(1) - t * t); } else l1b = L1b;
    l2b = L2b;
    l3b = L3b;
    // the acoustic eigenvalues |U_F.n +- a_F| fall under 2 eps only near sonic faces: one branch
    // that warps skip, instead of two short ones that a warp would run with its lanes masked
    if (__builtin_expect(s2 || s3, 0)) {
        if (s2) { R t = hre * l2; l2b = L2b * t; epsb += L2b * (R(1) - t * t); }
        if (s3) { R t = hre * l3; l3b = L3b * t; epsb += L3b * (R(1) - t * t); }
    }
    R eab = mul_sgn(ea, h * epsb);
    R ebb = mul_sgn(eb_, h * epsb);
    // c = sqrt(g Rg T): dc/dT = g Rg / (2 c)
    TLb += ebb * consts<R>(P).hgRg * rcL;
    TRb += -ebb * consts<R>(P).hgRg * rcR;
    // lam = |UnF|, |UnF + aF|, |UnF - aF|
    R b2 = mul_sgn(UnF + aF, l2b), b3 = mul_sgn(UnF - aF, l3b);
    UnFb += mul_sgn(UnF, l1b) + b2 + b3;
    aFb += b2 - b3;
    // drhoE = (hR rhoR - pR) - (hL rhoL - pL)
    R hLb = -drhoEb * rhoL, hRb = drhoEb * rhoR;
    rhoRb += drhoEb * hR;
    rhoLb += -drhoEb * hL;
    pRb += -drhoEb;
    pLb += drhoEb;
    // dU = rhoR UR - rhoL UL ; drho = rhoR - rhoL
    rhoRb += dot3(dUb, UR) + drhob;
    rhoLb += -dot3(dUb, UL) - drhob;
    for (int k = 0; k < 3; k++) { URb[k] += dUb[k] * rhoR; ULb[k] += -dUb[k] * rhoL; }
    // UnF = UF.N ; aF = sqrt(a2F) ; a2F = gm1 (hF - qF) ; qF = |UF|^2/2
    for (int k = 0; k < 3; k++) UFb[k] += UnFb * N[k];
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += UnFb * UF[k];
    a2Fb += aFb * (h * raF);
    R g2 = gm1 * a2Fb;
    hFb += g2;
    qFb += -g2;
    for (int k = 0; k < 3; k++) UFb[k] += qFb * UF[k];
    // hF = hL wL + hR wR, UF = UL wL + UR wR with the weights wL = sL/(sL + sR), wR = sR/(sL + sR):
    // d/dsL of (xL sL + xR sR)/(sL + sR) = (xL - xR) wR/(sL + sR), d/dsR = -(xL - xR) wL/(sL + sR)
    hLb += hFb * wL;
    hRb += hFb * wR;
    for (int k = 0; k < 3; k++) {
        ULb[k] += UFb[k] * wL;
        URb[k] += UFb[k] * wR;
    }
    R X = hFb * (hL - hR) + (UFb[0] * (UL[0] - UR[0]) + UFb[1] * (UL[1] - UR[1]) + UFb[2] * (UL[2] - UR[2]));
    R Xr = X * rD;
    // sL = rho rsL: dsL/drho = 1/(2 sqrt(rho))
    rhoLb += (Xr * wR) * (h * rsL);
    rhoRb += -(Xr * wL) * (h * rsR);
    // fe = (rhoUnL hL + rhoUnR hR)/2 ; fu = (rhoUnL UL + rhoUnR UR + (pL+pR) N)/2 ; fr = (rhoUnL + rhoUnR)/2
    R rhoUnLb = G4 * hL + dot3(Gu, UL) + G0;
    R rhoUnRb = G4 * hR + dot3(Gu, UR) + G0;
    hLb += G4 * rhoUnL;
    hRb += G4 * rhoUnR;
    for (int k = 0; k < 3; k++) { ULb[k] += Gu[k] * rhoUnL; URb[k] += Gu[k] * rhoUnR; }
    R pn = dot3(Gu, N);
    pLb += pn;
    pRb += pn;
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += Gu[k] * (pL + pR);
    // hL = Cp TL + qL/2
    TLb += hLb * Cp;
    TRb += hRb * Cp;
    for (int k = 0; k < 3; k++) { ULb[k] += hLb * UL[k]; URb[k] += hRb * UR[k]; }
    // rhoUn = rho Un ; Un = U.N ; eps term ea = UnL - UnR
    rhoLb += rhoUnLb * UnL;
    rhoRb += rhoUnRb * UnR;
    R UnLb = rhoUnLb * rhoL + eab, UnRb = rhoUnRb * rhoR - eab;
    for (int k = 0; k < 3; k++) { ULb[k] += UnLb * N[k]; URb[k] += UnRb * N[k]; }
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += UnLb * UL[k] + UnRb * UR[k];
}

// riemann.eulerLaxFriedrichs
template <typename R, typename Src, typename G = GeoNone>
AFVM_HD void laxf_vjp(const Phys& P, R pL, R pR, R TL, R TR, const R* UL, const R* UR, R rhoL, R rhoR,
                      const R* rhoUL, const R* rhoUR, R rhoEL, R rhoER, const R* N, const R* Fb, const Src& t,
                      R& pLb, R& pRb, R& TLb, R& TRb, R* ULb, R* URb, R& rhoLb, R& rhoRb, R* rhoULb, R* rhoURb,
                      R& rhoELb, R& rhoERb, G* geo = nullptr) {
    const R gRg = consts<R>(P).gRg, h = R(0.5);
    R UnL = t.get(T_UNL), UnR = t.get(T_UNR);
    R rcL = t.get(T_RCL), rcR = t.get(T_RCR);
    R cL, cR;
    if constexpr (Src::kFull) {
        cL = t.get(T_CL); cR = t.get(T_CR);
    } else {
        R c2L = gRg * TL, c2R = gRg * TR;
        cL = c2L > R(0) ? c2L * rcL : R(0); cR = c2R > R(0) ? c2R * rcR : R(0);
    }
    R A = fabs(UnL) + cL, B = fabs(UnR) + cR;
    R aF = (A >= B) ? A : B;
    R ha = h * aF;
    R Fu[3] = {Fb[1], Fb[2], Fb[3]};
    R hab = -(Fb[0] * (rhoR - rhoL) + Fu[0] * (rhoUR[0] - rhoUL[0]) + Fu[1] * (rhoUR[1] - rhoUL[1]) +
              Fu[2] * (rhoUR[2] - rhoUL[2]) + Fb[4] * (rhoER - rhoEL));
    R aFb = h * hab;
    rhoLb += h * Fb[0] * UnL + ha * Fb[0];
    rhoRb += h * Fb[0] * UnR - ha * Fb[0];
    R UnLb = h * Fb[0] * rhoL + h * dot3(Fu, rhoUL) + h * Fb[4] * (rhoEL + pL);
    R UnRb = h * Fb[0] * rhoR + h * dot3(Fu, rhoUR) + h * Fb[4] * (rhoER + pR);
    for (int k = 0; k < 3; k++) {
        rhoULb[k] += h * Fu[k] * UnL + ha * Fu[k];
        rhoURb[k] += h * Fu[k] * UnR - ha * Fu[k];
    }
    R pn = h * dot3(Fu, N);
    pLb += pn + h * Fb[4] * UnL;
    pRb += pn + h * Fb[4] * UnR;
    rhoELb += h * Fb[4] * UnL + ha * Fb[4];
    rhoERb += h * Fb[4] * UnR - ha * Fb[4];
    R Ab = (A >= B) ? aFb : R(0), Bb = (A >= B) ? R(0) : aFb;
    UnLb += mul_sgn(UnL, Ab);
    UnRb += mul_sgn(UnR, Bb);
    TLb += Ab * consts<R>(P).hgRg * rcL;
    TRb += Bb * consts<R>(P).hgRg * rcR;
    for (int k = 0; k < 3; k++) { ULb[k] += UnLb * N[k]; URb[k] += UnRb * N[k]; }
    if constexpr (kGeo<G>)
        for (int k = 0; k < 3; k++) geo->N[k] += UnLb * UL[k] + UnRb * UR[k] + h * Fu[k] * (pL + pR);
}

// RCF.viscousFlux: F[1..3] += -sigma, F[4] += -(q + sigma.UF)
// (mu = mu(TF), gT and gU the corrected face gradients: the forward's values). The face
// velocity is passed as UFs with UF = us UFs (us = 1/2: UFs is the two sides' sum; 1: the
// ghost's own), and UFb receives the adjoint of each side's velocity, us times UF's. Likewise
// gTFb and gUFb receive the adjoints of the cell gradients the face gradient is formed from:
// gs times those of the face gradient (gs = 1/2 where it is the two sides' average - avg true -
// and 1 where it is the ghost's own). So each side's share needs no further product.
template <typename R>
AFVM_HD void viscous_vjp_t(const Phys& P, const R* UFs, R us, R mu, R dmu, R gTn, const R* tmp2, R tmp3, R ts,
                           const R* sigma, const R* D, const R* N, const R* Nt, R ND, R rdel, R gs, bool avg,
                           const R* Fb, R& TLb, R& TRb, R* ULb, R* URb, R& TFb, R* UFb, R* gTFb, R* gUFb) {
    R kappa = mu * consts<R>(P).kFac;
    // reverse
    R sb[3];
    R f4 = Fb[4] * us;
    for (int i = 0; i < 3; i++) {
        sb[i] = -Fb[1 + i] - f4 * UFs[i];
        UFb[i] += -f4 * sigma[i];
    }
    R qFb = -Fb[4];
    R mub = acc0<R>();
    R tmp2b[3];
    // (tmp2, tmp3: the forward's, divided by ts); the gradient adjoints below carry the factor gs
    R c23 = R(2.0 / 3) * tmp3;
    R mug = mu * gs;
    for (int i = 0; i < 3; i++) {
        mub += sb[i] * (tmp2[i] - c23 * N[i]);
        tmp2b[i] = sb[i] * mug;
    }
    mub = mub * ts;
    R tmp3b = (-R(2.0 / 3) * mug) * dot3(sb, N);
    R kappab = qFb * gTn;
    R qk = (qFb * kappa) * gs;
    mub += kappab * consts<R>(P).kFac;
    // gUb[i][k] = tmp2b_i N_k + tmp2b_k N_i (+ tmp3b on the diagonal) is symmetric: each
    // off-diagonal pair is formed once
    R gUb[9];
    for (int i = 0; i < 3; i++) gUb[4 * i] = (R(2) * tmp2b[i]) * N[i] + tmp3b;
    gUb[1] = gUb[3] = tmp2b[0] * N[1] + tmp2b[1] * N[0];
    gUb[2] = gUb[6] = tmp2b[0] * N[2] + tmp2b[2] * N[0];
    gUb[5] = gUb[7] = tmp2b[1] * N[2] + tmp2b[2] * N[1];
    // snGrad = (phi_N - phi_P) / deltas: the cell values' share, less the factor gs
    R rdg = avg ? twice_pos(rdel) : rdel;
    for (int i = 0; i < 3; i++) {
        R snUb = gUb[3 * i] * D[0] + gUb[3 * i + 1] * D[1] + gUb[3 * i + 2] * D[2];
        for (int k = 0; k < 3; k++) gUFb[3 * i + k] += gUb[3 * i + k] - snUb * D[k];
        URb[i] += snUb * rdg;
        ULb[i] += -snUb * rdg;
    }
    // the temperature gradient enters through its corrected normal component gTs.Nt + snGrad ND
    // (viscous())
    for (int k = 0; k < 3; k++) gTFb[k] += qk * Nt[k];
    R snTb = qk * ND;
    TRb += snTb * rdg;
    TLb += -snTb * rdg;
    // d mu/dT (viscosity(); 0 for a constant mu)
    TFb += mub * dmu;
}

template <typename R>
AFVM_HD void viscous_vjp(const Phys& P, R TL, R TR, const R* UL, const R* UR, R TF, const R* UF, const R* gTF,
                         const R* gUF, const R* D, const R* N, R rdel, const R* Fb, R& TLb, R& TRb, R* ULb, R* URb,
                         R& TFb, R* UFb, R* gTFb, R* gUFb) {
    R dmu;
    R mu = viscosity<R>(P, TF, &dmu);
    R gTD = dot3(gTF, D);
    R cT = (TR - TL) * rdel - gTD;
    R gT[3];
    for (int k = 0; k < 3; k++) gT[k] = gTF[k] + cT * D[k];
    R gU[9];
    for (int i = 0; i < 3; i++) {
        R gUD = gUF[3 * i] * D[0] + gUF[3 * i + 1] * D[1] + gUF[3 * i + 2] * D[2];
        R cU = (UR[i] - UL[i]) * rdel - gUD;
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUF[3 * i + k] + cU * D[k];
    }
    R tmp3 = gU[0] + gU[4] + gU[8];
    R tmp2[3], sigma[3];
    for (int i = 0; i < 3; i++) {
        tmp2[i] = (gU[3 * i] + gU[i]) * N[0] + (gU[3 * i + 1] + gU[3 + i]) * N[1] + (gU[3 * i + 2] + gU[6 + i]) * N[2];
        sigma[i] = mu * (tmp2[i] - R(2.0 / 3) * tmp3 * N[i]);
    }
    R ND = dot3(N, D), Nt[3];
    for (int k = 0; k < 3; k++) Nt[k] = N[k] - ND * D[k];
    viscous_vjp_t<R>(P, UF, R(1), mu, dmu, dot3(gT, N), tmp2, tmp3, R(1), sigma, D, N, Nt, ND, rdel, R(1), false, Fb,
                     TLb, TRb, ULb, URb, TFb, UFb, gTFb, gUFb);
}

// The geometry part of the viscous flux's VJP (deltasUnit D, normals N, 1/deltas): the forward
// is evaluated again from the face inputs, and only the geometry adjoints are accumulated (the
// state adjoints come from viscous_vjp / viscous_vjp_t)
template <typename R, typename G>
AFVM_HD void viscous_geo_vjp(const Phys& P, R TL, R TR, const R* UL, const R* UR, R TF, const R* UF, const R* gTF,
                             const R* gUF, const R* D, const R* N, R rdel, const R* Fb, G* geo) {
    R mu = viscosity<R>(P, TF);
    R kappa = mu * consts<R>(P).kFac;
    R snT = (TR - TL) * rdel;
    R gTD = dot3(gTF, D);
    R gT[3];
    for (int k = 0; k < 3; k++) gT[k] = gTF[k] + snT * D[k] - gTD * D[k];
    R snU[3], gUD[3], gU[9];
    for (int i = 0; i < 3; i++) {
        snU[i] = (UR[i] - UL[i]) * rdel;
        gUD[i] = gUF[3 * i] * D[0] + gUF[3 * i + 1] * D[1] + gUF[3 * i + 2] * D[2];
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUF[3 * i + k] + snU[i] * D[k] - gUD[i] * D[k];
    }
    R tmp3 = gU[0] + gU[4] + gU[8];
    // reverse: F[1+i] -= sigma_i, F[4] -= qF + sigma.UF
    R sb[3], tmp2b[3], tmp3b = R(0);
    R qFb = -Fb[4];
    for (int i = 0; i < 3; i++) {
        sb[i] = -Fb[1 + i] - Fb[4] * UF[i];
        tmp2b[i] = sb[i] * mu;
        tmp3b += -R(2.0 / 3) * mu * sb[i] * N[i];
    }
    // sigma_i = mu (tmp2_i - 2/3 tmp3 N_i) ; tmp2_i = sum_k (gU[i][k] + gU[k][i]) N_k ; qF = kappa gT.N
    for (int i = 0; i < 3; i++) geo->N[i] += sb[i] * (-R(2.0 / 3) * mu * tmp3);
    for (int k = 0; k < 3; k++) {
        R a = R(0);
        for (int i = 0; i < 3; i++) a += tmp2b[i] * (gU[3 * i + k] + gU[3 * k + i]);
        geo->N[k] += a + qFb * kappa * gT[k];
    }
    R gTb[3], gUb[9];
    for (int k = 0; k < 3; k++) gTb[k] = qFb * kappa * N[k];
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) gUb[3 * i + k] = tmp2b[i] * N[k] + tmp2b[k] * N[i];
    gUb[0] += tmp3b; gUb[4] += tmp3b; gUb[8] += tmp3b;
    // gT_k = gTF_k + snT D_k - (gTF.D) D_k, snT = (TR - TL)/deltas; the same per row of gU
    R snTb = dot3(gTb, D);
    for (int j = 0; j < 3; j++) geo->D[j] += gTb[j] * (snT - gTD) - gTF[j] * snTb;
    geo->rdelta += snTb * (TR - TL);
    for (int i = 0; i < 3; i++) {
        R snUb = gUb[3 * i] * D[0] + gUb[3 * i + 1] * D[1] + gUb[3 * i + 2] * D[2];
        for (int j = 0; j < 3; j++) geo->D[j] += gUb[3 * i + j] * (snU[i] - gUD[i]) - gUF[3 * i + j] * snUb;
        geo->rdelta += snUb * (UR[i] - UL[i]);
    }
}

template <typename R, typename Src, typename G = GeoNone>
AFVM_HD void face_vjp_t(const Phys& P, int kind, bool inviscid, const FaceIn<R>& in, const Src& t, const R* Fb,
                        FaceBar<R>& o, G* geo = nullptr);

// the corrected face gradient of U that viscous() forms (face-averaged cell gradients, or the
// ghost's on a characteristic face, with the normal component replaced by snGrad)
template <typename R>
AFVM_HD void corrected_gradU(const FaceIn<R>& in, bool chr, R* gU) {
    R gUF[9];
    for (int k = 0; k < 9; k++) gUF[k] = chr ? in.gUN[k] : R(0.5) * (in.gUP[k] + in.gUN[k]);
    for (int i = 0; i < 3; i++) {
        R gUD = gUF[3 * i] * in.D[0] + gUF[3 * i + 1] * in.D[1] + gUF[3 * i + 2] * in.D[2];
        R cU = (in.UN[i] - in.UP[i]) * in.rdelta - gUD;
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUF[3 * i + k] + cU * in.D[k];
    }
}

// <Fbar, F> differentiated with respect to all 40 inputs of the face (accumulated into out) and,
// given a GeoBar, with respect to the face geometry as well (accumulated into *geo)
template <typename R, typename G = GeoNone>
AFVM_HD void face_vjp(const Phys& P, int kind, bool inviscid, const FaceIn<R>& in, const R* Fb, FaceBar<R>& o,
                      G* geo = nullptr) {
    if (kind == FACE_BOUNDARY) {
        R rho, rhoU[3], rhoE;
        conservative<R>(P, in.UN, in.TN, in.pN, rho, rhoU, rhoE);
        R Un = dot3(in.UN, in.N);
        R rhob = Fb[0] * Un, rhoUb[3] = {Fb[1] * Un, Fb[2] * Un, Fb[3] * Un}, rhoEb = Fb[4] * Un;
        R Fu[3] = {Fb[1], Fb[2], Fb[3]};
        R Unb = Fb[0] * rho + dot3(Fu, rhoU) + Fb[4] * (rhoE + in.pN);
        o.pN += dot3(Fu, in.N) + Fb[4] * Un;
        for (int k = 0; k < 3; k++) o.UN[k] += Unb * in.N[k];
        if constexpr (kGeo<G>)
            for (int k = 0; k < 3; k++) geo->N[k] += Unb * in.UN[k] + Fu[k] * in.pN;
        conservative_vjp<R>(P, in.UN, in.TN, in.pN, rhob, rhoUb, rhoEb, o.UN, o.TN, o.pN);
        if (!inviscid) {
            R TFb = acc0<R>(), UFb[3] = {acc0<R>(), acc0<R>(), acc0<R>()};
            viscous_vjp<R>(P, in.TP, in.TN, in.UP, in.UN, in.TN, in.UN, in.gTN, in.gUN, in.D, in.N, in.rdelta, Fb,
                           o.TP, o.TN, o.UP, o.UN, TFb, UFb, o.gTN, o.gUN);
            o.TN += TFb;
            for (int k = 0; k < 3; k++) o.UN[k] += UFb[k];
            if constexpr (kGeo<G>)
                viscous_geo_vjp<R>(P, in.TP, in.TN, in.UP, in.UN, in.TN, in.UN, in.gTN, in.gUN, in.D, in.N,
                                   in.rdelta, Fb, geo);
        }
        return;
    }
    TapeLocal<R, sizeof(R) == 8> t;
    R F[5], maxaF;   // dead after inlining: only the tape values are used
    face_flux<R>(P, kind, inviscid, in, F, maxaF, t);
    face_vjp_t<R>(P, kind, inviscid, in, t, Fb, o, geo);
}

// the VJP of a non-boundary face from the tape of its forward evaluation: of the face inputs
// only the geometry (N, D, lw, qw, 1/deltas) is read from in - unless geometry adjoints are
// asked for (geo), which read every face input
template <typename R, typename Src, typename G>
AFVM_HD void face_vjp_t(const Phys& P, int kind, bool inviscid, const FaceIn<R>& in, const Src& t, const R* Fb,
                        FaceBar<R>& o, G* geo) {
    const bool chr = kind == FACE_CHARACTERISTIC;
    // forward values
    R ULF[3], TLF = t.get(T_TLF), pLF = t.get(T_PLF), URF[3], TRF = t.get(T_TRF), pRF = t.get(T_PRF);
    for (int k = 0; k < 3; k++) { ULF[k] = t.get(T_ULF + k); URF[k] = t.get(T_URF + k); }
    R rdL = t.get(T_RDL), rdR = t.get(T_RDR);
    R rhoL = pLF * rdL, rhoR = pRF * rdR;      // conservative(): rho = p * rd
    R ULFb[3] = {acc0<R>(), acc0<R>(), acc0<R>()}, URFb[3] = {acc0<R>(), acc0<R>(), acc0<R>()};
    R TLFb = acc0<R>(), TRFb = acc0<R>(), pLFb = acc0<R>(), pRFb = acc0<R>();
    // viscous part
    if (!inviscid) {
        // TF and the face velocity as us times UFs (the two sides' sum, or the ghost's own)
        R TF, UFs[3], us;
        if (chr) {
            TF = TRF;                            // the ghost's values (in.TN, in.UN)
            for (int k = 0; k < 3; k++) UFs[k] = URF[k];
            us = R(1);
        } else {
            TF = R(0.5) * (TLF + TRF);
            for (int k = 0; k < 3; k++) UFs[k] = ULF[k] + URF[k];
            us = R(0.5);
        }

        // gTFb, gUFb: each side's share of the face gradients' adjoints (viscous_vjp_t)
        R TFb = acc0<R>(), UFb[3] = {acc0<R>(), acc0<R>(), acc0<R>()}, gTFb[3], gUFb[9];
        for (int k = 0; k < 3; k++) gTFb[k] = acc0<R>();
        for (int k = 0; k < 9; k++) gUFb[k] = acc0<R>();
        R tmp2[3], sigma[3], tmp3, mu = t.get(T_MU), dmu, ts;
        if constexpr (Src::kFull) {
            // the taped stress terms are the forward's divided by its scale (viscous())
            for (int k = 0; k < 3; k++) { tmp2[k] = t.get(T_TMP2 + k); sigma[k] = t.get(T_SIG + k); }
            tmp3 = t.get(T_TMP3);
            dmu = t.get(T_DMU);
            ts = chr ? R(1) : R(0.5);
        } else {
            ts = R(1);
            viscosity<R>(P, TF, &dmu);
            // the stress terms from the corrected face gradient, as viscous() forms them
            R gUl[9];
            corrected_gradU<R>(in, chr, gUl);
            tmp3 = gUl[0] + gUl[4] + gUl[8];
            for (int i = 0; i < 3; i++) {
                tmp2[i] = (gUl[3 * i] + gUl[i]) * in.N[0] + (gUl[3 * i + 1] + gUl[3 + i]) * in.N[1] +
                          (gUl[3 * i + 2] + gUl[6 + i]) * in.N[2];
                sigma[i] = mu * (tmp2[i] - R(2.0 / 3) * tmp3 * in.N[i]);
            }
        }
        viscous_vjp_t<R>(P, UFs, us, mu, dmu, t.get(T_GTN), tmp2, tmp3, ts, sigma, in.D, in.N, in.Nt, in.ND,
                         in.rdelta, chr ? R(1) : R(0.5), !chr, Fb, o.TP, o.TN, o.UP, o.UN, TFb, UFb, gTFb,
                         gUFb);
        if constexpr (kGeo<G>) {
            R gTF[3], gUF[9];
            for (int k = 0; k < 3; k++) gTF[k] = chr ? in.gTN[k] : R(0.5) * (in.gTP[k] + in.gTN[k]);
            for (int k = 0; k < 9; k++) gUF[k] = chr ? in.gUN[k] : R(0.5) * (in.gUP[k] + in.gUN[k]);
            R UF[3];
            for (int k = 0; k < 3; k++) UF[k] = us * UFs[k];
            viscous_geo_vjp<R>(P, in.TP, in.TN, in.UP, in.UN, TF, UF, gTF, gUF, in.D, in.N, in.rdelta, Fb, geo);
        }
        if (chr) {
            o.TN += TFb;
            for (int k = 0; k < 3; k++) { o.UN[k] += UFb[k]; o.gTN[k] += gTFb[k]; }
            for (int k = 0; k < 9; k++) o.gUN[k] += gUFb[k];
        } else {
            TLFb += R(0.5) * TFb;
            TRFb += R(0.5) * TFb;
            for (int k = 0; k < 3; k++) {
                ULFb[k] += UFb[k];
                URFb[k] += UFb[k];
                o.gTP[k] += gTFb[k];
                o.gTN[k] += gTFb[k];
            }
            for (int k = 0; k < 9; k++) { o.gUP[k] += gUFb[k]; o.gUN[k] += gUFb[k]; }
        }
    }
    // Riemann part
    R rhoLb = acc0<R>(), rhoRb = acc0<R>(), rhoULb[3] = {acc0<R>(), acc0<R>(), acc0<R>()};
    R rhoURb[3] = {acc0<R>(), acc0<R>(), acc0<R>()};
    R rhoELb = acc0<R>(), rhoERb = acc0<R>();
    int solver = chr ? P.briemann : P.riemann;
    if (solver == AFVM_RIEMANN_ROE) {
        roe_vjp<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, in.N, Fb, t, pLFb, pRFb, TLFb, TRFb, ULFb, URFb,
                   rhoLb, rhoRb, geo);
        // conservative(): the Roe flux uses only rho = p rd of each side (rd = 1/(Rg T),
        // drho/dp = rd, drho/dT = -rho/T = -rho rd Rg)
        const R k = consts<R>(P).Rg;
        pLFb += rhoLb * rdL;
        TLFb += -rhoLb * (rhoL * (rdL * k));
        pRFb += rhoRb * rdR;
        TRFb += -rhoRb * (rhoR * (rdR * k));
    } else {
        // conservative()'s rhoU and rhoE of each side
        R eL = consts<R>(P).Cv * TLF, eR = consts<R>(P).Cv * TRF;
        R rhoEL = rhoL * (eL + R(0.5) * dot3(ULF, ULF)), rhoER = rhoR * (eR + R(0.5) * dot3(URF, URF));
        R rhoUL[3], rhoUR[3];
        for (int k = 0; k < 3; k++) { rhoUL[k] = ULF[k] * rhoL; rhoUR[k] = URF[k] * rhoR; }
        laxf_vjp<R>(P, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, rhoUL, rhoUR, rhoEL, rhoER, in.N, Fb, t, pLFb, pRFb,
                    TLFb, TRFb, ULFb, URFb, rhoLb, rhoRb, rhoULb, rhoURb, rhoELb, rhoERb, geo);
        conservative_vjp_t<R>(P, ULF, TLF, pLF, rdL, rhoLb, rhoULb, rhoELb, ULFb, TLFb, pLFb);
        conservative_vjp_t<R>(P, URF, TRF, pRF, rdR, rhoRb, rhoURb, rhoERb, URFb, TRFb, pRFb);
    }
    // reconstruction
    if constexpr (kGeo<G>) {
        // phiF = phiC + (phiD - phiC) lw + qw.grad phiC, per side
        for (int k = 0; k < 3; k++) {
            geo->lw0 += ULFb[k] * (in.UN[k] - in.UP[k]);
            for (int j = 0; j < 3; j++) geo->qw0[j] += ULFb[k] * in.gUP[3 * k + j];
        }
        geo->lw0 += TLFb * (in.TN - in.TP) + pLFb * (in.pN - in.pP);
        for (int j = 0; j < 3; j++) geo->qw0[j] += TLFb * in.gTP[j] + pLFb * in.gpP[j];
        if (!chr) {
            for (int k = 0; k < 3; k++) {
                geo->lw1 += URFb[k] * (in.UP[k] - in.UN[k]);
                for (int j = 0; j < 3; j++) geo->qw1[j] += URFb[k] * in.gUN[3 * k + j];
            }
            geo->lw1 += TRFb * (in.TP - in.TN) + pRFb * (in.pP - in.pN);
            for (int j = 0; j < 3; j++) geo->qw1[j] += TRFb * in.gTN[j] + pRFb * in.gpN[j];
        }
    }
    for (int k = 0; k < 3; k++) recon_vjp<R>(ULFb[k], in.lw0, in.qw0, o.UP[k], o.UN[k], o.gUP + 3 * k);
    recon_vjp<R>(TLFb, in.lw0, in.qw0, o.TP, o.TN, o.gTP);
    recon_vjp<R>(pLFb, in.lw0, in.qw0, o.pP, o.pN, o.gpP);
    if (chr) {
        for (int k = 0; k < 3; k++) o.UN[k] += URFb[k];
        o.TN += TRFb;
        o.pN += pRFb;
    } else {
        for (int k = 0; k < 3; k++) recon_vjp<R>(URFb[k], in.lw1, in.qw1, o.UN[k], o.UP[k], o.gUN + 3 * k);
        recon_vjp<R>(TRFb, in.lw1, in.qw1, o.TN, o.TP, o.gTN);
        recon_vjp<R>(pRFb, in.lw1, in.qw1, o.pN, o.pP, o.gpN);
    }
}

}  // namespace afvm
