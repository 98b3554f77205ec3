// Device-side physics of the compressible finite-volume residual.
//
// Each function states the reference expression it evaluates; operands are combined in the
// reference's order (left to right). FMA contraction is allowed, so results agree with the
// reference to rounding, not bit for bit.
#pragma once
#include <stdint.h>
#include <type_traits>
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

// The face tape: the values of the forward face flux that its VJP would otherwise recompute
// at the highest FP64 cost - the reconstructed face states, the reciprocals and reciprocal
// square roots, mu(T_F), the Roe and viscous intermediates. The forward flux writes them through
// a sink (nothing, a local array, or a column of a device tape); the VJP reads them back.
constexpr int T_ULF = 0, T_TLF = 3, T_PLF = 4, T_URF = 5, T_TRF = 8, T_PRF = 9;   // face states
constexpr int T_RDL = 10, T_RDR = 11;            // 1/(Rg T), Rg = Cv (g-1), of each side (conservative)
constexpr int T_UNL = 12, T_UNR = 13;            // U.n of each side
constexpr int T_RSL = 14, T_RSR = 15;            // 1/sqrt(rho)
constexpr int T_RD = 16, T_RAF = 17;             // 1/(sL + sR), 1/a_F (Roe average)
constexpr int T_RCL = 18, T_RCR = 19;            // 1/c of each side
constexpr int T_RE = 20;                         // 1/eps of the entropy fix (0 when inactive)
constexpr int T_MU = 21;                         // mu(T_F)
constexpr int T_GTN = 22;                        // (corrected face grad T).n
// Roe intermediates the reverse sweep uses (eulerRoe's names, riemann.py:21-70)
constexpr int T_HL = 23, T_HR = 24;              // total enthalpies
constexpr int T_UFR = 25, T_HF = 28, T_QF = 29;  // Roe-averaged U (3), H, |U|^2/2
constexpr int T_UNF = 30, T_DU = 31;             // U_F.n, the jump of rho U (3)
constexpr int T_DRHOE = 34, T_EPS = 35;          // the jump of rho E, the entropy-fix width
constexpr int T_L1 = 36, T_L2 = 37, T_L3 = 38;   // |eigenvalues| after the entropy fix
constexpr int T_ABV4 = 39, T_ABV5 = 40, T_ABV6 = 41, T_ABV7 = 42;
// viscous intermediates: (grad U + grad U^T).n (3), sigma (3), tr grad U (corrected face gradient)
constexpr int T_TMP2 = 43, T_SIG = 46, T_TMP3 = 49;
// more Roe forward values, so that the reverse sweep re-derives none: rho U.n and the Roe
// weight sqrt(rho)/(sqrt(rhoL) + sqrt(rhoR)) of each side, the sound speeds, the Roe-average
// sound speed and 1/a_F^2, and abv2, abv3
constexpr int T_RUNL = 50, T_RUNR = 51, T_WL = 52, T_WR = 53, T_CL = 54, T_CR = 55;
constexpr int T_AF = 56, T_RA2F = 57, T_ABV2 = 58, T_ABV3 = 59;
constexpr int T_DMU = 60;                        // d mu / d T at T_F
constexpr int TAPE = 61;
constexpr int T_LEAN = 23;   // the values up to here: those that cost the most to re-evaluate

struct TapeNone {
    template <typename R>
    AFVM_HD void put(int, R) const {}
};

// A sink/source in registers for the untaped VJP. FULL: all TAPE values (FP64: the VJP then
// re-evaluates nothing); otherwise the first T_LEAN and the VJP re-evaluates the Roe and
// viscous intermediates (FP32: fewer values live across the forward, faster)
template <typename R, bool FULL>
struct TapeLocal {
    static constexpr bool kFull = FULL;
    R v[FULL ? TAPE : T_LEAN];
    AFVM_HD void put(int k, R x) {
        if (FULL || k < T_LEAN) v[k] = x;
    }
    AFVM_HD R get(int k) const { return v[k]; }
};

// the gas constants in the working precision, so that the templated physics issues no FP64
// conversion or division in FP32 (ggm1 = gamma/(gamma-1), Rg = Cv (gamma-1) the gas constant,
// gRg = gamma Rg, rgm1 = 1/(gamma-1); hgRg = gRg/2, muTs15 = 3 Ts/2: products that would
// otherwise cost an instruction a face); gP, gT, gH, gK: the gauge state of FP32 records (below)
template <typename R>
struct PhysR {
    R gamma, gm1, ggm1, Cp, Cv, rCv, kFac, mu0, muAs, muTs, small;
    R Rg, gRg, rgm1, hgRg, muTs15;
    R gP, gT, gH, gK;
};

// FP32 cell records hold the pressure and temperature as offsets from a gauge state,
// p - gaugeP and T - gaugeT, and the FP32 face fluxes carry the momentum flux without
// gaugeP N and the energy flux less gaugeH times the mass flux. The update adds gaugeH times
// the mass residual and gaugeP times the cell's sum of A/V N back, and the gradient kernel
// gaugeT and gaugeP times that sum (it vanishes when a cell's face area vectors close, but
// the reference takes a face's normal from three of its points, so warped faces leave it
// nonzero). In a low-Mach flow the pressure (1e5 Pa) varies by ~1e2 Pa: a float holding p
// keeps four digits of those variations, a float holding p - gaugeP keeps all seven, and the
// face sums no longer round values 1e3 times larger than their result. FP64 records hold the
// absolute values (gauge unused).
struct Phys {
    double gamma, gm1, Cp, Cv, rCv, kFac, mu0, muAs, muTs, small;
    int muModel, riemann, briemann;
    double gaugeP = 0.0, gaugeT = 0.0, gaugeH = 0.0;
    PhysR<double> d;
    PhysR<float> f;
};

// the record types that hold gauge offsets
template <typename R>
constexpr bool kGauge = std::is_same<R, float>::value;

// a record's temperature / pressure as an absolute value: in double (objectives, adjoint
// viscosity) and in the record type (face VJP inputs, boundary transposes)
template <typename R>
AFVM_HD double rec_T(const Phys& P, R v) {
    if constexpr (kGauge<R>) return (double)v + P.gaugeT;
    else return (double)v;
}
template <typename R>
AFVM_HD double rec_p(const Phys& P, R v) {
    if constexpr (kGauge<R>) return (double)v + P.gaugeP;
    else return (double)v;
}

template <typename R>
inline void fill_consts(const Phys& P, PhysR<R>& q) {
    q.gamma = R(P.gamma); q.gm1 = R(P.gm1); q.ggm1 = R(P.gamma / P.gm1); q.Cp = R(P.Cp); q.Cv = R(P.Cv);
    q.rCv = R(P.rCv); q.kFac = R(P.kFac); q.mu0 = R(P.mu0); q.muAs = R(P.muAs); q.muTs = R(P.muTs);
    q.small = R(P.small);
    q.Rg = R(P.Cv * P.gm1); q.gRg = R(P.gamma * P.Cv * P.gm1); q.rgm1 = R(1.0 / P.gm1);
    q.hgRg = R(0.5 * P.gamma * P.Cv * P.gm1); q.muTs15 = R(1.5 * P.muTs);
    q.gP = R(P.gaugeP); q.gT = R(P.gaugeT); q.gH = R(P.gaugeH); q.gK = R(P.gaugeH - P.Cp * P.gaugeT);
}

// host: derive the working-precision copies once the double fields are set
inline void finish_phys(Phys& P) {
    fill_consts(P, P.d);
    fill_consts(P, P.f);
}

template <typename R>
AFVM_HD const PhysR<R>& consts(const Phys& P);
template <>
AFVM_HD const PhysR<double>& consts<double>(const Phys& P) { return P.d; }
template <>
AFVM_HD const PhysR<float>& consts<float>(const Phys& P) { return P.f; }

template <typename R>
AFVM_HD R rec_abs_T(const Phys& P, R v) {
    if constexpr (kGauge<R>) return v + consts<R>(P).gT;
    else return v;
}
template <typename R>
AFVM_HD R rec_abs_p(const Phys& P, R v) {
    if constexpr (kGauge<R>) return v + consts<R>(P).gP;
    else return v;
}

template <typename R>
AFVM_HD R dot3(const R* a, const R* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// y sign(x) with sign(0) = 0 (and 0 for a NaN x, as the comparisons give). On the device it is
// formed from the bits of x with integer operations: an FP64 compare issues on the FP64 pipe,
// the face kernels' bound.
template <typename R>
AFVM_HD R mul_sgn(R x, R y) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(R) == 8) {
        int hi = __double2hiint(x);
        unsigned lo = (unsigned)__double2loint(x);
        unsigned mag = (unsigned)hi & 0x7fffffffu;
        bool zero = (mag | lo) == 0u;
        bool nan = mag > 0x7ff00000u || (mag == 0x7ff00000u && lo != 0u);
        double r = __hiloint2double(__double2hiint(y) ^ (hi & (int)0x80000000), __double2loint(y));
        return (zero || nan) ? 0.0 : r;
    } else {
        unsigned b = __float_as_uint(x);
        unsigned mag = b & 0x7fffffffu;
        float r = __uint_as_float(__float_as_uint(y) ^ (b & 0x80000000u));
        return (mag == 0u || mag > 0x7f800000u) ? 0.0f : r;
    }
#else
    return (x > R(0)) ? y : ((x < R(0)) ? -y : R(0));
#endif
}

// a * b rounded on its own, never contracted into an FMA: sums of such products cancel exactly
// where their terms do (a uniform field's face fluxes in the cell gather)
AFVM_HD double mul_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
AFVM_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

// a < b for non-negative a, b: such floating-point numbers order like their bit patterns, so
// the device compares them as integers (no FP64 compare)
template <typename R>
AFVM_HD bool lt_nonneg(R a, R b) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(R) == 8) return __double_as_longlong(a) < __double_as_longlong(b);
    else return __float_as_int(a) < __float_as_int(b);
#else
    return a < b;
#endif
}

// a < 2 b for non-negative a and a positive normal b, as a/2 < b: on the device a's exponent
// field is lowered by one with an integer subtraction (exact for normal a; a zero or
// subnormal a turns negative and compares below b, as a/2 does), so no FP64 product is issued.
// An inf or NaN b compares above every finite a, as 2 b does.
template <typename R>
AFVM_HD bool lt_twice(R a, R b) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(R) == 8) return __double_as_longlong(a) - (1LL << 52) < __double_as_longlong(b);
    else return __float_as_int(a) - (1 << 23) < __float_as_int(b);
#else
    return a < R(2) * b;
#endif
}

// 2 x for a positive normal x below 2^1023 (2^127 in float): on the device the exponent field
// is raised by one with an integer add, exactly, and no FP64 product is issued
template <typename R>
AFVM_HD R twice_pos(R x) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(R) == 8) return __longlong_as_double(__double_as_longlong(x) + (1LL << 52));
    else return __int_as_float(__float_as_int(x) + (1 << 23));
#else
    return R(2) * x;
#endif
}

// ---- reciprocal and reciprocal square root
//
// On the GB300 the FP64 pipe runs at 1/57 of the FP32 rate, and an IEEE FP64 division or
// square root costs about nine FP64 instructions. In double these are built here from a
// 23-bit FP32 seed y (PTX rcp.approx / rsqrt.approx on the mantissa, the exponent handled with
// integer operations, so no FP64 conversion instruction is issued) and one third-order
// correction from the series of the exact answer in the seed's residual e (|e| < 2^-21):
//   1/x       = y / (1 - e)        = y (1 + e + e^2 + ...),          e = 1 - x y
//   1/sqrt(x) = y (1 - e)^(-1/2)   = y (1 + e/2 + 3 e^2/8 + ...),    e = 1 - x y^2
// The dropped terms are below 2^-63 relative. The seed has 24 significant bits, so x y is
// formed exactly inside the FMA and y^2 is exact in double; the last FMA rounds once: about
// half a unit in the last place, as the IEEE operations (3 FP64 instructions for 1/x and 5
// for 1/sqrt(x), against 4 and 8 for two Newton-Raphson steps). Arguments outside
// 2^[-120, 120] (and 0, inf, NaN) take the IEEE operation. In float the hardware
// approximations are used directly (about two units in the last place).
#if defined(__CUDACC__)
__device__ __forceinline__ double rcp_nr(double x) {
    int hi = __double2hiint(x);
    unsigned lo = (unsigned)__double2loint(x);
    int ex = (hi >> 20) & 0x7ff;
    if (ex < 1023 - 120 || ex > 1023 + 120) return 1.0 / x;
    unsigned mb = 0x3f800000u | (((unsigned)hi & 0xfffffu) << 3) | (lo >> 29);
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(mb)));
    unsigned rb = __float_as_uint(rf);
    long long dexp = (long long)((int)(rb >> 23) - ex + 1919);
    unsigned long long bits = ((unsigned long long)((unsigned)hi & 0x80000000u) << 32) |
                              ((unsigned long long)dexp << 52) | ((unsigned long long)(rb & 0x7fffffu) << 29);
    double y = __longlong_as_double((long long)bits);
    double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    int hi = __double2hiint(x);
    unsigned lo = (unsigned)__double2loint(x);
    int ex = (hi >> 20) & 0x7ff;
    if (hi < 0 || ex < 1023 - 120 || ex > 1023 + 120) return 1.0 / sqrt(x);
    int u = ex - 1023;
    int odd = u & 1;
    // mantissa as a float in [1,2) (u even) or [2,4) (u odd)
    unsigned mb = ((unsigned)(127 + odd) << 23) | (((unsigned)hi & 0xfffffu) << 3) | (lo >> 29);
    float rf;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(mb)));
    unsigned rb = __float_as_uint(rf);
    int half = (u - odd) / 2;                       // exact: u - odd is even
    long long dexp = (long long)((int)(rb >> 23) - 127 - half + 1023);
    unsigned long long bits = ((unsigned long long)dexp << 52) | ((unsigned long long)(rb & 0x7fffffu) << 29);
    double y = __longlong_as_double((long long)bits);
    double e = fma(-x, y * y, 1.0);
    return fma(y * e, fma(e, 0.375, 0.5), y);
}
#endif

AFVM_HD double rcp(double x) {
#if defined(__CUDA_ARCH__)
    return rcp_nr(x);
#else
    return 1.0 / x;
#endif
}

AFVM_HD float rcp(float x) {
#if defined(__CUDA_ARCH__)
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}

AFVM_HD double rsqrt_(double x) {
#if defined(__CUDA_ARCH__)
    return rsqrt_nr(x);
#else
    return 1.0 / sqrt(x);
#endif
}

AFVM_HD float rsqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrt(x);
#endif
}

// x > 0 from the bits (true for +inf and a positive NaN): no FP64 compare on the device
template <typename R>
AFVM_HD bool pos_(R x) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(R) == 8) return __double_as_longlong(x) > 0;
    else return __float_as_int(x) > 0;
#else
    return x > R(0);
#endif
}

// sqrt(x) for x >= 0 as x / sqrt(x) (0 for x <= 0)
template <typename R>
AFVM_HD R sqrt_(R x) { return pos_(x) ? x * rsqrt_(x) : R(0); }

// mu(T): constant, or Sutherland 1.4792e-06*T**1.5/(T+116.) (adFVM/density.py:27), written as
// As T^2 / sqrt(T (T + Ts)^2): one reciprocal square root (0 for T <= 0, as T sqrt(T) was).
// With dmu, also d mu / dT = mu (T/2 + 3 Ts/2) / (T (T + Ts)), where 1/(T (T + Ts)) is
// (T + Ts) y^2 with the same y = 1/sqrt(T (T + Ts)^2).
template <typename R>
AFVM_HD R viscosity(const Phys& P, R T, R* dmu = nullptr) {
    if (P.muModel == AFVM_MU_SUTHERLAND) {
        if (!pos_(T)) {
            if (dmu) *dmu = R(0);
            return R(0);
        }
        const R Ts = consts<R>(P).muTs;
        R a = T + Ts;
        R y = rsqrt_(T * (a * a));
        R mu = (consts<R>(P).muAs * (T * T)) * y;
        if (dmu) *dmu = (mu * (R(0.5) * T + consts<R>(P).muTs15)) * (a * (y * y));
        return mu;
    }
    if (dmu) *dmu = R(0);
    return consts<R>(P).mu0;
}

// RCF.conservative (adFVM/density.py:173-181)
template <typename R>
AFVM_HD void conservative(const Phys& P, const R* U, R T, R p, R& rho, R* rhoU, R& rhoE, R* rdOut = nullptr) {
    R e = consts<R>(P).Cv * T;
    R rd = rcp(T * consts<R>(P).Rg);        // 1/(e (g-1)); e itself only for rhoE
    if (rdOut) *rdOut = rd;
    rho = p * rd;
    rhoE = rho * (e + R(0.5) * dot3(U, U));
    rhoU[0] = U[0] * rho; rhoU[1] = U[1] * rho; rhoU[2] = U[2] * rho;
}

// interp.secondOrder for one side (adFVM/interp.py:20-28): phiC + (phiD-phiC)*lw + qw.grad,
// as one chain of FMAs, given dCD = phiD - phiC. A face's two sides share one difference: the
// neighbour side passes the owner side's negated, the same number as its own phiD - phiC.
template <typename R>
AFVM_HD R recon(R phiC, R dCD, const R* g, R lw, const R* qw) {
    R phiF = phiC + dCD * lw;
    return qw[2] * g[2] + (qw[1] * g[1] + (qw[0] * g[0] + phiF));
}

// riemann.eulerRoe (adFVM/riemann.py:21-70). Divisions become products with shared
// reciprocals; rhoUn/rho is Un (the same number in exact arithmetic). With rho = p / (Rg T)
// (conservative()), the enthalpy g p / ((g-1) rho) + |U|^2/2 is Cp T + |U|^2/2 and the sound
// speed sqrt(g p / rho) is sqrt(g Rg T): the same numbers in exact arithmetic, without 1/rho.
// Fv: the viscous terms (viscous()), subtracted from the momentum and energy fluxes.
template <typename R, typename Sink = TapeNone>
AFVM_HD void roe(const Phys& P, R pL, R pR, R TL, R TR, const R* UL, const R* UR, R rhoL, R rhoR,
                 const R* N, const R* Fv, R* F, Sink&& tp = Sink()) {
    const R gm1 = consts<R>(P).gm1, Cp = consts<R>(P).Cp;
    R UnL = dot3(UL, N), UnR = dot3(UR, N);
    tp.put(T_UNL, UnL);
    tp.put(T_UNR, UnR);
    R rhoUnL = rhoL * UnL, rhoUnR = rhoR * UnR;
    tp.put(T_RUNL, rhoUnL);
    tp.put(T_RUNR, rhoUnR);
    R hL = Cp * TL + R(0.5) * dot3(UL, UL);
    R hR = Cp * TR + R(0.5) * dot3(UR, UR);
    tp.put(T_HL, hL);
    tp.put(T_HR, hR);
    R UF[3], dU[3];
    R rsL = rsqrt_(rhoL), rsR = rsqrt_(rhoR);
    R sL = rhoL * rsL, sR = rhoR * rsR;
    R rD = rcp(sL + sR);
    // the Roe averages with the weights sL/(sL + sR), sR/(sL + sR) formed once
    R wL = sL * rD, wR = sR * rD;
    tp.put(T_RSL, rsL);
    tp.put(T_RSR, rsR);
    tp.put(T_WL, wL);
    tp.put(T_WR, wR);
    tp.put(T_RD, rD);
    for (int k = 0; k < 3; k++) UF[k] = UL[k] * wL + UR[k] * wR;
    R hF = hL * wL + hR * wR;
    R qF = R(0.5) * dot3(UF, UF);
    R a2F = gm1 * (hF - qF);
    R raF = rsqrt_(a2F);
    tp.put(T_RAF, raF);
    R aF = a2F * raF;
    R ra2F = raF * raF;
    tp.put(T_AF, aF);
    tp.put(T_RA2F, ra2F);
    R UnF = dot3(UF, N);
    R drho = rhoR - rhoL;
    for (int k = 0; k < 3; k++) dU[k] = rhoR * UR[k] - rhoL * UL[k];
    R drhoE = (hR * rhoR - pR) - (hL * rhoL - pL);
    for (int k = 0; k < 3; k++) { tp.put(T_UFR + k, UF[k]); tp.put(T_DU + k, dU[k]); }
    tp.put(T_HF, hF);
    tp.put(T_QF, qF);
    tp.put(T_UNF, UnF);
    tp.put(T_DRHOE, drhoE);
    R lam1 = fabs(UnF), lam2 = fabs(UnF + aF), lam3 = fabs(UnF - aF);
    // sound speeds c = sqrt(g Rg T) as c^2 / c with the reciprocal kept for the VJP
    R c2L = consts<R>(P).gRg * TL, c2R = consts<R>(P).gRg * TR;
    R rcL = rsqrt_(c2L), rcR = rsqrt_(c2R);
    tp.put(T_RCL, rcL);
    tp.put(T_RCR, rcR);
    R cL = pos_(c2L) ? c2L * rcL : R(0), cR = pos_(c2R) ? c2R * rcR : R(0);
    tp.put(T_CL, cL);
    tp.put(T_CR, cR);
    // the entropy-fix width; eps >= 0 (a sum of magnitudes), so the reference's
    // eps < 0 ? eps - small : eps + small is eps + small. 0.5 |a| + 0.5 |b| is taken as
    // 0.5 (|a| + |b|): halving is exact, so the bits are the same.
    R eps = R(0.5) * (fabs(UnL - UnR) + fabs(cL - cR)) + consts<R>(P).small;
    R re = R(0);
    bool s1 = lt_twice(lam1, eps), s2 = lt_twice(lam2, eps), s3 = lt_twice(lam3, eps);
    if (s1 || s2 || s3) {
        re = rcp(eps);
        if (s1) lam1 = R(0.25) * lam1 * lam1 * re + eps;
        // (the acoustic eigenvalues take the fix only near sonic faces: a branch warps skip)
        if (__builtin_expect(s2 || s3, 0)) {
            if (s2) lam2 = R(0.25) * lam2 * lam2 * re + eps;
            if (s3) lam3 = R(0.25) * lam3 * lam3 * re + eps;
        }
    }
    tp.put(T_RE, re);
    tp.put(T_EPS, eps);
    tp.put(T_L1, lam1);
    tp.put(T_L2, lam2);
    tp.put(T_L3, lam3);
    R abv1 = R(0.5) * (lam2 + lam3);
    R abv2 = R(0.5) * (lam2 - lam3);
    R abv3 = abv1 - lam1;
    R abv4 = gm1 * (qF * drho - dot3(UF, dU) + drhoE);
    R abv5 = UnF * drho - dot3(dU, N);
    R abv6 = abv3 * abv4 * ra2F - abv2 * abv5 * raF;
    R abv7 = abv3 * abv5 - abv2 * abv4 * raF;
    tp.put(T_ABV2, abv2);
    tp.put(T_ABV3, abv3);
    tp.put(T_ABV4, abv4);
    tp.put(T_ABV5, abv5);
    tp.put(T_ABV6, abv6);
    tp.put(T_ABV7, abv7);
    // central flux minus the dissipation, (F_L + F_R)/2 - |A| dq/2, with the common half taken
    // once: the pressure term's N and the dissipation's abv7 N share one product. The halving
    // is exact, so the viscous terms go in with it in one FMA, with the bits of a separate sum.
    F[0] = R(0.5) * ((rhoUnL + rhoUnR) - (lam1 * drho + abv6));
    const R pa = (pL + pR) + abv7;
    for (int k = 0; k < 3; k++)
        F[1 + k] = R(0.5) * (rhoUnL * UL[k] + rhoUnR * UR[k] + pa * N[k] - lam1 * dU[k] - UF[k] * abv6) - Fv[k];
    F[4] = R(0.5) * (rhoUnL * hL + rhoUnR * hR - lam1 * drhoE - hF * abv6 + UnF * abv7) - Fv[3];
}

// riemann.eulerLaxFriedrichs (adFVM/riemann.py:6-18)
template <typename R, typename Sink = TapeNone>
AFVM_HD void laxf(const Phys& P, R pL, R pR, R TL, R TR, const R* UL, const R* UR, R rhoL, R rhoR,
                  const R* rhoUL, const R* rhoUR, R rhoEL, R rhoER, const R* N, R* F, Sink&& tp = Sink()) {
    R UnL = dot3(UL, N), UnR = dot3(UR, N);
    // c = sqrt(g p / rho) = sqrt(g Rg T) (roe())
    R c2L = consts<R>(P).gRg * TL, c2R = consts<R>(P).gRg * TR;
    R rcL = rsqrt_(c2L), rcR = rsqrt_(c2R);
    tp.put(T_UNL, UnL);
    tp.put(T_UNR, UnR);
    tp.put(T_RCL, rcL);
    tp.put(T_RCR, rcR);
    R cL = pos_(c2L) ? c2L * rcL : R(0);
    R cR = pos_(c2R) ? c2R * rcR : R(0);
    tp.put(T_CL, cL);
    tp.put(T_CR, cR);
    R aF = fmax(fabs(UnL) + cL, fabs(UnR) + cR);
    R ha = R(0.5) * aF;
    F[0] = R(0.5) * (rhoL * UnL + rhoR * UnR) - ha * (rhoR - rhoL);
    for (int k = 0; k < 3; k++)
        F[1 + k] = R(0.5) * (rhoUL[k] * UnL + rhoUR[k] * UnR + (pL + pR) * N[k]) - ha * (rhoUR[k] - rhoUL[k]);
    F[4] = R(0.5) * ((rhoEL + pL) * UnL + (rhoER + pR) * UnR) - ha * (rhoER - rhoEL);
}

// ---- gauge forms of the Riemann fluxes (FP32 records; the gauge state is in PhysR)
//
// Inputs: the face states with pressure and temperature as gauge offsets (pg = p - gP,
// Tg = T - gT), the densities and 1/(Rg T) of conservative(). Output: eulerRoe's /
// eulerLaxFriedrichs's flux F with gP N taken out of F[1..3] and gH F[0] out of F[4]. The jumps
// of rho, rho U and rho E are formed from the gauge offsets and the velocity jump instead of as
// differences of the two sides' values (rho ~ 1 with 1e-3 variations, rho E ~ 2.5e5 with ~1e2):
//   rhoR - rhoL = (pR TL - pL TR) / (Rg TL TR),
//     pR TL - pL TR = (pgR - pgL) gT + pgR TgL - pgL TgR + gP (TgL - TgR)
//   rhoR UR - rhoL UL = rhoR (UR - UL) + (rhoR - rhoL) UL
//   rhoER - rhoEL = (pgR - pgL)/(g-1) + (rhoR (qR - qL) + (rhoR - rhoL) qL)/2,  q = |U|^2
// and the enthalpies as h - gH = Cp Tg + q/2 - gK (gK = gH - Cp gT). In exact arithmetic the
// flux is the reference's minus those two terms.
template <typename R>
struct GaugeJumps {
    R drho, dU[3], drhoE, drhoEg, hLg, hRg;
};

template <typename R>
AFVM_HD void gauge_jumps(const PhysR<R>& Q, R pgL, R pgR, R TgL, R TgR, const R* UL, const R* UR, R rhoL, R rhoR,
                         R rdL, R rdR, GaugeJumps<R>& j) {
    R num = (pgR - pgL) * Q.gT + (pgR * TgL - pgL * TgR) + Q.gP * (TgL - TgR);
    j.drho = num * ((rdL * rdR) * Q.Rg);
    R dUv[3];
    for (int k = 0; k < 3; k++) dUv[k] = UR[k] - UL[k];
    for (int k = 0; k < 3; k++) j.dU[k] = rhoR * dUv[k] + j.drho * UL[k];
    R qL = dot3(UL, UL), qR = dot3(UR, UR);
    R dq = dUv[0] * (UR[0] + UL[0]) + dUv[1] * (UR[1] + UL[1]) + dUv[2] * (UR[2] + UL[2]);
    j.drhoE = (pgR - pgL) * Q.rgm1 + R(0.5) * (rhoR * dq + j.drho * qL);
    j.drhoEg = j.drhoE - Q.gH * j.drho;
    j.hLg = Q.Cp * TgL + (R(0.5) * qL - Q.gK);
    j.hRg = Q.Cp * TgR + (R(0.5) * qR - Q.gK);
}

// riemann.eulerRoe (adFVM/riemann.py:21-70) in gauge form
template <typename R>
AFVM_HD void roe_gauge(const Phys& P, R pgL, R pgR, R TgL, R TgR, const R* UL, const R* UR, R rhoL, R rhoR, R rdL,
                       R rdR, const R* N, R* F) {
    const PhysR<R>& Q = consts<R>(P);
    const R gm1 = Q.gm1;
    GaugeJumps<R> j;
    gauge_jumps<R>(Q, pgL, pgR, TgL, TgR, UL, UR, rhoL, rhoR, rdL, rdR, j);
    R UnL = dot3(UL, N), UnR = dot3(UR, N);
    R rhoUnL = rhoL * UnL, rhoUnR = rhoR * UnR;
    R fr = R(0.5) * (rhoUnL + rhoUnR);
    R pgLR = pgL + pgR;
    R fu[3], UF[3];
    for (int k = 0; k < 3; k++) fu[k] = R(0.5) * (rhoUnL * UL[k] + rhoUnR * UR[k] + pgLR * N[k]);
    R fe = R(0.5) * (rhoUnL * j.hLg + rhoUnR * j.hRg);
    R rsL = rsqrt_(rhoL), rsR = rsqrt_(rhoR);
    R sL = rhoL * rsL, sR = rhoR * rsR;
    R rD = rcp(sL + sR);
    for (int k = 0; k < 3; k++) UF[k] = (UL[k] * sL + UR[k] * sR) * rD;
    R hFg = (j.hLg * sL + j.hRg * sR) * rD;
    R qF = R(0.5) * dot3(UF, UF);
    R a2F = gm1 * (Q.gH + (hFg - qF));
    R raF = rsqrt_(a2F);
    R aF = a2F * raF;
    R ra2F = raF * raF;
    R UnF = dot3(UF, N);
    R lam1 = fabs(UnF), lam2 = fabs(UnF + aF), lam3 = fabs(UnF - aF);
    // sound speeds sqrt(g p / rho) = sqrt(g Rg T)
    R c2L = Q.gRg * (TgL + Q.gT), c2R = Q.gRg * (TgR + Q.gT);
    R cL = sqrt_(c2L), cR = sqrt_(c2R);
    R eps = R(0.5) * (fabs(UnL - UnR) + fabs(cL - cR)) + Q.small;   // eps >= 0 (roe())
    bool s1 = lt_twice(lam1, eps), s2 = lt_twice(lam2, eps), s3 = lt_twice(lam3, eps);
    if (s1 || s2 || s3) {
        R re = rcp(eps);
        if (s1) lam1 = R(0.25) * lam1 * lam1 * re + eps;
        if (s2) lam2 = R(0.25) * lam2 * lam2 * re + eps;
        if (s3) lam3 = R(0.25) * lam3 * lam3 * re + eps;
    }
    R abv1 = R(0.5) * (lam2 + lam3);
    R abv2 = R(0.5) * (lam2 - lam3);
    R abv3 = abv1 - lam1;
    R abv4 = gm1 * (qF * j.drho - dot3(UF, j.dU) + j.drhoE);
    R abv5 = UnF * j.drho - dot3(j.dU, N);
    R abv6 = abv3 * abv4 * ra2F - abv2 * abv5 * raF;
    R abv7 = abv3 * abv5 - abv2 * abv4 * raF;
    F[0] = fr - R(0.5) * (lam1 * j.drho + abv6);
    for (int k = 0; k < 3; k++) F[1 + k] = fu[k] - R(0.5) * (lam1 * j.dU[k] + UF[k] * abv6 - abv7 * N[k]);
    F[4] = fe - R(0.5) * (lam1 * j.drhoEg + hFg * abv6 - UnF * abv7);
}

// riemann.eulerLaxFriedrichs (adFVM/riemann.py:6-18) in gauge form
template <typename R>
AFVM_HD void laxf_gauge(const Phys& P, R pgL, R pgR, R TgL, R TgR, const R* UL, const R* UR, R rhoL, R rhoR, R rdL,
                        R rdR, const R* N, R* F) {
    const PhysR<R>& Q = consts<R>(P);
    GaugeJumps<R> j;
    gauge_jumps<R>(Q, pgL, pgR, TgL, TgR, UL, UR, rhoL, rhoR, rdL, rdR, j);
    R UnL = dot3(UL, N), UnR = dot3(UR, N);
    R cL = sqrt_(Q.gRg * (TgL + Q.gT)), cR = sqrt_(Q.gRg * (TgR + Q.gT));
    R aF = fmax(fabs(UnL) + cL, fabs(UnR) + cR);
    R ha = R(0.5) * aF;
    R pgLR = pgL + pgR;
    F[0] = R(0.5) * (rhoL * UnL + rhoR * UnR) - ha * j.drho;
    for (int k = 0; k < 3; k++)
        F[1 + k] = R(0.5) * (rhoL * UL[k] * UnL + rhoR * UR[k] * UnR + pgLR * N[k]) - ha * j.dU[k];
    F[4] = R(0.5) * (rhoL * j.hLg * UnL + rhoR * j.hRg * UnR) - ha * j.drhoEg;
}

// RCF.viscousFlux (adFVM/density.py:192-222): the terms the flux subtracts, Fv[0..2] = sigma
// (from F[1..3]) and Fv[3] = q + sigma.UF (from F[4]);
// rdel = 1/deltas (a mesh table), the divisor of snGrad (op.py:66-67). The face velocity and
// gradients arrive as hs times Us, gTs, gUs: hs = 1/2 with the two sides' sums (sums true; the
// reference's averages), hs = 1 with the ghost's values. The corrected gradients are formed
// divided by hs, and so are the (grad U + grad U^T).n and tr grad U the tape keeps (the VJP
// scales them back); sigma, (grad T).n and the flux are the reference's. Nt = N - (N.D) D and
// ND = N.D: mesh-only factors of the corrected gradient's normal component.
template <typename R, typename Sink = TapeNone>
AFVM_HD void viscous(const Phys& P, R TL, R TR, const R* UL, const R* UR, R TF, const R* Us, const R* gTs,
                     const R* gUs, R hs, bool sums, const R* D, const R* N, const R* Nt, R ND, R rdel, R* Fv,
                     Sink&& tp = Sink()) {
    R dmu;
    R mu = viscosity<R>(P, TF, &dmu);
    tp.put(T_MU, mu);
    tp.put(T_DMU, dmu);
    R kappa = mu * consts<R>(P).kFac;
    // the face gradient with its normal component replaced by snGrad: g + (snGrad - g.D) D,
    // here divided by hs (1/deltas doubled on the integer pipe for the sums)
    R rdh = sums ? twice_pos(rdel) : rdel;
    R gU[9];
    for (int i = 0; i < 3; i++) {
        R gUD = gUs[3 * i] * D[0] + gUs[3 * i + 1] * D[1] + gUs[3 * i + 2] * D[2];
        R cU = (UR[i] - UL[i]) * rdh - gUD;
        for (int k = 0; k < 3; k++) gU[3 * i + k] = gUs[3 * i + k] + cU * D[k];
    }
    // of the corrected temperature gradient only its normal component enters: (gTs + cT D).N with
    // cT = (TR - TL) rdh - gTs.D is gTs.Nt + (TR - TL) rdh ND (Nt = N - (N.D) D, ND = N.D:
    // mesh-only tables)
    R gTn = hs * (dot3(gTs, Nt) + ((TR - TL) * rdh) * ND);
    tp.put(T_GTN, gTn);
    R qF = kappa * gTn;
    R tmp3 = gU[0] + gU[4] + gU[8];
    tp.put(T_TMP3, tmp3);
    R muh = mu * hs;
    R sigma[3];
    for (int i = 0; i < 3; i++) {
        R tmp2 = (gU[3 * i] + gU[i]) * N[0] + (gU[3 * i + 1] + gU[3 + i]) * N[1] + (gU[3 * i + 2] + gU[6 + i]) * N[2];
        sigma[i] = muh * (tmp2 - R(2.0 / 3) * tmp3 * N[i]);
        tp.put(T_TMP2 + i, tmp2);
        tp.put(T_SIG + i, sigma[i]);
    }
    Fv[0] = sigma[0];
    Fv[1] = sigma[1];
    Fv[2] = sigma[2];
    Fv[3] = qF + hs * dot3(sigma, Us);
}

}  // namespace afvm
