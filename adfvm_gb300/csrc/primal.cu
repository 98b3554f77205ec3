// Primal residual and SSP-RK3 step on the device (sm_103a).
//
// One stage of the reference's time step (adFVM/timestep.py:27-55 over RCF.equation,
// adFVM/density.py:339-414) is four kernels:
//   k_prim    cells + ghost cells: conservative -> primitive (density.py:162-171) and the
//             ghost-cell boundary conditions (BCs.py via Solver.boundary, solver.py:106-114)
//   k_grad    cells: Green-Gauss gradient, a gather over the 6 cellFaces (op.py:45-63)
//   k_flux    faces: reconstruction, Riemann flux, viscous flux, CFL term (density.py:253-331)
//   k_update  cells: gather of the face fluxes in the reference's collate order (no atomics),
//             the SSP-RK stage combination (timestep.py:35-45) and, at stage 1, the CFL max
// Data: one record of REC values per cell (primitives + gradients), one FREC record per
// face, mesh constants in SoA arrays; the conservative state keeps the reference layout
// (rho (n), rhoU (n x 3), rhoE (n)).
#include <cuda_runtime.h>
#include "ctx.cuh"
#include "facedev.cuh"
#include "vane.cuh"

namespace afvm {

// max(a, b) that keeps a NaN operand (fmax drops it)
__device__ __forceinline__ double nan_max(double a, double b) { return (b > a || b != b) ? b : a; }

// RCF.primitive (adFVM/density.py:162-171) in double. One out-of-line body, so that a ghost
// cell and its source cell get bit-identical values.
__device__ __noinline__ void primitive_d(const Phys& P, double rho, double r0, double r1, double r2, double rhoE,
                                         double* out) {
    double rr = rcp(rho);
    double U0 = r0 * rr, U1 = r1 * rr, U2 = r2 * rr;
    double E = rhoE * rr;
    double e = E - 0.5 * (U0 * U0 + U1 * U1 + U2 * U2);
    out[0] = U0; out[1] = U1; out[2] = U2;
    out[4] = (P.gm1 * rho) * e;
    out[3] = e * P.rCv;
}

// FP32 state: velocity and temperature in float; the internal energy rho*e = rhoE - |rhoU|^2/(2 rho)
// (the low-Mach cancellation) and the pressure recovered in double from the float state.
__device__ __noinline__ void primitive_f(const Phys& P, float rho, float r0, float r1, float r2, float rhoE,
                                         float* out) {
    float rr = rcp(rho);
    out[0] = r0 * rr; out[1] = r1 * rr; out[2] = r2 * rr;
    double q = (double)r0 * r0 + (double)r1 * r1 + (double)r2 * r2;
    double rhoe = (double)rhoE - 0.5 * q * (double)rr;
    out[4] = (float)(P.gm1 * rhoe - P.gaugeP);
    out[3] = (float)(rhoe * (double)rr * P.rCv - P.gaugeT);
}

// primitives of one state (element type S) into the record type R
__device__ __forceinline__ void prim_values(const Phys& P, double r, double u0, double u1, double u2, double e,
                                            double* out) {
    primitive_d(P, r, u0, u1, u2, e, out);
}
__device__ __forceinline__ void prim_values(const Phys& P, float r, float u0, float u1, float u2, float e,
                                            float* out) {
    primitive_f(P, r, u0, u1, u2, e, out);
}
// FP64 state, FP32 record: the primitives in double, the gauge offsets of T and p taken in
// double, then rounded once
__device__ __forceinline__ void prim_values(const Phys& P, double r, double u0, double u1, double u2, double e,
                                            float* out) {
    double v[5];
    primitive_d(P, r, u0, u1, u2, e, v);
    v[3] -= P.gaugeT;
    v[4] -= P.gaugeP;
    for (int k = 0; k < 5; k++) out[k] = (float)v[k];
}

// primitives of cell c from the state arrays
template <typename R, typename S>
__device__ __forceinline__ void load_prim(const Phys& P, const S* rho, const S* rhoU, const S* rhoE, int c, R* out) {
    prim_values(P, rho[c], rhoU[3 * c], rhoU[3 * c + 1], rhoU[3 * c + 2], rhoE[c], out);
}

// the five primitives at the head of a 16-byte aligned record: a 16-byte store and a scalar
// (two L2 write requests a cell instead of five)
__device__ __forceinline__ void store_prims(float* r, const float* v) {
    *reinterpret_cast<float4*>(r) = make_float4(v[0], v[1], v[2], v[3]);
    r[4] = v[4];
}
__device__ __forceinline__ void store_prims(double* r, const double* v) {
    *reinterpret_cast<double2*>(r) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(r + 2) = make_double2(v[2], v[3]);
    r[4] = v[4];
}

// one cell's term of a cell-sum objective on its primitives U (3), T, p (record values: FP32
// ones hold gauge offsets): AFVM_OBJ_KINETIC_ENERGY 0.5 rho |U|^2 V in the record type, or
// AFVM_OBJ_SUM_T the temperature; accumulated in double
template <typename R>
__device__ __forceinline__ double cell_objective(const Phys& P, int kind, const R* r, R vol) {
    if (kind == AFVM_OBJ_KINETIC_ENERGY) {
        R rho = rec_abs_p<R>(P, r[R_P]) * rcp((consts<R>(P).Cv * rec_abs_T<R>(P, r[R_T])) * consts<R>(P).gm1);
        return (double)(R(0.5) * rho * (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) * vol);
    }
    return rec_T<R>(P, r[R_T]);
}

// the objectives that are sums over cells (evaluated in the stage-0 update, which writes the
// objective stage's primitives)
inline bool cell_sum_objective(int kind) { return kind == AFVM_OBJ_KINETIC_ENERGY || kind == AFVM_OBJ_SUM_T; }

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (threadIdx.x < BLOCK / 32) ? sh[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1) r += __shfl_down_sync(0xffffffffu, r, off);
    }
    return r;
}

// ghost cell g's primitives from its source cell's (v, replaced in place): the boundary
// conditions of BCs.py:62-184 (FP32 records: T and p as gauge offsets, so a zero-gradient
// ghost keeps its source's bits)
template <typename R>
__device__ __forceinline__ void ghost_prims(const MeshDev<R>& m, const Phys& P, int g, R* v) {
    int kind = m.gkind[g];
    int kU = kind & 7, kT = (kind >> 3) & 7, kp = (kind >> 6) & 7;
    const R gT = kGauge<R> ? consts<R>(P).gT : R(0), gP = kGauge<R> ? consts<R>(P).gP : R(0);
    if (kU == GK_TOTALPT) {
        // CBC_TOTAL_PT (BCs.py:178-184): Un = U.d, Ub = Un d, Tb = Tt - Un^2/(2 Cp),
        // pb = pt (T/Tt)^(gamma/(gamma-1)) with U, T of the owner cell
        R d[3] = {m.gval[g], m.gval[(size_t)m.nG + g], m.gval[2 * (size_t)m.nG + g]};
        R Tt = m.gval[3 * (size_t)m.nG + g], pt = m.gval[4 * (size_t)m.nG + g];
        R Un = dot3(v, d);
        R T = kGauge<R> ? v[3] + gT : v[3];
        for (int k = 0; k < 3; k++) v[k] = Un * d[k];
        v[3] = Tt - R(0.5) * Un * Un / consts<R>(P).Cp;
        v[4] = pt * pow(T / Tt, consts<R>(P).ggm1);
        if constexpr (kGauge<R>) {
            v[3] = v[3] - gT;
            v[4] = v[4] - gP;
        }
        return;
    }
    if (kU == GK_FIXED) {
        for (int k = 0; k < 3; k++) v[k] = m.gval[(size_t)k * m.nG + g];
    } else if (kU == GK_SYM) {
        int f = m.nIF + g;
        R n[3] = {m.nrm[f], m.nrm[(size_t)m.nF + f], m.nrm[2 * (size_t)m.nF + f]};
        R un = dot3(v, n);
        for (int k = 0; k < 3; k++) v[k] = v[k] - un * n[k];
    }
    if (kT == GK_FIXED) v[3] = kGauge<R> ? m.gval[3 * (size_t)m.nG + g] - gT : m.gval[3 * (size_t)m.nG + g];
    if (kp == GK_FIXED) v[4] = kGauge<R> ? m.gval[4 * (size_t)m.nG + g] - gP : m.gval[4 * (size_t)m.nG + g];
}

template <typename R, typename S>
__global__ void __launch_bounds__(BLOCK) k_prim(MeshDev<R> m, Phys P, const S* __restrict__ rho,
                                                const S* __restrict__ rhoU, const S* __restrict__ rhoE,
                                                R* __restrict__ rec) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m.nIC) {
        R v[5];
        load_prim<R, S>(P, rho, rhoU, rhoE, t, v);
        store_prims(rec + (size_t)t * REC, v);
        return;
    }
    int g = t - m.nIC;
    if (g >= m.nG) return;
    R v[5];
    load_prim<R, S>(P, rho, rhoU, rhoE, m.gsrc[g], v);
    ghost_prims<R>(m, P, g, v);
    store_prims(rec + (size_t)t * REC, v);
}

template <typename R>
__device__ __forceinline__ void grad_cell(const MeshDev<R>& m, const Phys& P, const R* __restrict__ rec, int c,
                                          R* row) {
    // the five primitives of a record as one 16-byte load and a scalar (records are 16-byte
    // aligned)
    R phic[5];
    load_vec(rec + (size_t)c * REC, phic, 4);
    phic[4] = rec[(size_t)c * REC + 4];
    // sum_s phiF_s S N'_s / V with phiF_s = phi_c (1 - w'_s) + phi_nb w'_s, regrouped as
    // phi_c sum_s (1 - w'_s) S N'_s / V + sum_s phi_nb (w'_s S N'_s / V): the mesh-only products
    // are tables, leaving 15 FMAs a slot (the face interpolation and the 1/V scaling were 25)
    const size_t n = m.nIC;
    R g[15];
    {
        R a[3] = {m.gAv[c], m.gAv[n + c], m.gAv[2 * n + c]};
        for (int i = 0; i < 5; i++)
            for (int j = 0; j < 3; j++) g[3 * i + j] = phic[i] * a[j];
    }
#pragma unroll
    for (int s = 0; s < 6; s++) {
        int nb = m.gnb[s * n + c];
        R ws[3] = {m.gws[(3 * s) * n + c], m.gws[(3 * s + 1) * n + c], m.gws[(3 * s + 2) * n + c]};
        R rn[5];
        load_vec(rec + (size_t)nb * REC, rn, 4);
        rn[4] = rec[(size_t)nb * REC + 4];
        for (int i = 0; i < 5; i++)
            for (int j = 0; j < 3; j++) g[3 * i + j] = g[3 * i + j] + rn[i] * ws[j];
    }
    if constexpr (kGauge<R>) {
        // FP32 records hold T - gT, p - gP: the gradient of the constant offsets is the offset
        // times the cell's sum of S N'/V, which warped faces leave nonzero
        R cl[3] = {m.gcl[c], m.gcl[n + c], m.gcl[2 * n + c]};
        for (int j = 0; j < 3; j++) {
            g[9 + j] = g[9 + j] + consts<R>(P).gT * cl[j];
            g[12 + j] = g[12 + j] + consts<R>(P).gP * cl[j];
        }
    }
    R v[REC];
    for (int k = 0; k < 5; k++) v[k] = phic[k];
    for (int k = 0; k < 15; k++) v[R_GU + k] = g[k];
    stage_row<R, REC>(row, v);
}

// the cell's whole record (its primitives again, then the gradients) is staged and the block's
// records written contiguously. Other blocks read the primitives of these records while they
// are rewritten: the rewrite stores the bits already there (each cell's primitives are read
// from its own record and written back unchanged), so every read sees the same value whether
// it lands before or after the store.
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_grad(MeshDev<R> m, Phys P, R* __restrict__ rec) {
    __shared__ __align__(16) R stage[BLOCK * REC];
    const int c0 = blockIdx.x * BLOCK;
    const int c = c0 + threadIdx.x;
    if (c < m.nIC) grad_cell<R>(m, P, rec, c, stage + threadIdx.x * REC);
    __syncthreads();
    if (c0 < m.nIC) store_staged<R, REC, BLOCK>(rec, c0, min(BLOCK, m.nIC - c0), stage);
}


// TAPED: also writes the face tape (TAPE values a face, column-major: tape[k nF + f]) that
// k_adj_flux<..., true> reads back instead of re-evaluating the forward flux
// CFL: the stage whose CFL sum is taken (the second, density.py:405-413); the other stages
// store 0 in the CFL slot and skip its square root
template <typename R, bool TAPED, bool CFL>
__global__ void __launch_bounds__(FLUX_BLOCK, sizeof(R) == 8 ? 3 : 8) k_flux(MeshDev<R> m, Phys P, const R* __restrict__ rec,
                                                R* __restrict__ fflux, int inviscid, R* __restrict__ tape) {
    // (the 6-value face records are stored directly: staging them through shared memory, as
    // the 20- and 40-value records are, made this kernel slower - 0.217 -> 0.269 ms at 128^3 in
    // FP32 - the barrier costs more than the six partly coalesced stores)
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nF) return;
    int kind = (f < m.nIF) ? FACE_INTERNAL : (int)m.fkind[f - m.nIF];
    FaceIn<R> in;
    load_face<R>(m, rec, f, in);
    R F[5], maxaF;
    // (FP32 records hold gauge offsets and their fluxes are the gauge form; only FP64
    // contexts keep face tapes)
    if constexpr (TAPED && !kGauge<R>)
        face_flux<R>(P, kind, inviscid != 0, in, F, maxaF, TapeStore<R>{tape + f, (size_t)m.nF});
    else
        face_flux<R, kGauge<R>>(P, kind, inviscid != 0, in, F, maxaF);
    R* out = fflux + (size_t)f * FREC;
    for (int k = 0; k < 5; k++) out[k] = F[k];
    out[5] = CFL ? maxaF : R(0);
}

// a 6-value face flux record in three 8- (FP32) or 16-byte (FP64) loads; records start on
// multiples of 24 / 48 bytes
__device__ __forceinline__ void load_flux_record(const float* __restrict__ p, float* o) {
#pragma unroll
    for (int i = 0; i < FREC; i += 2) {
        float2 v = __ldg(reinterpret_cast<const float2*>(p + i));
        o[i] = v.x; o[i + 1] = v.y;
    }
}
__device__ __forceinline__ void load_flux_record(const double* __restrict__ p, double* o) {
#pragma unroll
    for (int i = 0; i < FREC; i += 2) {
        double2 v = __ldg(reinterpret_cast<const double2*>(p + i));
        o[i] = v.x; o[i + 1] = v.y;
    }
}

// Gather of the face fluxes (op.div / op.absDiv, op.py:12-29, collated in the order of
// density.py:390-402) and the SSP-RK3 stage update (timestep.py:35-45).
template <typename R, typename S, int STAGE>
__global__ void __launch_bounds__(BLOCK) k_update(MeshDev<R> m, const R* __restrict__ fflux, double dtv,
                                                  const double* dtp,
                                                  const S* u0r, const S* u0u, const S* u0e,
                                                  const S* u1r, const S* u1u, const S* u1e,
                                                  const S* u2r, const S* u2u, const S* u2e,
                                                  const S* __restrict__ Sr, const S* __restrict__ Su,
                                                  const S* __restrict__ Se,
                                                  S* outr, S* outu, S* oute,
                                                  unsigned long long* dtcBits, Phys P, R* __restrict__ recNext,
                                                  int objKind, double* __restrict__ objPartials) {
    // the gather (and the CFL sum) in the flux type R, the stage update in the state's type S:
    // under FP32 fluxes with an FP64 state the six fluxes are summed in FP32 (each carries FP32
    // rounding already; summing them in FP64 cost six FP64 conversions, products and sums a
    // cell and component) and the state is updated in FP64
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    R dtc = R(0);
    double objv = 0.0;     // this cell's term of a cell-sum objective (stage 0, objPartials)
    if (c < m.nIC) {
        const size_t n = m.nIC;
        // the sums start at -0, which the compiler drops from the first term's add (-0 + x is x,
        // while +0 + x is one more add; the values differ at most in the sign of a zero)
        R res[5] = {R(-0.0), R(-0.0), R(-0.0), R(-0.0), R(-0.0)};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            int e = m.accf[k * n + c];
            R w = m.accw[k * n + c];
            bool ownerSide = e >= 0;
            int f = ownerSide ? e : ~e;
            R F[FREC];
            load_flux_record(fflux + (size_t)f * FREC, F);
            // the side's sign on the weight (one select a face, not one a term); each product
            // rounded before it is added, as the reference's collate sum does, so that equal
            // and opposite terms cancel exactly
            R ws = ownerSide ? w : -w;
            for (int q = 0; q < 5; q++) res[q] = res[q] + mul_rn(F[q], ws);
            dtc = dtc + F[5] * w;
        }
        S rs[5];
        for (int q = 0; q < 5; q++) rs[q] = S(res[q]);
        // gauge-form fluxes (FP32): the energy residual is the gathered one plus gaugeH times
        // the mass residual, the momentum residual the gathered one plus gaugeP times the
        // cell's sum of A/V N (the gaugeP N the face fluxes leave out; zero when the cell's
        // face area vectors close), both added in the state's type
        if constexpr (kGauge<R>) {
            rs[4] = rs[4] + S(P.gaugeH) * rs[0];
            // (a float state reads the float copy of the closure sums: half the bytes)
            for (int k = 0; k < 3; k++)
                rs[1 + k] = rs[1 + k] + S(P.gaugeP) * (sizeof(S) == 4 ? S(m.gcl[k * n + c]) : S(m.gclD[k * n + c]));
        }
        S Sv[5] = {Sr[c], Su[3 * c], Su[3 * c + 1], Su[3 * c + 2], Se[c]};
        S a[5] = {u0r[c], u0u[3 * c], u0u[3 * c + 1], u0u[3 * c + 2], u0e[c]};
        S o[5];
        const S rdt = S(dtp ? *dtp : dtv);
        // u = sum_j alpha_j u_j - beta dt (R - S) with -beta dt formed once a cell
        if (STAGE == 0) {
            const S k = -rdt;
            for (int q = 0; q < 5; q++) o[q] = a[q] + k * (rs[q] - Sv[q]);
        } else if (STAGE == 1) {
            S b[5] = {u1r[c], u1u[3 * c], u1u[3 * c + 1], u1u[3 * c + 2], u1e[c]};
            const S k = S(-(1. / 4)) * rdt;
            for (int q = 0; q < 5; q++) o[q] = (S(3. / 4) * a[q] + S(1. / 4) * b[q]) + k * (rs[q] - Sv[q]);
        } else {
            S b[5] = {u2r[c], u2u[3 * c], u2u[3 * c + 1], u2u[3 * c + 2], u2e[c]};
            const S k = S(-(2. / 3)) * rdt;
            for (int q = 0; q < 5; q++) o[q] = (S(1. / 3) * a[q] + S(2. / 3) * b[q]) + k * (rs[q] - Sv[q]);
        }
        outr[c] = o[0];
        outu[3 * c] = o[1]; outu[3 * c + 1] = o[2]; outu[3 * c + 2] = o[3];
        oute[c] = o[4];
        if (recNext) {
            // the next stage's k_prim, fused: this cell's primitives and those of the ghost
            // cells whose source it is, from the values just stored (the same bits k_prim
            // would read back)
            R v[5];
            prim_values(P, o[0], o[1], o[2], o[3], o[4], v);
            store_prims(recNext + (size_t)c * REC, v);
            if (STAGE == 0 && objPartials) objv = cell_objective<R>(P, objKind, v, m.vol[c]);
            for (int q = m.gsStart[c]; q < m.gsStart[c + 1]; q++) {
                int g = m.gsList[q];
                R w[5] = {v[0], v[1], v[2], v[3], v[4]};
                ghost_prims<R>(m, P, g, w);
                store_prims(recNext + (size_t)(m.nIC + g) * REC, w);
            }
        }
    }
    if (STAGE == 0 && objPartials) {
        // the objective stage's primitives are the ones this stage-0 update writes: the
        // objective's block partial sums (the same terms and order as k_objective)
        __shared__ double osh[BLOCK / 32];
        double sum = block_sum(objv, osh);
        if (threadIdx.x == 0) objPartials[blockIdx.x] = sum;
    }
    if (STAGE == 1) {
        // reduce_max of the CFL sums (density.py:405-410): warp shuffle, block, then an atomic
        // max on the bit pattern (non-negative doubles order like their bits). A NaN wins every
        // comparison, as in the reference's max (a NaN's bits are above every finite double's),
        // so a state gone non-finite gives a non-finite CFL sum and the step reports it
        double d = (double)dtc;
        for (int off = 16; off > 0; off >>= 1) d = nan_max(d, __shfl_down_sync(0xffffffffu, d, off));
        __shared__ double wmax[BLOCK / 32];
        if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = d;
        __syncthreads();
        if (threadIdx.x < 32) {
            d = (threadIdx.x < BLOCK / 32) ? wmax[threadIdx.x] : 0.0;
            for (int off = 16; off > 0; off >>= 1) d = nan_max(d, __shfl_down_sync(0xffffffffu, d, off));
            if (threadIdx.x == 0) atomicMax(dtcBits, (unsigned long long)__double_as_longlong(d));
        }
    }
}

// rows of U (3), T, p with absolute T and p from records of stride `stride` (FP32 records hold
// gauge offsets) into out (n x 5)
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_abs_prims(const R* __restrict__ rec, int stride, int n, Phys P,
                                                     R* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const R* r = rec + (size_t)t * stride;
    R* o = out + (size_t)t * 5;
    o[0] = r[0]; o[1] = r[1]; o[2] = r[2];
    o[3] = rec_abs_T<R>(P, r[3]);
    o[4] = rec_abs_p<R>(P, r[4]);
}
void launch_abs_prims(const Ctx* c, const float* rec, int stride, int n, float* out, cudaStream_t s) {
    if (n > 0) k_abs_prims<float><<<nblocks(n), BLOCK, 0, s>>>(rec, stride, n, c->phys, out);
}

// ---- objectives, evaluated on the ghost-completed primitives of stage 1 ----

// per-block partial sums; kinds: AFVM_OBJ_KINETIC_ENERGY, AFVM_OBJ_SUM_T (cells) and
// AFVM_OBJ_DRAG (faces [start, start+n) of one patch, templates/cylinder_test.py:9-19)
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_objective(MeshDev<R> m, Phys P, const R* __restrict__ rec, int kind,
                                                     int start, int n, double* partials) {
    __shared__ double sh[BLOCK / 32];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (t < n) {
        if (kind == AFVM_OBJ_KINETIC_ENERGY || kind == AFVM_OBJ_SUM_T) {
            // per-cell term in the working precision R, accumulated in double
            v = cell_objective<R>(P, kind, rec + (size_t)t * REC, m.vol[t]);
        } else {
            int f = start + t;
            const R* rN = rec + (size_t)m.nbr[f] * REC;
            const R* rP = rec + (size_t)m.own[f] * REC;
            double U0 = rN[0], U0i = rP[0], p0 = rec_p<R>(P, rN[R_P]), T0 = rec_T<R>(P, rN[R_T]);
            double nx = m.nrm[f];
            double mu = (P.muModel == AFVM_MU_SUTHERLAND) ? (P.muAs * (T0 * sqrt(T0))) / (T0 + P.muTs) : P.mu0;
            double mungUx = mu * (U0 - U0i) / (double)m.dlt[f];
            v = (p0 * nx - mungUx) * (double)m.area[f];
        }
    }
    double s = block_sum(v, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// turbine-vane objective on the stage-1 primitives (adFVM/objectives/vane.py:7-60): threads
// [0, nPlane) take the plane cells (pressure-loss and weighting terms), the next nHeat threads
// the heat-transfer faces; three block partial sums (FP64) in partials[0|1|2][block]
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_obj_vane(MeshDev<R> m, Phys P, const R* __restrict__ rec, VaneDev v,
                                                    int nBlocks, double* partials) {
    __shared__ double sh0[BLOCK / 32], sh1[BLOCK / 32], sh2[BLOCK / 32];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0, w = 0.0, h = 0.0;
    if (t < v.nPlane) {
        const R* r = rec + (size_t)v.planeCells[t] * REC;
        double U[3] = {r[0], r[1], r[2]};
        vane_cell(P, v, U, rec_T<R>(P, r[R_T]), rec_p<R>(P, r[R_P]), v.planeArea[t], l, w);
    } else if (t < v.nPlane + v.nHeat) {
        int q = t - v.nPlane;
        int f = v.heatFaces[q];
        h = v.heatCoef[q] * (v.Tw - rec_T<R>(P, rec[(size_t)m.own[f] * REC + R_T]));
    }
    double s0 = block_sum(l, sh0), s1 = block_sum(w, sh1), s2 = block_sum(h, sh2);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s0;
        partials[nBlocks + blockIdx.x] = s1;
        partials[2 * nBlocks + blockIdx.x] = s2;
    }
}

// fixed-order sums of the vane partials into sums[0..2]; with objOut, also the objective
// a L/W + b H/sum(A w) and the dtc bits, as k_finish does
__global__ void k_vane_finish(const double* partials, int nBlocks, VaneDev v, double* sums,
                              const unsigned long long* dtcBits, double* dtcOut, double* objOut) {
    __shared__ double sh0[BLOCK / 32], sh1[BLOCK / 32], sh2[BLOCK / 32];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nBlocks; i += BLOCK) {
        a += partials[i];
        b += partials[nBlocks + i];
        c += partials[2 * nBlocks + i];
    }
    double L = block_sum(a, sh0), W = block_sum(b, sh1), H = block_sum(c, sh2);
    if (threadIdx.x == 0) {
        sums[0] = L;
        sums[1] = W;
        sums[2] = H;
        if (objOut) *objOut = v.a * (L / W) + v.b * (H * v.rw2);
        if (dtcOut) *dtcOut = __longlong_as_double((long long)*dtcBits);
    }
}

template <typename R>
void launch_vane_sums(Ctx* c, cudaStream_t s, double* dtcOut, double* objOut, const R* rec) {
    const MeshDev<R>& m = meshOf<R>(c);
    {
        ProfScope ps(c, KID_OBJECTIVE, s);
        k_obj_vane<R><<<c->nVaneBlocks, BLOCK, 0, s>>>(m, c->phys, rec ? rec : (const R*)c->rec, c->vane,
                                                      c->nVaneBlocks, c->vanePartials);
    }
    ProfScope ps(c, KID_FINISH, s);
    k_vane_finish<<<1, BLOCK, 0, s>>>(c->vanePartials, c->nVaneBlocks, c->vane, c->vaneSums, c->dtcBits, dtcOut,
                                      objOut);
}

// fixed-order final sum of the partials (deterministic) and the dtc bits -> double
__global__ void k_finish(const double* partials, int nPartials, const unsigned long long* dtcBits,
                         double* dtcOut, double* objOut, int haveObj) {
    __shared__ double sh[BLOCK / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < nPartials; i += BLOCK) v += partials[i];
    double s = block_sum(haveObj ? v : 0.0, sh);
    if (threadIdx.x == 0) {
        if (objOut) *objOut = haveObj ? s : 0.0;
        if (dtcOut) *dtcOut = __longlong_as_double((long long)*dtcBits);
    }
}


template <typename R, typename S>
void launch_prim(Ctx* c, const S* r, const S* ru, const S* re, cudaStream_t s, R* rec) {
    const MeshDev<R>& m = meshOf<R>(c);
    ProfScope ps(c, KID_PRIM, s);
    k_prim<R, S><<<nblocks(m.nIC + m.nG), BLOCK, 0, s>>>(m, c->phys, r, ru, re, rec ? rec : (R*)c->rec);
}

template <typename R, typename S>
void launch_prim_grad(Ctx* c, const S* r, const S* ru, const S* re, cudaStream_t s, R* rec) {
    const MeshDev<R>& m = meshOf<R>(c);
    if (!rec) rec = (R*)c->rec;
    launch_prim<R, S>(c, r, ru, re, s, rec);
    {
        ProfScope ps(c, KID_GRAD, s);
        k_grad<R><<<nblocks(m.nIC), BLOCK, 0, s>>>(m, c->phys, rec);
    }
}

// faces -> fluxes, then the gather + stage update u_{st+1} = ... (timestep.py:35-45)
template <typename R, typename S>
void launch_flux_update(Ctx* c, int st, double dt, const double* dtDev, const S* const* u0, const S* const* u1,
                        const S* const* u2, const S* Sr, const S* Su, const S* Se, S* const* out, cudaStream_t s,
                        bool nextPrims, R* tape, R* recIn, R* recOut, double* objPartials) {
    const MeshDev<R>& m = meshOf<R>(c);
    const Phys& P = c->phys;
    R* rec = recIn ? recIn : (R*)c->rec;
    R* ff = (R*)c->fflux;
    int inviscid = (P.muModel == AFVM_MU_CONSTANT && P.mu0 == 0.0) ? 1 : 0;
    {
        ProfScope ps(c, KID_FLUX, s);
        int nbF = (m.nF + FLUX_BLOCK - 1) / FLUX_BLOCK;
        if (tape && st == 1)
            k_flux<R, true, true><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, ff, inviscid, tape);
        else if (tape)
            k_flux<R, true, false><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, ff, inviscid, tape);
        else if (st == 1)
            k_flux<R, false, true><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, ff, inviscid, nullptr);
        else
            k_flux<R, false, false><<<nbF, FLUX_BLOCK, 0, s>>>(m, P, rec, ff, inviscid, nullptr);
    }
    int nb = nblocks(m.nIC);
    R* recNext = nextPrims ? (recOut ? recOut : rec) : nullptr;
    ProfScope ps(c, KID_UPDATE, s);
    if (st == 0)
        k_update<R, S, 0><<<nb, BLOCK, 0, s>>>(m, ff, dt, dtDev, u0[0], u0[1], u0[2], nullptr, nullptr, nullptr, nullptr,
                                            nullptr, nullptr, Sr, Su, Se, out[0], out[1], out[2], c->dtcBits, P,
                                            recNext, c->objective, recNext ? objPartials : nullptr);
    else if (st == 1)
        k_update<R, S, 1><<<nb, BLOCK, 0, s>>>(m, ff, dt, dtDev, u0[0], u0[1], u0[2], u1[0], u1[1], u1[2], nullptr,
                                            nullptr, nullptr, Sr, Su, Se, out[0], out[1], out[2], c->dtcBits, P,
                                            recNext, c->objective, nullptr);
    else
        k_update<R, S, 2><<<nb, BLOCK, 0, s>>>(m, ff, dt, dtDev, u0[0], u0[1], u0[2], nullptr, nullptr, nullptr, u2[0],
                                            u2[1], u2[2], Sr, Su, Se, out[0], out[1], out[2], c->dtcBits, P,
                                            recNext, c->objective, nullptr);
}

template <typename S>
void default_sources(Ctx* c, const S*& Srho, const S*& SrhoU, const S*& SrhoE) {
    const S* zs = (const S*)c->zeroS;
    if (!Srho) Srho = zs;
    if (!SrhoU) SrhoU = zs + c->nIC;
    if (!SrhoE) SrhoE = zs + 4 * (size_t)c->nIC;
}

template <typename R, typename S>
int primal_step_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, double dt, const double* dtDev,
                    const S* Srho, const S* SrhoU, const S* SrhoE, S* rhoN, S* rhoUN, S* rhoEN,
                    double* dtcDev, double* objDev, cudaStream_t s, S* stages, R* tape) {
    const MeshDev<R>& m = meshOf<R>(c);
    const Phys& P = c->phys;
    default_sources<S>(c, Srho, SrhoU, SrhoE);
    S* u1[3] = {(S*)c->u1[0], (S*)c->u1[1], (S*)c->u1[2]};
    S* u2[3] = {(S*)c->u2[0], (S*)c->u2[1], (S*)c->u2[2]};
    if (stages) stage_views<S, S>(stages, m.nIC, u1, u2);
    S* outN[3] = {rhoN, rhoUN, rhoEN};
    const S* u0c[3] = {rho, rhoU, rhoE};
    const S* u1c[3] = {u1[0], u1[1], u1[2]};
    const S* u2c[3] = {u2[0], u2[1], u2[2]};
    cudaMemsetAsync(c->dtcBits, 0, sizeof(unsigned long long), s);
    int nObjBlocks = 0;
    bool vaneDone = false;
    if (c->objective == AFVM_OBJ_VANE && !c->vaneSet)
        return fail(c, AFVM_ERR_BAD_ARG, "AFVM_OBJ_VANE needs afvm_set_objective_vane before the first step");
    // with a tape each stage's cell records are built in the tape's record part (kept for the
    // adjoint step), else in the context's one record buffer
    R* faceTape = nullptr;
    R* recTape = nullptr;
    split_tape<R>(c, tape, faceTape, recTape);
    R* recs[3];
    for (int st = 0; st < 3; st++) recs[st] = recTape ? recTape + (size_t)st * m.nC * REC : (R*)c->rec;
    for (int st = 0; st < 3; st++) {
        const S* const* in = st == 0 ? u0c : (st == 1 ? u1c : u2c);
        if (st == 0) {
            launch_prim_grad<R, S>(c, in[0], in[1], in[2], s, recs[0]);
        } else {
            // the primitives of stages 1 and 2 were written by the previous stage's update
            ProfScope ps(c, KID_GRAD, s);
            k_grad<R><<<nblocks(m.nIC), BLOCK, 0, s>>>(m, c->phys, recs[st]);
        }
        if (st == 1 && c->objSink) {
            // the objective stage's primitives U (3), T, p of every cell, ghosts included, for an
            // objective evaluated by the caller (absolute values: FP32 records add their gauge)
            if constexpr (kGauge<R>)
                k_abs_prims<R><<<nblocks(m.nC), BLOCK, 0, s>>>(recs[1], REC, m.nC, P, (R*)c->objSink);
            else
                cudaMemcpy2DAsync(c->objSink, 5 * sizeof(R), recs[1], REC * sizeof(R), 5 * sizeof(R), (size_t)m.nC,
                                  cudaMemcpyDeviceToDevice, s);
        }
        if (st == 1 && c->objective == AFVM_OBJ_VANE) {
            // the partial sums now, while rec holds the stage-1 primitives; combined at the end
            const MeshDev<R>& mm = meshOf<R>(c);
            ProfScope ps(c, KID_OBJECTIVE, s);
            k_obj_vane<R><<<c->nVaneBlocks, BLOCK, 0, s>>>(mm, P, (const R*)recs[1], c->vane, c->nVaneBlocks,
                                                          c->vanePartials);
            vaneDone = true;
        } else if (st == 1 && c->objective != AFVM_OBJ_NONE) {
            int start = 0, n = m.nIC;
            if (c->objective == AFVM_OBJ_DRAG) { start = c->objStart; n = c->objN; }
            nObjBlocks = nblocks(n);
            if (nObjBlocks > c->nPartials) return fail(c, AFVM_ERR_BAD_ARG, "objective partials overflow");
            // a cell-sum objective's partials were written by the stage-0 update
            if (n > 0 && !cell_sum_objective(c->objective)) {
                ProfScope ps(c, KID_OBJECTIVE, s);
                k_objective<R><<<nObjBlocks, BLOCK, 0, s>>>(m, P, (const R*)recs[1], c->objective, start, n,
                                                            c->partials);
            }
        }
        S* const* out = st == 0 ? u1 : (st == 1 ? u2 : outN);
        double* objPartials = (st == 0 && cell_sum_objective(c->objective) && nblocks(m.nIC) <= c->nPartials)
                                  ? c->partials : nullptr;
        if (st == 0 && cell_sum_objective(c->objective) && !objPartials)
            return fail(c, AFVM_ERR_BAD_ARG, "objective partials overflow");
        launch_flux_update<R, S>(c, st, dt, dtDev, u0c, u1c, u2c, Srho, SrhoU, SrhoE, out, s, st < 2,
                                 faceTape ? faceTape + (size_t)st * TAPE * m.nF : nullptr, recs[st],
                                 st < 2 ? recs[st + 1] : nullptr, objPartials);
    }
    if (vaneDone) {
        ProfScope ps(c, KID_FINISH, s);
        k_vane_finish<<<1, BLOCK, 0, s>>>(c->vanePartials, c->nVaneBlocks, c->vane, c->vaneSums, c->dtcBits, dtcDev,
                                          objDev);
    } else {
        ProfScope ps(c, KID_FINISH, s);
        k_finish<<<1, BLOCK, 0, s>>>(c->partials, nObjBlocks, c->dtcBits, dtcDev, objDev, nObjBlocks > 0);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "primal step launch");
    return AFVM_OK;
}

// time-step rule of the reference loop, dt <- min(2*CFL/dtc, stepFactor*dt)
// (adFVM/solver.py:365), kept on the device; records the dt each step used
__global__ void k_next_dt(double* dt, const double* dtc, double CFL, double stepFactor, int fixed, double* dtHist) {
    double d = *dt;
    if (dtHist) *dtHist = d;
    if (!fixed) *dt = fmin(2 * CFL / *dtc, d * stepFactor);
}

template <typename R, typename S>
int primal_run_dev(Ctx* c, S* rho, S* rhoU, S* rhoE, int nSteps, double dt0, double CFL, double stepFactor,
                   int fixed, const S* Srho, const S* SrhoU, const S* SrhoE, double* dtHist, double* dtcHist,
                   double* objHist, cudaStream_t s) {
    double* dtDev = c->scal + 2;
    cudaMemcpyAsync(dtDev, &dt0, sizeof(double), cudaMemcpyHostToDevice, s);
    for (int n = 0; n < nSteps; n++) {
        double* dtcOut = dtcHist ? dtcHist + n : c->scal;
        int st = primal_step_dev<R, S>(c, rho, rhoU, rhoE, 0.0, dtDev, Srho, SrhoU, SrhoE, rho, rhoU, rhoE, dtcOut,
                                    objHist ? objHist + n : c->scal + 1, s);
        if (st != AFVM_OK) return st;
        k_next_dt<<<1, 1, 0, s>>>(dtDev, dtcOut, CFL, stepFactor, fixed, dtHist ? dtHist + n : nullptr);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "primal run launch");
    return AFVM_OK;
}

#define AFVM_PRIMAL_INST(R, S)                                                                                 \
    template int primal_step_dev<R, S>(Ctx*, const S*, const S*, const S*, double, const double*, const S*,       \
                                       const S*, const S*, S*, S*, S*, double*, double*, cudaStream_t, S*, R*);   \
    template int primal_run_dev<R, S>(Ctx*, S*, S*, S*, int, double, double, double, int, const S*, const S*,     \
                                      const S*, double*, double*, double*, cudaStream_t);                         \
    template void launch_prim<R, S>(Ctx*, const S*, const S*, const S*, cudaStream_t, R*);                       \
    template void launch_prim_grad<R, S>(Ctx*, const S*, const S*, const S*, cudaStream_t, R*);                  \
    template void launch_flux_update<R, S>(Ctx*, int, double, const double*, const S* const*, const S* const*,   \
                                           const S* const*, const S*, const S*, const S*, S* const*, cudaStream_t,  \
                                           bool, R*, R*, R*, double*);
AFVM_PRIMAL_INST(double, double)
AFVM_PRIMAL_INST(float, float)
AFVM_PRIMAL_INST(float, double)
template void default_sources<double>(Ctx*, const double*&, const double*&, const double*&);
template void default_sources<float>(Ctx*, const float*&, const float*&, const float*&);
template void launch_vane_sums<double>(Ctx*, cudaStream_t, double*, double*, const double*);
template void launch_vane_sums<float>(Ctx*, cudaStream_t, double*, double*, const float*);

}  // namespace afvm
