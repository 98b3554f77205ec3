// Adjoint stabilisation by artificial viscosity (adFVM/postpro.py:491-718 with the compiled
// helpers of adFVM/cpp/scaling.cpp:84-159 and the heat equation of matop_petsc.cpp:230-372).
//
// For a primal state u:
//   k_visc_cell   per cell, gathered over its faces in the reference's collate order: face
//                 values (central on internal and coupled faces, the ghost value on other
//                 boundary faces) -> gradU, divU, gradp, gradc (op.grad / op.div); the 5x5
//                 symmetriser M of the 'turkel' or 'abarbanel' kind, MS = (M + M^T)/2, and its
//                 largest eigenvalue by cyclic Jacobi rotations (FP64, in registers); 'uniform'
//                 is 1. Block partial sums of M^2 V.
//   k_visc_scale  M <- scaling M / sqrt(sum M^2 V / sum V); ghost values of the default
//                 boundary (the ghost's source cell); per face DT = w M_own + (1-w) M_nbr and
//                 the coefficient dt A DT / delta of the implicit heat equation.
// and the adjoint fields a (plain gradients) are replaced by V x, where x solves, for each of
// the 5 components,
//   V_c x_c + sum_k dt A_k DT_k / delta_k (x_c - x_nbr(k)) = V_c (a_c / V_c)
// over the faces k of c with an internal neighbour - the symmetric form of the reference's
// (1 + sum coef) x_c - sum coef x_nbr = x0_c, coef = dt A DT / (delta V_c). It is solved by
// preconditioned conjugate gradients (Jacobi preconditioner), the five components in lockstep,
// to a relative residual of 1e-13 (the reference: 1000 Jacobi sweeps on the GPU or GMRES
// through PETSc on the CPU). Everything here is FP64 whatever the context's precision.
#include <cuda_runtime.h>
#include <math.h>
#include "ctx.cuh"
#include "physics.cuh"

namespace afvm {

namespace {

constexpr double UREF = 33., PREF = 1e5;   // RCF reference scales (adFVM/density.py:57-59)

__device__ __forceinline__ double vblock_sum(double v, double* sh) {
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

// largest eigenvalue of a symmetric 5x5 (upper triangle used) by cyclic Jacobi rotations
// (Golub & Van Loan, Matrix Computations, the symmetric Schur decomposition); at most 40
// sweeps, stopping when the off-diagonal mass is below 1e-32 of the whole
__device__ double max_eig5(double a[5][5]) {
    for (int sweep = 0; sweep < 40; sweep++) {
        double off = 0.0, dia = 0.0;
        for (int i = 0; i < 5; i++) {
            dia += a[i][i] * a[i][i];
            for (int j = i + 1; j < 5; j++) off += a[i][j] * a[i][j];
        }
        if (off <= 1e-32 * (dia + off) || off == 0.0) break;
        for (int p = 0; p < 4; p++) {
            for (int q = p + 1; q < 5; q++) {
                double apq = a[p][q];
                if (apq == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0);
                double s = t * c;
                // A <- J^T A J on rows/columns p, q of the symmetric matrix (upper triangle)
                for (int k = 0; k < 5; k++) {
                    if (k == p || k == q) continue;
                    double akp = (k < p) ? a[k][p] : a[p][k];
                    double akq = (k < q) ? a[k][q] : a[q][k];
                    double np_ = c * akp - s * akq;
                    double nq_ = s * akp + c * akq;
                    if (k < p) a[k][p] = np_; else a[p][k] = np_;
                    if (k < q) a[k][q] = nq_; else a[q][k] = nq_;
                }
                double app = a[p][p], aqq = a[q][q];
                a[p][p] = app - t * apq;
                a[q][q] = aqq + t * apq;
                a[p][q] = 0.0;
                (void)app; (void)aqq;
            }
        }
    }
    double m = a[0][0];
    for (int i = 1; i < 5; i++) m = fmax(m, a[i][i]);
    return m;
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_visc_cell(MeshDev<R> m, Phys P, const R* __restrict__ rec, int kind,
                                                     double* __restrict__ M, double* __restrict__ partials) {
    __shared__ double sh[BLOCK / 32];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    double contrib = 0.0;
    if (c < m.nIC) {
        const size_t n = m.nIC;
        const size_t nF = m.nF;
        const double g = P.gamma, Rg = P.Cp - P.Cv;
        double gU[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, dU = 0.0, gp[3] = {0, 0, 0}, gc[3] = {0, 0, 0};
        for (int k = 0; k < 6; k++) {
            int e = m.accf[k * n + c];
            double wt = m.accw[k * n + c];
            bool ownerSide = e >= 0;
            int f = ownerSide ? e : ~e;
            const R* rN = rec + (size_t)m.nbr[f] * REC;
            double UF[3], pF, cF;
            bool central = f < m.nIF || m.fkind[f - m.nIF] == FACE_COUPLED;
            if (central) {
                const R* rO = rec + (size_t)m.own[f] * REC;
                double w = m.wts[f];
                for (int i = 0; i < 3; i++) UF[i] = (double)rO[i] * w + (double)rN[i] * (-w + 1);
                pF = (double)rO[R_P] * w + (double)rN[R_P] * (-w + 1);
                double cL = sqrt(g * rec_T<R>(P, rO[R_T]) * Rg), cR = sqrt(g * rec_T<R>(P, rN[R_T]) * Rg);
                cF = cR * (-w + 1) + cL * w;
            } else {
                for (int i = 0; i < 3; i++) UF[i] = rN[i];
                pF = rN[R_P];
                cF = sqrt(g * rec_T<R>(P, rN[R_T]) * Rg);
            }
            double N[3] = {(double)m.nrm[f], (double)m.nrm[nF + f], (double)m.nrm[2 * nF + f]};
            double sw = ownerSide ? wt : -wt;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) gU[i][j] += (UF[i] * N[j]) * sw;
            dU += (UF[0] * N[0] + UF[1] * N[1] + UF[2] * N[2]) * sw;
            for (int j = 0; j < 3; j++) {
                gp[j] += (pF * N[j]) * sw;
                gc[j] += (cF * N[j]) * sw;
            }
        }
        // FP32 records hold p - gaugeP: the sum above missed gaugeP times the cell's sum of A/V N
        // (zero when the cell's face area vectors close, not for warped faces)
        if constexpr (kGauge<R>)
            for (int j = 0; j < 3; j++) gp[j] += P.gaugeP * m.gclD[j * n + c];
        double val = 1.0;
        if (kind != AFVM_VISC_UNIFORM) {
            const R* r = rec + (size_t)c * REC;
            double T = rec_T<R>(P, r[R_T]), p = rec_p<R>(P, r[R_P]);
            double rho = p / ((P.Cv * T) * (g - 1));
            double cc = sqrt(g * p / rho);
            double grho[3];
            for (int j = 0; j < 3; j++) grho[j] = g * (gp[j] - cc * p) / (cc * cc);
            double g1 = g - 1;
            double A[5][5];
            for (int i = 0; i < 5; i++)
                for (int j = 0; j < 5; j++) A[i][j] = 0.0;
            // M = M1/2 - M2 (postpro.py:571-602)
            if (kind == AFVM_VISC_TURKEL) {
                for (int i = 0; i < 5; i++) A[i][i] = dU / 2;
                for (int j = 0; j < 3; j++) { A[0][1 + j] += gc[j] / 2; A[1 + j][0] += gc[j] / 2; }
                A[0][0] -= g1 * dU / 2;
                for (int j = 0; j < 3; j++) {
                    A[0][1 + j] -= gp[j] / (rho * cc);
                    A[1 + j][0] -= g1 * gp[j] / (2 * rho * cc);
                    A[1 + j][4] -= gp[j] * PREF / (2 * g * p * rho * UREF);
                    A[4][1 + j] -= (gp[j] - cc * cc * grho[j]) * UREF / PREF;
                    for (int k = 0; k < 3; k++) A[1 + j][1 + k] -= gU[j][k];
                }
                A[0][4] -= dU * PREF / (2 * rho * cc * UREF);
                A[4][4] -= g1 * dU / 2;
            } else {
                double sg = sqrt(g), sg1 = sqrt(g1);
                double b = cc / sg, a = sg1 * cc / sg;
                double gb[3], ga[3];
                for (int j = 0; j < 3; j++) { gb[j] = gc[j] / sg; ga[j] = gc[j] * sg1 / sg; }
                for (int i = 0; i < 5; i++) A[i][i] = dU / 2;
                for (int j = 0; j < 3; j++) {
                    A[0][1 + j] += gb[j] / 2; A[1 + j][0] += gb[j] / 2;
                    A[1 + j][4] += ga[j] / 2; A[4][1 + j] += ga[j] / 2;
                }
                for (int j = 0; j < 3; j++) {
                    A[0][1 + j] -= b * grho[j] / rho;
                    A[1 + j][4] -= a * gp[j] / (2 * p);
                    A[4][1 + j] -= 2 * ga[j] / g1;
                    for (int k = 0; k < 3; k++) A[1 + j][1 + k] -= gU[j][k];
                }
                A[0][4] -= sg1 * dU / 2;
                A[4][4] -= g1 * dU / 2;
            }
            // MS = (M + M^T)/2, upper triangle
            double S[5][5];
            for (int i = 0; i < 5; i++)
                for (int j = i; j < 5; j++) S[i][j] = (A[i][j] + A[j][i]) / 2;
            val = max_eig5(S);
        }
        M[c] = val;
        contrib = val * val * (double)m.vol[c];
    }
    double s = vblock_sum(contrib, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void k_visc_norm(const double* partials, int nb, double Vt, double scaling, double* fac) {
    __shared__ double sh[BLOCK / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < nb; i += BLOCK) v += partials[i];
    double s = vblock_sum(v, sh);
    if (threadIdx.x == 0) fac[0] = scaling / sqrt(s / Vt);
}

// scaled M with ghost values, then per face DT and the heat-equation coefficient dt A DT / delta
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_visc_scale(MeshDev<R> m, double* __restrict__ M, const double* fac) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < m.nIC) M[c] = M[c] * fac[0];
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_visc_ghost(MeshDev<R> m, double* __restrict__ M) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < m.nG) M[m.nIC + g] = M[m.gsrc[g]];
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_visc_face(MeshDev<R> m, const double* __restrict__ M, double dt,
                                                     double* __restrict__ DT, double* __restrict__ coef) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nF) return;
    double w = m.wts[f];
    double d = M[m.own[f]] * w + M[m.nbr[f]] * (-w + 1);
    DT[f] = d;
    coef[f] = dt * ((double)m.area[f] * d / (double)m.dlt[f]);
}

// ---- PCG on (V + dt L) x = V b, five right-hand sides in lockstep (component-major, 5 x n)

// y = A x over internal-neighbour faces (cellFaces slots with an internal neighbour); also the
// diagonal when diag != NULL
template <typename R>
__global__ void __launch_bounds__(BLOCK) k_heat_apply(MeshDev<R> m, const double* __restrict__ coef,
                                                      const double* __restrict__ x, double* __restrict__ y,
                                                      double* __restrict__ diag, const double* __restrict__ pz,
                                                      double* __restrict__ partials, int nb) {
    __shared__ double sh[5][BLOCK / 32];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = m.nIC;
    double dots[5] = {0, 0, 0, 0, 0};
    if (c < m.nIC) {
        double V = m.vol[c];
        double d = V;
        double acc[5];
        for (int q = 0; q < 5; q++) acc[q] = V * x[q * n + c];
        for (int k = 0; k < 6; k++) {
            int e = m.accf[k * n + c];
            int f = e >= 0 ? e : ~e;
            if (f >= m.nIF) continue;
            int nbh = e >= 0 ? m.nbr[f] : m.own[f];
            double w = coef[f];
            d += w;
            for (int q = 0; q < 5; q++) acc[q] += w * (x[q * n + c] - x[q * n + nbh]);
        }
        for (int q = 0; q < 5; q++) y[q * n + c] = acc[q];
        if (diag) diag[c] = d;
        if (pz)
            for (int q = 0; q < 5; q++) dots[q] = pz[q * n + c] * acc[q];
    }
    if (partials) {
        for (int q = 0; q < 5; q++) {
            double s = vblock_sum(dots[q], sh[q]);
            if (threadIdx.x == 0) partials[q * nb + blockIdx.x] = s;
        }
    }
}

// per component: the sum of the partials -> out[q]
__global__ void k_sum5(const double* partials, int nb, double* out) {
    __shared__ double sh[BLOCK / 32];
    for (int q = 0; q < 5; q++) {
        double v = 0.0;
        for (int i = threadIdx.x; i < nb; i += BLOCK) v += partials[q * nb + i];
        double s = vblock_sum(v, sh);
        if (threadIdx.x == 0) out[q] = s;
        __syncthreads();
    }
}

// r = rhs - Ax (Ax in r on entry); z = r / diag; p = z; partial r.z and r.r
__global__ void k_cg_init(int n, const double* __restrict__ rhs, const double* __restrict__ diag,
                          double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                          double* __restrict__ partials, int nb) {
    __shared__ double sh[10][BLOCK / 32];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    double rz[5] = {0, 0, 0, 0, 0}, rr[5] = {0, 0, 0, 0, 0};
    if (c < n) {
        for (int q = 0; q < 5; q++) {
            size_t i = (size_t)q * n + c;
            double rv = rhs[i] - r[i];
            double zv = rv / diag[c];
            r[i] = rv; z[i] = zv; p[i] = zv;
            rz[q] = rv * zv; rr[q] = rv * rv;
        }
    }
    for (int q = 0; q < 5; q++) {
        double a = vblock_sum(rz[q], sh[q]);
        double b = vblock_sum(rr[q], sh[5 + q]);
        if (threadIdx.x == 0) { partials[q * nb + blockIdx.x] = a; partials[(5 + q) * nb + blockIdx.x] = b; }
    }
}

// x += alpha p; r -= alpha q; z = r / diag; partial r.z (new) and r.r; alpha = rz / pq per component
__global__ void k_cg_update(int n, const double* __restrict__ sc, double* __restrict__ x, double* __restrict__ r,
                            double* __restrict__ z, const double* __restrict__ p, const double* __restrict__ q,
                            const double* __restrict__ diag, double* __restrict__ partials, int nb) {
    __shared__ double sh[10][BLOCK / 32];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    double rz[5] = {0, 0, 0, 0, 0}, rr[5] = {0, 0, 0, 0, 0};
    if (c < n) {
        for (int k = 0; k < 5; k++) {
            double pq = sc[5 + k];
            double alpha = (pq != 0.0) ? sc[k] / pq : 0.0;
            size_t i = (size_t)k * n + c;
            x[i] += alpha * p[i];
            double rv = r[i] - alpha * q[i];
            double zv = rv / diag[c];
            r[i] = rv; z[i] = zv;
            rz[k] = rv * zv; rr[k] = rv * rv;
        }
    }
    for (int k = 0; k < 5; k++) {
        double a = vblock_sum(rz[k], sh[k]);
        double b = vblock_sum(rr[k], sh[5 + k]);
        if (threadIdx.x == 0) { partials[k * nb + blockIdx.x] = a; partials[(5 + k) * nb + blockIdx.x] = b; }
    }
}

// sc layout: [0..5) r.z, [5..10) p.Ap, [10..15) new r.z, [15..20) r.r, [20..25) |rhs|^2
__global__ void k_cg_scalars(const double* partials, int nb, double* sc, int init) {
    __shared__ double sh[BLOCK / 32];
    for (int k = 0; k < 10; k++) {
        double v = 0.0;
        for (int i = threadIdx.x; i < nb; i += BLOCK) v += partials[k * nb + i];
        double s = vblock_sum(v, sh);
        if (threadIdx.x == 0) {
            if (k < 5) sc[init ? k : 10 + k] = s;
            else sc[15 + (k - 5)] = s;
        }
        __syncthreads();
    }
}

// p = z + beta p, beta = rz_new / rz_old; then rz_old <- rz_new
__global__ void k_cg_direction(int n, double* __restrict__ sc, const double* __restrict__ z, double* __restrict__ p) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) {
        for (int k = 0; k < 5; k++) {
            double beta = (sc[k] != 0.0) ? sc[10 + k] / sc[k] : 0.0;
            size_t i = (size_t)k * n + c;
            p[i] = z[i] + beta * p[i];
        }
    }
}

__global__ void k_cg_shift(double* sc) {
    if (threadIdx.x < 5) sc[threadIdx.x] = sc[10 + threadIdx.x];
}

template <typename S>
__global__ void k_heat_rhs(int n, const S* __restrict__ ar, const S* __restrict__ au, const S* __restrict__ ae,
                           double* __restrict__ rhs, double* __restrict__ partials, int nb) {
    __shared__ double sh[5][BLOCK / 32];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    double v[5] = {0, 0, 0, 0, 0};
    if (c < n) {
        // V (a / V) = a: the right-hand side of the symmetric form is the adjoint field itself
        v[0] = ar[c]; v[1] = au[3 * c]; v[2] = au[3 * c + 1]; v[3] = au[3 * c + 2]; v[4] = ae[c];
        for (int q = 0; q < 5; q++) rhs[(size_t)q * n + c] = v[q];
    }
    for (int q = 0; q < 5; q++) {
        double s = vblock_sum(v[q] * v[q], sh[q]);
        if (threadIdx.x == 0) partials[q * nb + blockIdx.x] = s;
    }
}

template <typename R>
__global__ void k_heat_x0(MeshDev<R> m, const double* __restrict__ rhs, double* __restrict__ x) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = m.nIC;
    if (c >= m.nIC) return;
    double V = m.vol[c];
    for (int k = 0; k < 5; k++) x[k * n + c] = rhs[k * n + c] / V;
}

template <typename R, typename S>
__global__ void k_heat_out(MeshDev<R> m, const double* __restrict__ x, S* __restrict__ ar, S* __restrict__ au,
                           S* __restrict__ ae) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = m.nIC;
    if (c >= m.nIC) return;
    double V = m.vol[c];
    ar[c] = (S)(x[c] * V);
    for (int k = 0; k < 3; k++) au[3 * c + k] = (S)(x[(1 + k) * n + c] * V);
    ae[c] = (S)(x[4 * n + c] * V);
}

}  // namespace

template <typename R, typename S>
int adjoint_viscosity_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, int kind, double scaling, double dt,
                          S* ar, S* au, S* ae, double* Mout, double* DTout, int* iters, cudaStream_t s) {
    const MeshDev<R>& m = meshOf<R>(c);
    const Phys& P = c->phys;
    const size_t n = c->nIC;
    const int nb = nblocks(c->nIC);
    if (!c->viscWork) {
        size_t words = (size_t)c->nC + 2 * (size_t)c->nF + 7 * 5 * n + 15 * (size_t)nb + 64;
        int st = ctx_alloc(c, (void**)&c->viscWork, sizeof(double) * words);
        if (st) return st;
    }
    double* M = c->viscWork;                 // nC: the viscosity with ghost values
    double* DT = M + c->nC;                  // nF
    double* coef = DT + c->nF;               // nF: dt A DT / delta
    double* x = coef + c->nF;                // five component-major vectors of 5n each
    double* r = x + 5 * n;
    double* z = r + 5 * n;
    double* p = z + 5 * n;
    double* q = p + 5 * n;
    double* rhs = q + 5 * n;
    double* diag = rhs + 5 * n;              // n used
    double* partials = diag + 5 * n;         // 15 x nb
    double* sc = partials + 15 * (size_t)nb; // 64 scalars
    ProfScope ps(c, KID_ADJ_VISC, s);
    launch_prim<R, S>(c, rho, rhoU, rhoE, s);
    k_visc_cell<R><<<nb, BLOCK, 0, s>>>(m, P, (const R*)c->rec, kind, M, partials);
    k_visc_norm<<<1, BLOCK, 0, s>>>(partials, nb, c->volTotal, scaling, sc + 40);
    k_visc_scale<R><<<nb, BLOCK, 0, s>>>(m, M, sc + 40);
    if (c->nG > 0) k_visc_ghost<R><<<nblocks(c->nG), BLOCK, 0, s>>>(m, M);
    k_visc_face<R><<<nblocks(c->nF), BLOCK, 0, s>>>(m, M, dt, DT, coef);
    // PCG on (V + dt L) x = a, from x0 = a / V (the unsmoothed field per unit volume)
    k_heat_rhs<S><<<nb, BLOCK, 0, s>>>(c->nIC, ar, au, ae, rhs, partials, nb);
    k_sum5<<<1, BLOCK, 0, s>>>(partials, nb, sc + 20);
    k_heat_x0<R><<<nb, BLOCK, 0, s>>>(m, rhs, x);
    k_heat_apply<R><<<nb, BLOCK, 0, s>>>(m, coef, x, r, diag, nullptr, nullptr, nb);
    k_cg_init<<<nb, BLOCK, 0, s>>>(c->nIC, rhs, diag, r, z, p, partials, nb);
    k_cg_scalars<<<1, BLOCK, 0, s>>>(partials, nb, sc, 1);
    double hs[25];
    const int maxIt = 500, checkEvery = 4;
    int it = 0;
    for (;; it++) {
        if (it % checkEvery == 0 || it >= maxIt) {
            cudaError_t e = cudaMemcpyAsync(hs, sc, sizeof(double) * 25, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_fail(c, e, "adjoint viscosity solve");
            bool done = true;
            for (int k = 0; k < 5; k++)
                if (!(hs[15 + k] <= 1e-26 * hs[20 + k])) done = false;
            if (done || it >= maxIt) break;
        }
        k_heat_apply<R><<<nb, BLOCK, 0, s>>>(m, coef, p, q, nullptr, p, partials + 10 * (size_t)nb, nb);
        k_sum5<<<1, BLOCK, 0, s>>>(partials + 10 * (size_t)nb, nb, sc + 5);
        k_cg_update<<<nb, BLOCK, 0, s>>>(c->nIC, sc, x, r, z, p, q, diag, partials, nb);
        k_cg_scalars<<<1, BLOCK, 0, s>>>(partials, nb, sc, 0);
        k_cg_direction<<<nb, BLOCK, 0, s>>>(c->nIC, sc, z, p);
        k_cg_shift<<<1, 32, 0, s>>>(sc);
    }
    if (iters) *iters = it;
    k_heat_out<R, S><<<nb, BLOCK, 0, s>>>(m, x, ar, au, ae);
    if (Mout) cudaMemcpyAsync(Mout, M, sizeof(double) * c->nC, cudaMemcpyDeviceToDevice, s);
    if (DTout) cudaMemcpyAsync(DTout, DT, sizeof(double) * c->nF, cudaMemcpyDeviceToDevice, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint viscosity launch");
    if (it >= maxIt) return fail(c, AFVM_ERR_TIMEOUT, "adjoint viscosity: the heat equation did not converge");
    return AFVM_OK;
}

template int adjoint_viscosity_dev<double, double>(Ctx*, const double*, const double*, const double*, int, double,
                                                   double, double*, double*, double*, double*, double*, int*,
                                                   cudaStream_t);
template int adjoint_viscosity_dev<float, float>(Ctx*, const float*, const float*, const float*, int, double, double,
                                                 float*, float*, float*, double*, double*, int*, cudaStream_t);
template int adjoint_viscosity_dev<float, double>(Ctx*, const double*, const double*, const double*, int, double,
                                                  double, double*, double*, double*, double*, double*, int*,
                                                  cudaStream_t);

}  // namespace afvm
