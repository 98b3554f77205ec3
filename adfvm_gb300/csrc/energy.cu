// Adjoint energy sum_c w^T A(u) w V (cmesh.computeEnergy, adFVM/cpp/cmesh.cpp:342-425): the
// symmetrised norm of the adjoint state that the reference's adjoint driver reports as
// sqrt(energy) (apps/adjoint.py:55). FP64 per cell, deterministic block partials + fixed-order
// final sum.
#include <cuda_runtime.h>
#include "ctx.cuh"

namespace afvm {

__device__ __forceinline__ double e_block_sum(double v, double* sh) {
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

template <typename R, typename S>
__global__ void __launch_bounds__(BLOCK) k_energy(MeshDev<R> m, double g, const S* __restrict__ ra,
                                                  const S* __restrict__ rua, const S* __restrict__ rea,
                                                  const S* __restrict__ r, const S* __restrict__ ru,
                                                  const S* __restrict__ re, double* partials) {
    __shared__ double sh[BLOCK / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < m.nIC) {
        double v = m.vol[i];
        double rho = r[i], rE = re[i];
        double u1 = ru[3 * i] / rho, u2 = ru[3 * i + 1] / rho, u3 = ru[3 * i + 2] / rho;
        double q2 = u1 * u1 + u2 * u2 + u3 * u3;
        double p = (rE - rho * q2 / 2) * (g - 1);
        double H = g * p / (rho * (g - 1)) + q2 / 2;
        double w1 = ra[i] / v, w2 = rua[3 * i] / v, w3 = rua[3 * i + 1] / v, w4 = rua[3 * i + 2] / v, w5 = rea[i] / v;
        double A11 = rho, A12 = rho * u1, A13 = rho * u2, A14 = rho * u3, A15 = rE;
        double A22 = rho * u1 * u1 + p, A23 = rho * u1 * u2, A24 = rho * u1 * u3, A25 = rho * H * u1;
        double A33 = rho * u2 * u2 + p, A34 = rho * u2 * u3, A35 = rho * H * u2;
        double A44 = rho * u3 * u3 + p, A45 = rho * H * u3;
        double A55 = rho * H * H - g * p * p / (rho * (g - 1));
        e = (A11 * w1 * w1 + A22 * w2 * w2 + A33 * w3 * w3 + A44 * w4 * w4 + A55 * w5 * w5 +
             2 * (A12 * w1 * w2 + A13 * w1 * w3 + A14 * w1 * w4 + A15 * w1 * w5 + A23 * w2 * w3 + A24 * w2 * w4 +
                  A25 * w2 * w5 + A34 * w3 * w4 + A35 * w3 * w5 + A45 * w4 * w5)) * v;
    }
    double s = e_block_sum(e, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(BLOCK) k_energy_finish(const double* __restrict__ partials, int n, double* out) {
    __shared__ double sh[BLOCK / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += BLOCK) v += partials[i];
    double s = e_block_sum(v, sh);
    if (threadIdx.x == 0) *out = s;
}

template <typename R, typename S>
int energy_dev(Ctx* c, const void* ra, const void* rua, const void* rea, const void* r, const void* ru,
               const void* re, double* out, cudaStream_t s) {
    const MeshDev<R>& m = meshOf<R>(c);
    int nb = nblocks(m.nIC);
    if (nb > c->nPartials) return fail(c, AFVM_ERR_BAD_ARG, "energy partials overflow");
    {
        ProfScope ps(c, KID_ADJ_MISC, s);
        k_energy<R, S><<<nb, BLOCK, 0, s>>>(m, c->phys.gamma, (const S*)ra, (const S*)rua, (const S*)rea,
                                            (const S*)r, (const S*)ru, (const S*)re, c->partials);
        k_energy_finish<<<1, BLOCK, 0, s>>>(c->partials, nb, c->scal + 4);
    }
    cudaError_t e = cudaMemcpyAsync(out, c->scal + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "afvm_adjoint_energy");
    return AFVM_OK;
}

}  // namespace afvm

using namespace afvm;

extern "C" int afvm_adjoint_energy(afvm_ctx* ctx, const void* rhoa, const void* rhoUa, const void* rhoEa,
                                   const void* rho, const void* rhoU, const void* rhoE, double* out, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rhoa || !rhoUa || !rhoEa || !rho || !rhoU || !rhoE || !out) return fail(c, AFVM_ERR_BAD_ARG, "null pointer");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c->device) cudaSetDevice(c->device);
    int st = (c->precision == AFVM_FP64)
                 ? energy_dev<double, double>(c, rhoa, rhoUa, rhoEa, rho, rhoU, rhoE, out, (cudaStream_t)stream)
                 : (c->precision == AFVM_FP32)
                       ? energy_dev<float, float>(c, rhoa, rhoUa, rhoEa, rho, rhoU, rhoE, out, (cudaStream_t)stream)
                       : energy_dev<float, double>(c, rhoa, rhoUa, rhoEa, rho, rhoU, rhoE, out, (cudaStream_t)stream);
    if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return st;
}
