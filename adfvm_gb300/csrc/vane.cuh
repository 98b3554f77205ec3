// Per-cell terms of the turbine-vane pressure-loss objective (adFVM/objectives/vane.py:39-60)
// and their derivatives, in FP64 on the stage-1 primitives of one plane cell:
//   rho = p / (Cv T (g-1)), rhoUn = rho U.n, M^2 = |U|^2 / c^2 with c^2 = g p / rho,
//   pt = p (1 + (g-1)/2 M^2)^(g/(g-1)),
//   w_c = rhoUn A (the weighting, objectivePressureLossWeighting), and
//   l_c = (ptin - pt) rhoUn A / ptin (the summand of objectivePressureLoss before / w).
#pragma once
#include "physics.cuh"
#include "ctx.cuh"

namespace afvm {

AFVM_HD void vane_cell(const Phys& P, const VaneDev& v, const double* U, double T, double p, double A, double& l,
                       double& w) {
    double g = P.gamma;
    double rho = p / (P.Cv * T * (g - 1));
    double rhoUn = rho * U[0] * v.n0 + rho * U[1] * v.n1 + rho * U[2] * v.n2;
    double c2 = g * p / rho;
    double M2 = (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]) / c2;
    double pt = p * pow(1 + 0.5 * (g - 1) * M2, g / (g - 1));
    w = rhoUn * A;
    l = (v.ptin - pt) * rhoUn * A / v.ptin;
}

// gradient of a*L/W (L = sum l_c, W = sum w_c, both given) with respect to U (3), T, p of the
// cell, times s
AFVM_HD void vane_cell_grad(const Phys& P, const VaneDev& v, const double* U, double T, double p, double A,
                            double L, double W, double s, double* g5) {
    double g = P.gamma, kap = g / (g - 1);
    double rho = p / (P.Cv * T * (g - 1));
    double n[3] = {v.n0, v.n1, v.n2};
    double Un = U[0] * n[0] + U[1] * n[1] + U[2] * n[2];
    double rhoUn = rho * Un;
    double q = U[0] * U[0] + U[1] * U[1] + U[2] * U[2];
    double M2 = q * rho / (g * p);
    double X = 1 + 0.5 * (g - 1) * M2;
    double Xk1 = pow(X, kap - 1);
    double pt = p * Xk1 * X;
    double dptdM2 = p * kap * Xk1 * 0.5 * (g - 1);
    double cl = s * v.a / W;                    // d(aL/W)/dl_c
    double cw = -s * v.a * L / (W * W);         // d(aL/W)/dw_c
    double fac = (v.ptin - pt) / v.ptin;        // l_c = fac w_c
    // d/dU: dpt/dU = dptdM2 2 U rho/(g p), drhoUn/dU = rho n
    for (int k = 0; k < 3; k++) {
        double dpt = dptdM2 * 2 * U[k] * rho / (g * p);
        double dr = rho * n[k];
        g5[k] += cl * (-dpt / v.ptin * rhoUn * A + fac * A * dr) + cw * A * dr;
    }
    // d/dT: M2 and rhoUn scale with 1/T
    {
        double dpt = dptdM2 * (-M2 / T);
        double dr = -rhoUn / T;
        g5[3] += cl * (-dpt / v.ptin * rhoUn * A + fac * A * dr) + cw * A * dr;
    }
    // d/dp: M2 does not depend on p (rho/p does not), rhoUn is proportional to p
    {
        double dpt = Xk1 * X;
        double dr = rhoUn / p;
        g5[4] += cl * (-dpt / v.ptin * rhoUn * A + fac * A * dr) + cw * A * dr;
    }
}

}  // namespace afvm
