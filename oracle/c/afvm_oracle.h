/*
 * Mesh, boundary and physics tables of the C oracle (TEST INFRASTRUCTURE ONLY), shared by the
 * C99 primal restatement (oracle/c/afvm_oracle.c) and the host adjoint baseline
 * (oracle/c/adjoint_host.cpp). Built by oracle/c_ref.py.
 */
#ifndef AFVM_ORACLE_H
#define AFVM_ORACLE_H
#include <stddef.h>
#include <stdint.h>

enum { K_COPY = 0, K_FIXED = 1, K_SYM = 2, K_TOTALPT = 3 };
enum { F_INTERNAL = 0, F_COUPLED = 1, F_CHAR = 2, F_BOUNDARY = 3 };

typedef struct {
    int nIC, nIF, nF, nG;
    const int32_t *own, *nbr;                      /* nF */
    const double *nrm, *area, *dlt, *du, *lw, *qw; /* AoS as the reference: nrm nF x 3 ... qw nF x 6 */
    const double *wts;                             /* weights nF */
    const double *vol;                             /* nIC */
    const int32_t *cellFaces, *cellNbr, *cellOwn;  /* nIC x 6 */
    const uint8_t *fkind;                          /* nG: face kind of each boundary face */
    const int32_t *gsrc, *gkind;                   /* nG */
    const double *gval;                            /* nG x 5 fixed U T p */
    const int32_t *accf;                           /* nIC x 6: face (owner side) or ~face */
    double gamma, Cp, Pr;
    int muModel; double mu0, muAs, muTs;
    int riemann, briemann;
    int objective, objStart, objN;                 /* 0 none 1 KE 2 drag 3 sumT 4 vane */
    /* turbine-vane objective (adFVM/objectives/vane.py:7-60, 118-131) */
    int nPlane; const int32_t* planeCells; const double* planeAreas;
    double vn[3], ptin, Tw, va, vb;
    int nHeat; const int32_t* heatFaces; const double* heatW; /* faces of the heat patches, weights */
} oracle_mesh;

#ifdef __cplusplus
extern "C" {
#endif
void oracle_step(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double dt,
                 const double* S, double* rhoN, double* rUN, double* rEN, double* dtcMax, double* obj,
                 double* work);
size_t oracle_work_doubles(const oracle_mesh* M);
void oracle_records(const oracle_mesh* M, const double* rho, const double* rU, const double* rE, double* work);
double* oracle_work_stage(const oracle_mesh* M, double* work, int k);
#ifdef __cplusplus
}
#endif
#endif
