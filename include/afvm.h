/*
 * afvm.h - C ABI of the GB300 compressible finite-volume residual and its discrete adjoint.
 *
 * Plain pointers and sizes only. Every call returns an AFVM_* status code and never aborts
 * the process; afvm_last_error() gives the message of the last failing call on a context.
 *
 * The entry points replace, for one GPU, the compiled functions that the reference solver
 * builds and calls inside its time loops:
 *   afvm_mesh_build       <- cmesh.build / cmesh.buildBeforeWrite  (adFVM/cpp/cmesh.cpp:3-270,
 *                            ghost cells adFVM/mesh.py:758-819)
 *   afvm_ctx_create       <- Function.initialize -> external_init   (adFVM/solver.py:61-71,
 *                            adFVM/cpp/external.cpp:21-42)
 *   afvm_ctx_destroy      <- external_exit                          (adFVM/cpp/external.cpp:44-51)
 *   afvm_primal_step      <- RCF.map(*inputs)                       (adFVM/solver.py:312-323,
 *                            graph built at adFVM/density.py:80-105)
 *   afvm_adjoint_step     <- Adjoint.map(*inputs)                   (apps/adjoint.py:268-291,
 *                            graph built at apps/adjoint.py:94-151)
 *   afvm_sensitivity      <- cmesh.computeSensitivity               (adFVM/cpp/cmesh.cpp:309-340)
 */
#ifndef AFVM_H
#define AFVM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define AFVM_OK              0
#define AFVM_ERR_BAD_ARG     1   /* invalid size, pointer, index or option               */
#define AFVM_ERR_OOM         2   /* device allocation failed                              */
#define AFVM_ERR_NONFINITE   3   /* a NaN/Inf appeared in a result (reference: MPI.Abort) */
#define AFVM_ERR_TIMEOUT     4   /* a bounded device-side wait gave up                    */
#define AFVM_ERR_CUDA        5   /* a CUDA runtime call failed                            */
#define AFVM_ERR_UNSUPPORTED 6   /* valid input outside what this library implements      */

/* ---- precision of a context ---- */
#define AFVM_FP64 0              /* all arithmetic and storage in double                  */
#define AFVM_FP32 1              /* float storage/flux/gradient; double for the pressure
                                    recovery, the objective and the sensitivity sums       */
#define AFVM_FP32_STATE64 2      /* AFVM_FP32's float mesh tables, cell records, face
                                    fluxes and face arithmetic, with the conservative
                                    state, RK stages, sources and adjoints in double: the
                                    RK update and its reverse accumulate in double          */

/* ---- mesh patch kinds (the 'type' entry of a polyMesh boundary patch) ---- */
#define AFVM_PATCH_PLAIN     0   /* patch / wall / empty / symmetryPlane                  */
#define AFVM_PATCH_CYCLIC    1   /* cyclic pair; neighbourPatch names the partner         */
#define AFVM_PATCH_PROCESSOR 2   /* processor halo: not supported on one GPU              */

typedef struct afvm_patch {
    int32_t startFace;
    int32_t nFaces;
    int32_t kind;            /* AFVM_PATCH_* */
    int32_t neighbourPatch;  /* index of the cyclic partner in the same table, else -1 */
} afvm_patch;

/* ---- mesh build (host) ---- */
typedef struct afvm_mesh_in {
    int32_t nPoints;
    const double* points;        /* nPoints x 3 */
    int32_t nFaces;
    const int32_t* faces;        /* nFaces x 5: count (4) + point ids */
    int32_t nInternalFaces;
    const int32_t* owner;        /* nFaces */
    const int32_t* neighbour;    /* nInternalFaces */
    int32_t nInternalCells;
    int32_t nPatches;
    const afvm_patch* patches;   /* any order; used for ghost cells */
} afvm_mesh_in;

typedef struct afvm_mesh_out {   /* all buffers caller-allocated */
    double* normals;             /* nFaces x 3 */
    double* faceCentres;         /* nFaces x 3 */
    double* areas;               /* nFaces */
    double* cellCentres;         /* nCells x 3 (ghost rows included) */
    double* volumes;             /* nInternalCells */
    int32_t* neighbour;          /* nFaces (ghost cell ids appended for boundary faces) */
    double* deltas;              /* nFaces */
    double* deltasUnit;          /* nFaces x 3 */
    double* weights;             /* nFaces */
    double* linearWeights;       /* nFaces x 2 */
    double* quadraticWeights;    /* nFaces x 2 x 3 */
    int32_t* cellFaces;          /* nInternalCells x 6 */
    int32_t* cellOwner;          /* nInternalCells x 6 */
    int32_t* cellNeighbours;     /* nInternalCells x 6 (ghost ids included) */
    int32_t* cellNeighboursMatOp;/* nInternalCells x 6 (-1 for boundary), may be NULL */
    int32_t nLocalCells;         /* written */
} afvm_mesh_out;

/* Geometry and connectivity of a hex mesh (host, OpenMP). Replaces cmesh.build /
 * cmesh.buildBeforeWrite (adFVM/cpp/cmesh.cpp:3-270) and Mesh.createGhostCells for one
 * rank (adFVM/mesh.py:758-819). */
int afvm_mesh_build(const afvm_mesh_in* in, afvm_mesh_out* out);

/* The same build on the GPU (one thread per face or cell), bitwise equal to afvm_mesh_build:
 * in->points, faces, owner, neighbour and every array of out are DEVICE pointers; in->patches
 * is a host array. Runs on stream and returns when the build is complete. Replaces the same
 * reference functions as afvm_mesh_build. */
int afvm_mesh_build_device(const afvm_mesh_in* in, afvm_mesh_out* out, void* stream);

/* Bandwidth renumbering of a hex mesh's cells on the GPU, for meshes admitted in any cell
 * order: reverse Cuthill-McKee over the cell graph (edges: internal faces and cyclic patch
 * face pairs), each component started from the cell of least (degree, id), neighbours
 * appended in increasing (degree, id), new id = nInternalCells - 1 - position; the highest
 * id then goes to a cell owning a boundary face (the reader's cell count is max(owner) + 1,
 * adFVM/mesh.py:521). Internal faces take the new ids, a face whose new owner id exceeds its
 * new neighbour id is flipped (ids swapped, points listed p2 p1 p0 p3 so that the normal of
 * adFVM/cpp/cmesh.cpp:72-87 is exactly negated), and internal faces are ordered by (owner,
 * neighbour, old face); boundary faces keep their places. No reference counterpart (the
 * reference takes meshes in file order, adFVM/mesh.py:84-127).
 * in->faces, owner, neighbour: DEVICE (points unused); in->patches: host. Outputs, DEVICE,
 * caller-allocated: facesOut (nFaces x 5), ownerOut (nFaces), neighbourOut (nInternalFaces),
 * cellNew (nInternalCells: new id of each old cell), faceOld (nFaces: old face of each new
 * face, ~old where flipped). bandwidth (host, may be NULL): max |id difference| over the
 * graph's edges before and after. Returns when done. AFVM_ERR_BAD_ARG for an index out of
 * range, a face between a cell and itself or a cell without faces, AFVM_ERR_UNSUPPORTED for a cell with more than six graph edges or processor
 * patches. */
int afvm_mesh_reorder_device(const afvm_mesh_in* in, int32_t* facesOut, int32_t* ownerOut,
                             int32_t* neighbourOut, int32_t* cellNew, int32_t* faceOld,
                             int32_t* bandwidth, void* stream);

/* ---- solver context ---- */

/* The mesh tensors in the order of Mesh.getTensor() (adFVM/mesh.py:27-32, 870-872) and
 * the constants of Mesh.getScalar() (adFVM/mesh.py:36-37, 874-881). Host pointers; they are
 * copied to the device once, at context creation. */
typedef struct afvm_mesh_tensors {
    const double* areas;            /* nFaces */
    const double* volumesL;         /* nFaces */
    const double* volumesR;         /* nInternalFaces */
    const double* weights;          /* nFaces */
    const double* deltas;           /* nFaces; each in [1e-30, 1e30] (else AFVM_ERR_BAD_ARG) */
    const double* normals;          /* nFaces x 3 */
    const double* deltasUnit;       /* nFaces x 3 */
    const double* linearWeights;    /* nFaces x 2 */
    const double* quadraticWeights; /* nFaces x 2 x 3 */
    const double* volumes;          /* nInternalCells */
    const int32_t* owner;           /* nFaces */
    const int32_t* neighbour;       /* nFaces */
    const int32_t* cellFaces;       /* nInternalCells x 6 */
    const int32_t* cellNeighbours;  /* nInternalCells x 6 */
    const int32_t* cellOwner;       /* nInternalCells x 6 */
    int32_t nCells, nFaces, nInternalCells, nInternalFaces;
    int32_t nLocalCells, nRemoteCells, nLocalFaces, nGhostCells;
    int32_t nPatches;               /* patches in sortedPatches order (alphabetical) */
    const afvm_patch* patches;      /* kind/neighbourPatch index into this same table */
} afvm_mesh_tensors;

/* boundary conditions of one field on one patch (adFVM/BCs.py) */
#define AFVM_BC_ZERO_GRADIENT  0     /* zeroGradient, empty, inletOutlet  (BCs.py:97-104, 136-137) */
#define AFVM_BC_FIXED_VALUE    1     /* fixedValue                        (BCs.py:111-118)         */
#define AFVM_BC_SYMMETRY_PLANE 2     /* symmetryPlane, slip               (BCs.py:120-135)         */
#define AFVM_BC_CYCLIC         3     /* cyclic                            (BCs.py:86-95)           */
#define AFVM_BC_CBC_UPT        4     /* characteristic U,T,p              (BCs.py:152-161)         */
#define AFVM_BC_CBC_TOTAL_PT   5     /* characteristic total p, T         (BCs.py:164-184)         */

typedef struct afvm_patch_bc {
    int32_t U, T, p;                 /* AFVM_BC_* per field; a CBC kind must be set on all three */
    const double* U_value;           /* nFaces x 3: fixedValue U; U0 (CBC_UPT); direction
                                        (CBC_TOTAL_PT; NULL = the face normals) */
    const double* T_value;           /* nFaces: fixedValue T; T0 (CBC_UPT); Tt (CBC_TOTAL_PT) */
    const double* p_value;           /* nFaces: fixedValue p; p0 (CBC_UPT); pt (CBC_TOTAL_PT) */
} afvm_patch_bc;

#define AFVM_RIEMANN_ROE 0           /* riemann.eulerRoe            (adFVM/riemann.py:21-70) */
#define AFVM_RIEMANN_LF  1           /* riemann.eulerLaxFriedrichs  (adFVM/riemann.py:6-18)  */

#define AFVM_MU_CONSTANT   0         /* mu(T) = mu0                                          */
#define AFVM_MU_SUTHERLAND 1         /* mu(T) = As*T**1.5/(T+Ts) (adFVM/density.py:27)       */

#define AFVM_OBJ_NONE           0    /* obj = 0 (adFVM/density.py:356-357)                    */
#define AFVM_OBJ_KINETIC_ENERGY 1    /* sum_c 0.5*rho*|U|^2*V over internal cells            */
#define AFVM_OBJ_DRAG           2    /* wall drag of templates/cylinder_test.py:9-37          */
#define AFVM_OBJ_SUM_T          3    /* sum_c T (templates/box.py:10-16)                      */
#define AFVM_OBJ_VANE           4    /* plane pressure loss + wall heat transfer, set with
                                        afvm_set_objective_vane (adFVM/objectives/vane.py)     */

typedef struct afvm_physics {
    double gamma, Cp, Pr;            /* defaults 1.4, 1004.5, 0.7 (adFVM/density.py:22-39) */
    int32_t mu_model;                /* AFVM_MU_* */
    double mu0;                      /* constant viscosity */
    double mu_As, mu_Ts;             /* Sutherland constants (1.4792e-06, 116.) */
    int32_t riemann;                 /* AFVM_RIEMANN_* for internal and coupled faces */
    int32_t boundary_riemann;        /* AFVM_RIEMANN_* for characteristic patches */
    int32_t objective;               /* AFVM_OBJ_* evaluated on the stage-1 primitives */
    int32_t objective_patch;         /* patch index (sorted order) for AFVM_OBJ_DRAG */
} afvm_physics;

typedef struct afvm_ctx afvm_ctx;

/* Upload the mesh, boundary conditions and physics; allocate all device work buffers.
 * bcs has mesh->nPatches entries in sortedPatches order. precision is AFVM_FP64, AFVM_FP32 or
 * AFVM_FP32_STATE64. device is a CUDA ordinal. */
int afvm_ctx_create(const afvm_mesh_tensors* mesh, const afvm_patch_bc* bcs,
                    const afvm_physics* physics, int32_t precision, int32_t device,
                    afvm_ctx** out);
int afvm_ctx_destroy(afvm_ctx* ctx);
const char* afvm_last_error(const afvm_ctx* ctx);
int afvm_ctx_precision(const afvm_ctx* ctx);
/* Device bytes held by the context (mesh + work buffers). */
int64_t afvm_ctx_device_bytes(const afvm_ctx* ctx);

/* The gauge state of FP32 cell records (AFVM_FP32 and AFVM_FP32_STATE64 contexts): their
 * records hold p - p_g and T - T_g, and their face fluxes leave out p_g N (momentum) and H_g
 * times the mass flux (energy; added back to the energy residual in the state's type), so that
 * float arithmetic keeps the digits of a low-Mach flow's small pressure and temperature
 * variations. Not part of the reference's arithmetic: results are the same to rounding. The
 * default, set by afvm_ctx_create, is the mean fixed boundary p and T (totals on CBC_TOTAL_PT
 * patches) and the mean Cp T + |U|^2/2 of ghosts with fixed U and T; 0 without such boundary
 * values. p_g and T_g are rounded to floats. Set it before the first step: records, tapes and
 * CUDA graphs made earlier keep the old gauge. FP64 contexts store it and do not use it.
 * afvm_get_gauge writes p_g, T_g, H_g. */
int afvm_set_gauge(afvm_ctx* ctx, double p, double T, double H);
int afvm_get_gauge(const afvm_ctx* ctx, double* pTH);

/* Replace the values of a fixedValue / CBC_UPT boundary input (host pointer, nFaces x dims)
 * - the per-call BC tensors of Solver.getBoundaryTensor (adFVM/solver.py:91-92). field: 0=U,
 * 1=T, 2=p. */
int afvm_set_bc_value(afvm_ctx* ctx, int32_t patch, int32_t field, const double* values);

/* The turbine-vane objective (adFVM/objectives/vane.py:7-140), for a context created with
 * objective AFVM_OBJ_VANE (which must be given these inputs before its first step):
 *   J = a * sum_c (ptin - pt_c) rhoUn_c A_c / ptin / sum_c rhoUn_c A_c
 *     + b * sum_f k (Tw - T_owner) / delta_f A_f w_f / sum_f A_f w_f,   k = Cp mu(Tw) / Pr,
 * over the plane cells c (the reference's getPlane extraArgs, vane.py:23-37) and the faces f of
 * the heat-transfer patches with weights w (getWeights, vane.py:68-80). All arrays are host
 * arrays, copied. */
typedef struct afvm_objective_vane {
    int32_t nPlaneCells;
    const int32_t* planeCells;      /* internal cell ids cut by the plane */
    const double* planeAreas;       /* the cut area of each */
    double normal[3];               /* direction of rho U.n (vane.py: (1, 0, 0)) */
    double ptin;                    /* inlet total pressure (vane.py: 175158) */
    int32_t nHeatPatches;
    const int32_t* heatPatches;     /* patch indices in sortedPatches order */
    const double* const* heatWeights;   /* per heat patch, nFaces weights */
    double Tw;                      /* wall temperature (vane.py: 300) */
    double a, b;                    /* weights of the two terms (vane.py: 0.4, 0) */
} afvm_objective_vane;
int afvm_set_objective_vane(afvm_ctx* ctx, const afvm_objective_vane* v);

/* An objective evaluated by the caller instead of one of the AFVM_OBJ_* kinds: the reference
 * evaluates its case file's objective(fields, solver) on the primitives of the step's second RK
 * stage, ghost cells included (adFVM/density.py:354-357, 412-413). afvm_set_objective_sink: a
 * DEVICE buffer of nCells x 5 values of the record type (double for AFVM_FP64, float otherwise)
 * into which every later primal step copies those primitives, U (3), T, p per cell, internal
 * cells then ghosts (NULL: no copy). afvm_set_objective_seed: the gradient of the caller's
 * objective with respect to the same nCells x 5 values (DEVICE, double), which every later
 * adjoint step adds, times obja, to the adjoint of its objective stage - where the built-in
 * objectives add theirs - and which afvm_adjoint_step_params passes on to the boundary inputs
 * (NULL: none). Both pointers are only recorded: they must stay valid while steps use them. */
int afvm_set_objective_sink(afvm_ctx* ctx, void* prims);
int afvm_set_objective_seed(afvm_ctx* ctx, const double* primBar);

/* Ghost-cell values of the primitive fields for a conservative state: the boundary map the
 * reference runs before writing fields (RCF.initFields -> mapBoundary, adFVM/density.py:140-143;
 * ghost rows per BCs.py:62-184). rho, rhoU, rhoE: DEVICE state as for afvm_primal_step. out:
 * DEVICE buffer of nGhostCells x 5 in the record type (double for AFVM_FP64, float for the
 * other two modes), rows in ghost-cell order (cell id
 * minus nInternalCells), columns U(3), T, p. Asynchronous on stream. */
int afvm_boundary_values(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                         void* out, void* stream);

/* One SSP-RK3 time step (adFVM/timestep.py:27-55 over RCF.equation, density.py:339-414).
 * State arrays are DEVICE pointers in the reference layout: rho (nInternalCells),
 * rhoU (nInternalCells x 3), rhoE (nInternalCells); element type double for AFVM_FP64 and
 * AFVM_FP32_STATE64, float for AFVM_FP32 (the "state type"; every state, source, stage and
 * adjoint array of this interface has it). Sources may be NULL (zero). Outputs may alias
 * the inputs.
 * dtc_out / obj_out (host, may be NULL) receive the stage-1 max CFL sum and objective; a
 * non-NULL one makes the call wait for the step to finish. */
int afvm_primal_step(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                     double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                     void* rhoN, void* rhoUN, void* rhoEN,
                     double* dtc_out, double* obj_out, void* stream);

/* afvm_primal_step that also keeps the step's two intermediate SSP-RK3 stage states in
 * stages (DEVICE, 10 x nInternalCells elements of the state type: u1 then u2, each
 * rho | rhoU | rhoE), at no extra cost - the step writes them anyway. Handing the same buffer
 * to afvm_adjoint_step_stages with the same state, sources and dt lets the adjoint skip its
 * forward recompute of the stages (the reference's reverse mode re-runs the forward,
 * apps/adjoint.py:124-126 over adpy's generated gradient). No reference counterpart. */
int afvm_primal_step_stages(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                            double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                            void* rhoN, void* rhoUN, void* rhoEN, void* stages,
                            double* dtc_out, double* obj_out, void* stream);

/* Same step with HOST buffers (pinned or pageable): copies in, steps, copies out. */
int afvm_primal_step_host(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                          double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                          void* rhoN, void* rhoUN, void* rhoEN,
                          double* dtc_out, double* obj_out, void* stream);

/* nSteps steps resident on the device with the reference's time-step rule
 * dt <- min(2*CFL/dtc, stepFactor*dt, endTime - t) (adFVM/solver.py:365) unless
 * fixed_dt != 0. dt_hist/dtc_hist/obj_hist are DEVICE double arrays of nSteps (may be NULL).
 * The state is advanced in place. No host synchronisation inside. */
int afvm_primal_run(afvm_ctx* ctx, void* rho, void* rhoU, void* rhoE, int32_t nSteps,
                    double dt0, double CFL, double stepFactor, int32_t fixed_dt,
                    const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                    double* dt_hist, double* dtc_hist, double* obj_hist, void* stream);

/* Vector-Jacobian product of one primal step with dt held fixed - the per-step call of the
 * adjoint sweep (apps/adjoint.py:268-291). Inputs: the step's input state (device), dt,
 * sources, the adjoint seeds of the step's outputs (rhoNa, rhoUNa, rhoENa; device) and of
 * its scalar outputs (dtca, obja). Outputs: the adjoint of the input state and, if non-NULL,
 * of the three source arrays. Only dtca == 0 is supported (the reference driver always
 * passes 0, apps/adjoint.py:268). Adjoint outputs may alias the adjoint inputs. */
int afvm_adjoint_step(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                      double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                      const void* rhoNa, const void* rhoUNa, const void* rhoENa,
                      double dtca, double obja,
                      void* rhoa, void* rhoUa, void* rhoEa,
                      void* S_rhoa, void* S_rhoUa, void* S_rhoEa, void* stream);

/* afvm_adjoint_step with the stage states a preceding afvm_primal_step_stages kept for this
 * state (stages != NULL), instead of recomputing them: the outputs are bitwise the same. */
int afvm_adjoint_step_stages(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                             double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                             const void* stages, const void* rhoNa, const void* rhoUNa,
                             const void* rhoENa, double dtca, double obja, void* rhoa, void* rhoUa,
                             void* rhoEa, void* S_rhoa, void* S_rhoUa, void* S_rhoEa, void* stream);

/* The tape of a step: what the primal step computed that its adjoint step would otherwise
 * compute again. In every precision the three RK stages' cell records (20 values a cell:
 * primitives and gradients), which spare the adjoint its primitive and gradient launches; in
 * AFVM_FP64 first also the face tape: per stage and face the 61 values of the forward face
 * flux that its VJP would otherwise re-evaluate (the reconstructed face states, the
 * reciprocals and reciprocal square roots of the Roe / Rusanov flux and of the conservative
 * variables, the normal velocities and sound speeds, mu(T_F) and its derivative, the Roe
 * average and eigenvalue terms, the viscous stress terms), the
 * face VJP being bound by the FP64 pipe there while HBM idles. Element type: the record type
 * (double for AFVM_FP64, float otherwise); afvm_tape_elements values a step (3 x 61 x nFaces,
 * rounded up to a multiple of 4, + 3 x 20 x nCells in FP64; 3 x 20 x nCells otherwise), 16-byte
 * aligned (AFVM_ERR_BAD_ARG otherwise). No reference counterpart (adpy's reverse mode re-runs
 * the forward). */
int64_t afvm_tape_elements(const afvm_ctx* ctx);

/* afvm_primal_step_stages that also writes the step's tape (DEVICE, afvm_tape_elements
 * values; tape needs stages). */
int afvm_primal_step_tape(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                          double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                          void* rhoN, void* rhoUN, void* rhoEN, void* stages, void* tape,
                          double* dtc_out, double* obj_out, void* stream);

/* afvm_adjoint_step_stages that reads the tape the primal step wrote for this state
 * (tape needs stages; NULL: re-evaluate the forward). The result agrees with the re-evaluating
 * step to rounding (the forward kernel may contract products into FMAs differently). */
int afvm_adjoint_step_tape(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                           double dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                           const void* stages, const void* tape, const void* rhoNa,
                           const void* rhoUNa, const void* rhoENa, double dtca, double obja,
                           void* rhoa, void* rhoUa, void* rhoEa, void* S_rhoa, void* S_rhoUa,
                           void* S_rhoEa, void* stream);

/* The adjoint step's gradients with respect to parameters other than the state and the
 * sources - the reference's Adjoint(parameters=...) (apps/adjoint.py:101-126): 'mesh' gives the
 * gradients of the ten Mesh.gradFields tensors (adFVM/mesh.py:28-31) in the reference's own
 * layouts, ('BCs', field, patch, key) the gradient of one boundary input
 * (apps/adjoint.py:111-118). Every pointer is a DEVICE double array that receives the step's
 * gradient (overwritten, summed over the three RK stages); any mesh pointer may be NULL. */
typedef struct afvm_param_grad {
    double* areas;            /* nFaces */
    double* volumesL;         /* nFaces */
    double* volumesR;         /* nInternalFaces */
    double* weights;          /* nFaces */
    double* deltas;           /* nFaces */
    double* normals;          /* nFaces x 3 */
    double* deltasUnit;       /* nFaces x 3 */
    double* linearWeights;    /* nFaces x 2 */
    double* quadraticWeights; /* nFaces x 2 x 3 */
    double* volumes;          /* nInternalCells */
    int32_t bcPatch;          /* boundary input: patch index (sortedPatches order), -1 for none */
    int32_t bcField;          /* the ghost field the input sets: 0 U (fixedValue value, CBC_UPT U0,
                                 CBC_TOTAL_PT direction), 1 T (value, T0, Tt), 2 p (value, p0, pt) */
    double* bc;               /* the patch's nFaces x (3 for field 0, else 1) */
} afvm_param_grad;

/* afvm_adjoint_step_tape that also returns the parameter gradients described by *pg. AFVM_FP64
 * contexts (AFVM_ERR_UNSUPPORTED otherwise, and for the vane objective's heat-transfer term);
 * AFVM_ERR_BAD_ARG for a patch / field without an input (zeroGradient, cyclic, symmetryPlane,
 * or a CBC_TOTAL_PT direction that is the face normals - a mesh input). */
int afvm_adjoint_step_params(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                             const void* S_rho, const void* S_rhoU, const void* S_rhoE, const void* stages,
                             const void* tape, const void* rhoNa, const void* rhoUNa, const void* rhoENa,
                             double dtca, double obja, void* rhoa, void* rhoUa, void* rhoEa, void* S_rhoa,
                             void* S_rhoUa, void* S_rhoEa, const afvm_param_grad* pg, void* stream);

/* FP64 sum over k of dot(grad[k], pert[k]) (adFVM/cpp/cmesh.cpp:309-340). DEVICE arrays of
 * n[k] doubles; result to *out (host) after the stream work completes. */
/* Adjoint stabilisation by artificial viscosity (adFVM/postpro.py:491-718, the viscous
 * adjoint step of apps/adjoint.py:127-139 and 288-289): from the primal state (DEVICE, as
 * afvm_adjoint_step) the per-cell viscosity M = the largest eigenvalue of the symmetrised 5x5
 * of the chosen kind, normalised to scaling * M / sqrt(sum M^2 V / sum V) (computeAdjoint-
 * Viscosity), its central face values DT, and then the implicit heat-equation smoothing of
 * the adjoint fields rhoa, rhoUa, rhoEa (DEVICE, in place; plain gradients of the state) over
 * the time step dt (viscositySolver with scaling.cpp:135-159): per component, x = a / V solves
 * (1 + sum_k c_k) x_c - sum_k c_k x_nbr = a_c / V_c, c_k = dt A_k DT_k / (delta_k V_c), over
 * the faces with an internal neighbour, and a <- V x. Solved by conjugate gradients to a
 * relative residual of 1e-13 (AFVM_ERR_TIMEOUT after 500 iterations). M_out (nCells) and
 * DT_out (nFaces) are optional DEVICE double buffers; iterations_out (host) the CG count. */
#define AFVM_VISC_UNIFORM   1        /* M = 1                                   */
#define AFVM_VISC_TURKEL    2        /* postpro.py:586-602                      */
#define AFVM_VISC_ABARBANEL 3        /* postpro.py:571-585                      */
int afvm_adjoint_viscosity(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE,
                           int32_t kind, double scaling, double dt, void* rhoa, void* rhoUa,
                           void* rhoEa, double* M_out, double* DT_out, int32_t* iterations_out,
                           void* stream);

int afvm_sensitivity(afvm_ctx* ctx, int32_t nArrays, const double* const* grad,
                     const double* const* pert, const int64_t* n, double* out, void* stream);

/* Adjoint energy sum_c w^T A(u) w V with w = adjoint / V (cmesh.computeEnergy,
 * adFVM/cpp/cmesh.cpp:342-425; the reference's adjoint driver reports its square root,
 * apps/adjoint.py:55). DEVICE arrays of the context's state type: the adjoint state
 * (rhoa, rhoUa, rhoEa) and the primal state. FP64 sum to *out (host) after the work. */
int afvm_adjoint_energy(afvm_ctx* ctx, const void* rhoa, const void* rhoUa, const void* rhoEa,
                        const void* rho, const void* rhoU, const void* rhoE, double* out, void* stream);

/* Allocation-free form of afvm_sensitivity. No counterpart in the reference. It is for
 * callers that may not allocate device memory: an application that hands this library a
 * fixed share of the GPU up front and owns every allocation itself, or a plug-in loaded
 * into a host program whose memory pool it must not touch. Such a caller cannot create a
 * context (afvm_ctx_create allocates) and cannot let afvm_sensitivity grow its scratch.
 * It needs no context: the grad/pert arrays live on CUDA device `device`; the scratch is a
 * static device array of the library that holds partial sums for at most
 * AFVM_SENSITIVITY_NOALLOC_MAX_ARRAYS arrays (about 129 KB, kept on every GPU that loads
 * the library until the process exits). nArrays outside 1..that limit, or a device outside
 * the visible ones, or an array that is not memory of that device (or a stream of another
 * device), is rejected with AFVM_ERR_BAD_ARG. The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) with that device current and caches
 * it, so make that first call before any stream capture; the cached address does not
 * survive cudaDeviceReset. Calls share the array: calls that overlap on the GPU race and
 * must be ordered by the caller. Blocks until the result is in *out (host); calls no
 * allocator. */
#define AFVM_SENSITIVITY_NOALLOC_MAX_ARRAYS 16
int afvm_sensitivity_noalloc(int32_t device, int32_t nArrays, const double* const* grad,
                             const double* const* pert, const int64_t* n, double* out, void* stream);

/* ---- field arrays between any host memory and the device ----
 * The reference passes its compiled step numpy arrays (pageable host memory) every call and
 * gets numpy arrays back (adFVM/solver.py:312-323 inputs and outputs of self.map;
 * apps/adjoint.py:268-291 for the adjoint map); these two calls are that transfer. `count`
 * values of srcBytes bytes each (8: double, 4: float) become `count` values of dstBytes bytes,
 * converted (round to nearest) when the sizes differ. Host memory may be pageable or pinned;
 * device arrays live on CUDA device `device`, and the copy is ordered on `stream`.
 * Copies of equal types take the CUDA driver's copy directly (a download into pageable memory first
 * touches the destination's pages with all OpenMP threads, so a new array takes its page faults
 * in parallel); converted data moves through two pinned 8 MB staging chunks per device, filled
 * or drained by all OpenMP threads while the other chunk is on the link; calls on one device
 * are serialised by a lock. afvm_copy_to_device returns once `src` has been read (the device
 * data is ready in stream order); afvm_copy_to_host returns when `dst` holds the values. */
int afvm_copy_to_device(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes,
                        int64_t count, void* stream);
int afvm_copy_to_host(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes,
                      int64_t count, void* stream);

/* ---- per-launch timing (the analogue of the reference's timeFunction decorator and
 * per-step timers, adFVM/config.py:158-168, adFVM/solver.py:322-346) ----
 * afvm_profile(ctx, 1) clears the record and brackets every later kernel launch of the
 * context with a CUDA event pair on the launching stream; afvm_profile_read sums the
 * elapsed milliseconds and launch counts per kernel id (maxKernels >= the number of ids;
 * afvm_profile_kernel_name gives an id's name, NULL past the last one). */
int afvm_profile(afvm_ctx* ctx, int32_t on);
int afvm_profile_read(afvm_ctx* ctx, int32_t maxKernels, double* ms, int64_t* launches);
const char* afvm_profile_kernel_name(int32_t id);

/* Measured fused-multiply-add throughput of a device in TFLOP/s (fp64 != 0: double,
 * else float): the compute ceiling that the FP64 residual kernels meet before the HBM one.
 * No counterpart in the reference (a measurement aid for the roofline). */
int afvm_fma_peak(int32_t device, int32_t fp64, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* AFVM_H */
