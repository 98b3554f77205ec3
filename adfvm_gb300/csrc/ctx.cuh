// Device context: mesh tables, boundary conditions and work buffers of one solver on one GPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "afvm.h"
#include "physics.cuh"

namespace afvm {

constexpr int BLOCK = 256;
// the face kernels hold 160-240 registers a thread in FP64: 128-thread blocks capped to three
// per SM (12 warps, a few registers spilled to L1 in the VJP) keep more FP64 instructions in
// flight than one 256-thread block (8 warps); in FP32 the forward flux is capped at 64
// registers (32 warps) and the VJP at five blocks (96 registers, 20 warps). Measured at 128^3:
// FP64 k_flux 5.47 -> 4.93 ms, k_adj_flux 11.08 -> 10.52 ms (untaped), FP32 k_flux 0.240 ->
// 0.217 ms, FP32 k_adj_flux 0.471 (4 blocks) -> 0.445 (5) / 0.456 ms (6).
constexpr int FLUX_BLOCK = 128;

// Block-staged record stores. A thread that stores its own W-value record at a W-value stride
// makes each scalar store a separate L2 write request into a partly written sector; instead
// each thread writes its record into the block's shared-memory stage (stage_row: 16-byte
// stores, rows of W values unpadded - W a multiple of 16 bytes, so a quarter-warp's 16-byte
// stores land in distinct banks for W = 20 floats and in two for W = 40), and after a
// __syncthreads() the block's records - one contiguous range of the output - are copied out
// as 16-byte vectors (store_staged).
template <typename T>
struct Vec16;
template <>
struct Vec16<float> { using type = float4; };
template <>
struct Vec16<double> { using type = double2; };

template <typename T, int W>
__device__ __forceinline__ void stage_row(T* __restrict__ row, const T* v) {
    using V = typename Vec16<T>::type;
    constexpr int PER = 16 / sizeof(T);
    static_assert(W % PER == 0, "record rows are whole 16-byte vectors");
#pragma unroll
    for (int j = 0; j < W / PER; j++) {
        V x;
        if constexpr (PER == 4) x = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        else x = make_double2(v[2 * j], v[2 * j + 1]);
        reinterpret_cast<V*>(row)[j] = x;
    }
}

template <typename T, int W, int NT>
__device__ __forceinline__ void store_staged(T* __restrict__ out, size_t first, int nValid,
                                             const T* __restrict__ stage) {
    using V = typename Vec16<T>::type;
    constexpr int PER = 16 / sizeof(T);
    const V* s = reinterpret_cast<const V*>(stage);
    V* o = reinterpret_cast<V*>(out + first * W);
    const int n = nValid * (W / PER);
    for (int i = threadIdx.x; i < n; i += NT) o[i] = s[i];
}

// boundary-condition kind codes stored per ghost cell (3 bits per field: U, T, p)
constexpr int GK_COPY = 0;     // zeroGradient / empty / cyclic: value of the source cell
constexpr int GK_FIXED = 1;    // fixedValue or CBC_UPT: stored value
constexpr int GK_SYM = 2;      // symmetryPlane: U minus its normal component
constexpr int GK_TOTALPT = 3;  // CBC_TOTAL_PT: U, T, p from the source cell and (direction, Tt, pt)

template <typename R>
struct MeshDev {
    int nIC, nIF, nF, nC, nG;
    // faces
    const int32_t* own;       // nF
    const int32_t* nbr;       // nF (ghost ids for boundary faces)
    const R* nrm;             // 3 x nF (SoA)
    const R* area;            // nF
    const R* dlt;             // nF  deltas
    const R* rdlt;            // nF  1/deltas (the viscous snGrad divisor, mesh-only)
    const R* ntd;             // 4 x nF  N - (N.D) D (3) and N.D, D = deltasUnit (mesh-only; FP64 only)
    const R* du;              // 3 x nF deltasUnit
    const R* wts;             // nF  weights (central interpolation, interp.py:15-18)
    const R* lw;              // 2 x nF linearWeights
    const R* qw;              // 6 x nF quadraticWeights (side0 xyz, side1 xyz)
    const uint8_t* fkind;     // nF - nIF: FACE_* of each boundary face
    const int32_t* gsrc;      // nG: source cell of a ghost (owner, or partner owner for cyclic)
    const int32_t* gkind;     // nG: 3-bit BC codes U | T<<3 | p<<6
    const R* gval;            // 5 x nG fixed U, T, p (fixedValue / CBC_UPT)
    // cells: gradient gather slots (cellFaces order), 6 x nIC each
    const int32_t* gnb;       // cellNeighbours
    const R* gw;              // w' = w + O - 2 w O
    const R* gsn;             // 3 x 6 x nIC: S * (2 N O - N)
    const R* rvol;            // nIC 1/V
    // cells: flux accumulation in collate order, 6 x nIC
    const int32_t* accf;      // face id, or ~face id on the neighbour side
    const R* accw;            // A/V_L (owner side) or A/V_R (neighbour side)
    const R* vol;             // nIC
    // adjoint tables
    const R* wpf;             // nF  A/V_L per face
    const R* wnf;             // nIF A/V_R per internal face
    const R* gwb;             // 6 x nIC: w' of the neighbour's slot that points back at this cell
    const R* gA;              // 3 x nIC: sum over the slots of (1 - w') S N
    // the gradient's mesh-only products, 1/V folded in: grad phi_c = phi_c gAv + sum_s phi_nb gws_s
    const R* gws;             // 3 x 6 x nIC: w' S N' / V
    const R* gAv;             // 3 x nIC: gA / V
    const R* gbs;             // 3 x 6 x nIC: -gwb S N' / V_nb (internal neighbours; 0 for ghosts)
    // 3 x nIC: sum over the cell's faces of S N' / V (= sum of A/V N, outward): zero for a cell
    // whose face area vectors close, not for cells with warped faces, whose normals come from
    // three of their points; in the record type and in double (the FP32 gauge terms)
    const R* gcl;
    const double* gclD;
    const int32_t* gsStart;   // nIC + 1: ghosts whose source is the cell, CSR offsets
    const int32_t* gsList;    // nG ghost ids ordered by source cell
    const int32_t* gslot;     // nG: slot of the ghost's face in its owner's cellFaces
};

// kernel ids for the optional per-launch event timing (afvm_profile_*)
enum KernelId { KID_PRIM = 0, KID_GRAD, KID_FLUX, KID_UPDATE, KID_OBJECTIVE, KID_FINISH, KID_ADJ_FLUX,
                KID_ADJ_GATHER, KID_ADJ_GRAD, KID_ADJ_PRIM, KID_ADJ_MISC, KID_SENS, KID_ADJ_VISC, KID_COUNT };
extern const char* const kKernelNames[KID_COUNT];

struct ProfEntry {
    int id;
    cudaEvent_t a, b;
};

// device view of the turbine-vane objective (AFVM_OBJ_VANE)
struct VaneDev {
    const int32_t* planeCells;   // nPlane internal cells cut by the plane
    const double* planeArea;     // nPlane cut areas
    const int32_t* cellPlane;    // nIC: index into the plane arrays, or -1
    const int32_t* heatFaces;    // nHeat boundary faces of the heat-transfer patches
    const double* heatCoef;      // nHeat: k A w / delta
    const double* bHeatCoef;     // nG (by boundary face): the same coefficient, 0 elsewhere
    const double* sums;          // [0] sum of pressure-loss terms, [1] sum of rhoUn A, [2] heat sum
    int nPlane, nHeat;
    double n0, n1, n2, ptin, Tw, a, b, rw2;   // rw2 = 1 / sum_f A_f w_f
};

struct Ctx {
    int precision;            // AFVM_FP64 / AFVM_FP32
    int device;
    std::string err;
    Phys phys;
    int objective, objPatch;
    int objStart, objN;       // face range of the objective patch
    int nIC, nIF, nF, nC, nG, nPatches;
    int nBoundaryFlux = 0;    // faces with FACE_BOUNDARY (the physical boundary flux)
    std::vector<int> patchStart, patchN, patchKind, patchCellStart;
    // device allocations
    std::vector<void*> allocs;
    int64_t bytes = 0;
    MeshDev<double> m64;
    MeshDev<float> m32;
    // work buffers (element type by precision)
    void* rec = nullptr;      // nC x REC
    void* fflux = nullptr;    // nF x FREC
    void* u1[3] = {nullptr, nullptr, nullptr};   // stage states rho, rhoU, rhoE
    void* u2[3] = {nullptr, nullptr, nullptr};
    void* zeroS = nullptr;    // nIC x 5 zeros (absent sources)
    double* partials = nullptr;   // reduction scratch (block partial sums)
    int nPartials = 0;
    double* scal = nullptr;   // device scalars: [0] dtc (stage 1 max), [1] obj, [2] dt, [3] sensitivity
    unsigned long long* dtcBits = nullptr;
    // ghost BC values on the host for updates
    std::vector<int> ghostPatchOffset;   // first ghost index of each patch (sorted order)
    std::vector<int> bcKinds;            // per patch: U,T,p kinds
    std::vector<char> patchDirNormals;   // per patch: a CBC_TOTAL_PT direction taken from the normals
    uint8_t* gdirn = nullptr;            // per ghost, the same flag (device; on first use)
    // adjoint buffers (allocated on first use)
    void* fadj = nullptr;     // nF x 40 face adjoint records
    void* cbar = nullptr;     // nIC x 20 cell primitive/gradient adjoints
    void* a1[3] = {nullptr, nullptr, nullptr};
    void* a2[3] = {nullptr, nullptr, nullptr};
    void* sbar = nullptr;     // 5 x nIC source adjoint scratch (component-major)
    int64_t adjBytes = 0;
    // device staging of the host-buffer entry point (allocated on first use)
    void* stageDev = nullptr;
    // sensitivity reduction scratch (grown on demand)
    void* sensScratch = nullptr;
    size_t sensBytes = 0;
    // an objective evaluated outside the library (afvm_set_objective_sink / _seed): the device
    // buffer that receives each primal step's objective-stage primitives (nC x 5, record type),
    // and the gradient of the objective with respect to them (nC x 5 double) the adjoint adds
    void* objSink = nullptr;
    const double* objSeed = nullptr;
    // turbine-vane objective inputs (afvm_set_objective_vane)
    bool vaneSet = false;
    VaneDev vane{};
    double* vanePartials = nullptr;   // 3 x nVaneBlocks
    int nVaneBlocks = 0;
    double* vaneSums = nullptr;       // 3 doubles
    // adjoint stabilisation work (allocated on first use) and the total volume
    double* viscWork = nullptr;
    double volTotal = 0.0;
    // per-launch event timing
    bool prof = false;
    std::vector<ProfEntry> profEntries;
    std::vector<cudaEvent_t> eventPool;
};

// Event pair around one kernel launch when timing is on (no effect otherwise).
struct ProfScope {
    Ctx* c;
    cudaStream_t s;
    ProfEntry e;
    bool on;
    ProfScope(Ctx* c_, int id, cudaStream_t s_);
    ~ProfScope();
};

int fail(Ctx* c, int code, const std::string& msg);
int cuda_fail(Ctx* c, cudaError_t e, const char* what);
// device allocation owned by the context (freed by afvm_ctx_destroy)
int ctx_alloc(Ctx* c, void** p, size_t bytes);
template <typename R, typename S = R>
int adjoint_viscosity_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, int kind, double scaling, double dt,
                          S* ar, S* au, S* ae, double* Mout, double* DTout, int* iters, cudaStream_t s);

// kernel launchers (primal.cu). R: the record/flux type (double or float); S: the state type
// (R, or double under FP32 fluxes with an FP64 state). dt: by value, or read on the device from
// dtDev when that is non-NULL
template <typename R, typename S = R>
int primal_step_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, double dt, const double* dtDev,
                    const S* Srho, const S* SrhoU, const S* SrhoE, S* rhoN, S* rhoUN, S* rhoEN,
                    double* dtcDev, double* objDev, cudaStream_t s, S* stages = nullptr, R* tape = nullptr);
template <typename R, typename S = R>
int primal_run_dev(Ctx* c, S* rho, S* rhoU, S* rhoE, int nSteps, double dt0, double CFL, double stepFactor,
                   int fixed, const S* Srho, const S* SrhoU, const S* SrhoE, double* dtHist, double* dtcHist,
                   double* objHist, cudaStream_t s);
int sensitivity_dev(Ctx* c, int nArrays, const double* const* grad, const double* const* pert,
                    const int64_t* n, double* out, cudaStream_t s);
// the parameter gradients of an adjoint step (adjoint_params.cu): the mesh tensors in the
// reference's layouts (any may be NULL) and one boundary input, all double, device
struct ParamDev {
    double* areas;       // nF
    double* volL;        // nF
    double* volR;        // nIF
    double* wts;         // nF
    double* dlt;         // nF
    double* nrm;         // nF x 3
    double* du;          // nF x 3
    double* lw;          // nF x 2
    double* qw;          // nF x 2 x 3
    double* vol;         // nIC
    int bcStart, bcN, bcField;   // faces of the boundary input's patch (bcN 0: none), U/T/p
    double* bc;          // bcN x (3 for U, else 1)
    const uint8_t* gdirn;
};
template <typename R, typename S = R>
int adjoint_step_dev(Ctx* c, const S* rho, const S* rhoU, const S* rhoE, double dt,
                     const S* Srho, const S* SrhoU, const S* SrhoE,
                     const S* rhoNa, const S* rhoUNa, const S* rhoENa, double obja,
                     S* rhoa, S* rhoUa, S* rhoEa, S* Srhoa, S* SrhoUa, S* SrhoEa, cudaStream_t s,
                     const S* stages = nullptr, const R* tape = nullptr, const ParamDev* params = nullptr);
// per stage of the reverse sweep, after the face records and cell sums of the stage (fadj,
// cbar) and before the stage's cell kernel: adds the stage's share of the parameter gradients
template <typename R, typename S>
void launch_param_grads(Ctx* c, const ParamDev& pd, const R* rec, R coef, const S* ar, const S* au, const S* ae,
                        bool objectiveStage, double obja, cudaStream_t s);

// a step's tape, written by the primal step and read by its adjoint step: in FP64 first the
// face tapes, one per RK stage, TAPE values a face each (value k of face f of stage st at
// [(st TAPE + k) nF + f]); then, in every precision, the three stages' cell records (REC values
// a cell, nCells rows each), which spare the adjoint its primitive and gradient launches
inline size_t face_tape_elements(const Ctx* c);
inline size_t tape_elements(const Ctx* c);
template <typename R>
inline void split_tape(const Ctx* c, R* tape, R*& face, R*& recs);

// the RK stage states u1, u2 of one step in a caller's buffer of 10 nIC values:
// u1 = [rho (n) | rhoU (3n) | rhoE (n)], then u2 in the same layout
template <typename R, typename P>
inline void stage_views(P* stages, int n, P** u1, P** u2) {
    u1[0] = stages; u1[1] = stages + n; u1[2] = stages + 4 * (size_t)n;
    u2[0] = stages + 5 * (size_t)n; u2[1] = stages + 6 * (size_t)n; u2[2] = stages + 9 * (size_t)n;
}

// turbine-vane objective partial sums of the stage-1 record now in c->rec into c->vaneSums
// rec: the cell records to read/write (NULL: the context's)
template <typename R>
void launch_vane_sums(Ctx* c, cudaStream_t s, double* dtcOut, double* objOut, const R* rec = nullptr);
template <typename R, typename S = R>
void launch_prim(Ctx* c, const S* r, const S* ru, const S* re, cudaStream_t s, R* rec = nullptr);
template <typename R, typename S = R>
void launch_prim_grad(Ctx* c, const S* r, const S* ru, const S* re, cudaStream_t s, R* rec = nullptr);
// nextPrims: the update also writes the primitives of the state it produces into the cell
// records (the next stage's k_prim, fused)
// tape: the stage's face tape to write (NULL: none)
template <typename R, typename S = R>
void launch_flux_update(Ctx* c, int st, double dt, const double* dtDev, const S* const* u0, const S* const* u1,
                        const S* const* u2, const S* Sr, const S* Su, const S* Se, S* const* out, cudaStream_t s,
                        bool nextPrims = false, R* tape = nullptr, R* recIn = nullptr, R* recOut = nullptr,
                        double* objPartials = nullptr);
template <typename S>
void default_sources(Ctx* c, const S*& Srho, const S*& SrhoU, const S*& SrhoE);
// count values between host memory of any kind and the device (element sizes 4 or 8, converted
// when they differ; hostcopy.cu). toDevice: returns once src has been read. Otherwise returns
// once dst holds the values, except for a pinned dst of the same type with syncPinned false
// (then the copy is only queued on the stream).
int host_copy(int32_t device, void* dst, int32_t dstBytes, const void* src, int32_t srcBytes, int64_t count,
              void* stream, bool toDevice, bool syncPinned);
static inline int nblocks(long long n) { return (int)((n + BLOCK - 1) / BLOCK); }

// rows of U (3), T, p with absolute T and p from FP32 records (stride values apart), which
// hold the gauge offsets of T and p
void launch_abs_prims(const Ctx* c, const float* rec, int stride, int n, float* out, cudaStream_t s);

template <typename R> inline const MeshDev<R>& meshOf(const Ctx* c);
template <> inline const MeshDev<double>& meshOf<double>(const Ctx* c) { return c->m64; }
template <> inline const MeshDev<float>& meshOf<float>(const Ctx* c) { return c->m32; }

// the three stages' face tapes, padded to a multiple of four values: the cell records that
// follow them are read with 16-byte vector loads, and 3 TAPE nF values (TAPE odd, nF odd)
// would leave them on an 8-byte boundary
inline size_t face_tape_elements(const Ctx* c) {
    if (c->precision != AFVM_FP64) return 0;
    return ((size_t)3 * TAPE * (size_t)c->nF + 3) & ~(size_t)3;
}
inline size_t tape_elements(const Ctx* c) { return face_tape_elements(c) + (size_t)3 * REC * (size_t)c->nC; }
template <typename R>
inline void split_tape(const Ctx* c, R* tape, R*& face, R*& recs) {
    face = nullptr;
    recs = nullptr;
    if (!tape) return;
    size_t nface = face_tape_elements(c);
    face = nface ? tape : nullptr;
    recs = tape + nface;
}

}  // namespace afvm
