// C ABI: context life cycle, mesh/BC upload and the step entry points (include/afvm.h).
//
// afvm_ctx_create mirrors the reference's Function.initialize -> external_init
// (adFVM/solver.py:61-71, adFVM/cpp/external.cpp:21-42): the mesh moves to the device once;
// every later call passes only the state. The derived per-cell tables are computed here in
// double with the reference's expressions (op.py:45-63 gradient weights, op.py:12-29 div
// weights, density.py:390-402 accumulation order).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>
#include "ctx.cuh"

namespace afvm {

int fail(Ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(Ctx* c, cudaError_t e, const char* what) {
    return fail(c, AFVM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

const char* const kKernelNames[KID_COUNT] = {"k_prim", "k_grad", "k_flux", "k_update", "k_objective",
                                             "k_finish", "k_adj_flux", "k_adj_gather", "k_adj_grad",
                                             "k_adj_prim", "k_adj_misc", "k_sensitivity", "k_adj_viscosity"};

static cudaEvent_t take_event(Ctx* c) {
    if (!c->eventPool.empty()) {
        cudaEvent_t ev = c->eventPool.back();
        c->eventPool.pop_back();
        return ev;
    }
    cudaEvent_t ev = nullptr;
    cudaEventCreate(&ev);
    return ev;
}

ProfScope::ProfScope(Ctx* c_, int id, cudaStream_t s_) : c(c_), s(s_), on(c_->prof) {
    if (!on) return;
    e.id = id;
    e.a = take_event(c);
    e.b = take_event(c);
    cudaEventRecord(e.a, s);
}

ProfScope::~ProfScope() {
    if (!on) return;
    cudaEventRecord(e.b, s);
    c->profEntries.push_back(e);
}

namespace {

// bounded allocation bookkeeping
int dalloc(Ctx* c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, AFVM_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    c->allocs.push_back(*p);
    c->bytes += (int64_t)bytes;
    return AFVM_OK;
}

}  // namespace

int ctx_alloc(Ctx* c, void** p, size_t bytes) { return dalloc(c, p, bytes); }

namespace {

template <typename T>
int upload(Ctx* c, const T** dst, const std::vector<T>& v) {
    void* p = nullptr;
    int st = dalloc(c, &p, v.size() * sizeof(T));
    if (st) return st;
    cudaError_t e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "mesh upload");
    *dst = (const T*)p;
    return AFVM_OK;
}

struct HostTables {
    // faces
    std::vector<int32_t> own, nbr;
    std::vector<double> nrm, area, dlt, du, lw, qw, wts;
    std::vector<uint8_t> fkind;
    std::vector<int32_t> gsrc, gkind;
    std::vector<double> gval;
    // cells
    std::vector<int32_t> gnb, accf;
    std::vector<double> gw, gsn, rvol, accw, vol;
    // adjoint
    std::vector<double> wpf, wnf, gwb, gA, gws, gAv, gbs, gcl;
    std::vector<int32_t> gsStart, gsList, gslot;
};

template <typename R>
std::vector<R> cast(const std::vector<double>& v) {
    return std::vector<R>(v.begin(), v.end());
}

template <typename R>
int upload_mesh(Ctx* c, const HostTables& h, MeshDev<R>& m) {
    int st;
    m.nIC = c->nIC; m.nIF = c->nIF; m.nF = c->nF; m.nC = c->nC; m.nG = c->nG;
    if ((st = upload(c, &m.own, h.own))) return st;
    if ((st = upload(c, &m.nbr, h.nbr))) return st;
    if ((st = upload(c, &m.nrm, cast<R>(h.nrm)))) return st;
    if ((st = upload(c, &m.area, cast<R>(h.area)))) return st;
    if ((st = upload(c, &m.dlt, cast<R>(h.dlt)))) return st;
    {
        std::vector<double> r(h.dlt.size());
        for (size_t i = 0; i < r.size(); i++) r[i] = 1.0 / h.dlt[i];
        if ((st = upload(c, &m.rdlt, cast<R>(r)))) return st;
    }
    m.ntd = nullptr;
    if constexpr (sizeof(R) == 8) {
        // N - (N.D) D and N.D in double (face_derived() forms the same numbers); FP32 face
        // kernels form them in registers instead (their loads, not their arithmetic, bind them)
        const size_t nF = h.dlt.size();
        std::vector<double> t(4 * nF);
        for (size_t f = 0; f < nF; f++) {
            double N[3] = {h.nrm[f], h.nrm[nF + f], h.nrm[2 * nF + f]};
            double D[3] = {h.du[f], h.du[nF + f], h.du[2 * nF + f]};
            double nd = N[0] * D[0] + N[1] * D[1] + N[2] * D[2];
            for (int k = 0; k < 3; k++) t[k * nF + f] = N[k] - nd * D[k];
            t[3 * nF + f] = nd;
        }
        if ((st = upload(c, &m.ntd, cast<R>(t)))) return st;
    }
    if ((st = upload(c, &m.du, cast<R>(h.du)))) return st;
    if ((st = upload(c, &m.wts, cast<R>(h.wts)))) return st;
    if ((st = upload(c, &m.lw, cast<R>(h.lw)))) return st;
    if ((st = upload(c, &m.qw, cast<R>(h.qw)))) return st;
    if ((st = upload(c, &m.fkind, h.fkind))) return st;
    c->nBoundaryFlux = 0;
    for (uint8_t k : h.fkind) c->nBoundaryFlux += (k == FACE_BOUNDARY);
    if ((st = upload(c, &m.gsrc, h.gsrc))) return st;
    if ((st = upload(c, &m.gkind, h.gkind))) return st;
    if ((st = upload(c, &m.gval, cast<R>(h.gval)))) return st;
    if ((st = upload(c, &m.gnb, h.gnb))) return st;
    if ((st = upload(c, &m.gw, cast<R>(h.gw)))) return st;
    if ((st = upload(c, &m.gsn, cast<R>(h.gsn)))) return st;
    if ((st = upload(c, &m.rvol, cast<R>(h.rvol)))) return st;
    if ((st = upload(c, &m.accf, h.accf))) return st;
    if ((st = upload(c, &m.accw, cast<R>(h.accw)))) return st;
    if ((st = upload(c, &m.vol, cast<R>(h.vol)))) return st;
    if ((st = upload(c, &m.wpf, cast<R>(h.wpf)))) return st;
    if ((st = upload(c, &m.wnf, cast<R>(h.wnf)))) return st;
    if ((st = upload(c, &m.gwb, cast<R>(h.gwb)))) return st;
    if ((st = upload(c, &m.gA, cast<R>(h.gA)))) return st;
    if ((st = upload(c, &m.gws, cast<R>(h.gws)))) return st;
    if ((st = upload(c, &m.gAv, cast<R>(h.gAv)))) return st;
    if ((st = upload(c, &m.gbs, cast<R>(h.gbs)))) return st;
    if ((st = upload(c, &m.gcl, cast<R>(h.gcl)))) return st;
    if ((st = upload(c, &m.gclD, h.gcl))) return st;
    if ((st = upload(c, &m.gsStart, h.gsStart))) return st;
    if ((st = upload(c, &m.gsList, h.gsList))) return st;
    if ((st = upload(c, &m.gslot, h.gslot))) return st;
    return AFVM_OK;
}

int bc_code(int kind, bool isU) {
    switch (kind) {
        case AFVM_BC_ZERO_GRADIENT: return GK_COPY;
        case AFVM_BC_CYCLIC: return GK_COPY;
        case AFVM_BC_SYMMETRY_PLANE: return isU ? GK_SYM : GK_COPY;
        case AFVM_BC_FIXED_VALUE: return GK_FIXED;
        case AFVM_BC_CBC_UPT: return GK_FIXED;
        case AFVM_BC_CBC_TOTAL_PT: return GK_TOTALPT;
        default: return -1;
    }
}

int build_tables(Ctx* c, const afvm_mesh_tensors* M, const afvm_patch_bc* bcs, HostTables& h) {
    const int nIC = M->nInternalCells, nIF = M->nInternalFaces, nF = M->nFaces, nC = M->nCells;
    const int nG = nC - nIC;
    if (nIC <= 0 || nIF < 0 || nF < nIF || nG != nF - nIF)
        return fail(c, AFVM_ERR_BAD_ARG, "inconsistent mesh sizes");
    if (M->nRemoteCells != 0) return fail(c, AFVM_ERR_UNSUPPORTED, "processor patches need a multi-partition run");
    c->nIC = nIC; c->nIF = nIF; c->nF = nF; c->nC = nC; c->nG = nG;
    c->nPatches = M->nPatches;
    // faces
    h.own.assign(M->owner, M->owner + nF);
    h.nbr.assign(M->neighbour, M->neighbour + nF);
    // the per-face and per-cell loops run on all host cores; a failed check sets a code (the
    // smallest index's message is reported)
    int bad = 0;
#pragma omp parallel for reduction(max : bad)
    for (int f = 0; f < nF; f++) {
        int e = 0;
        if (h.own[f] < 0 || h.own[f] >= nIC) e = 1;
        else if (h.nbr[f] < 0 || h.nbr[f] >= nC) e = 2;
        else if (f < nIF && h.nbr[f] >= nIC) e = 3;
        else if (f >= nIF && h.nbr[f] != nIC + (f - nIF)) e = 4;
        bad = std::max(bad, e);
    }
    if (bad) {
        const char* msg[] = {"", "owner out of range", "neighbour out of range", "internal face with a ghost neighbour",
                             "ghost id of a boundary face"};
        return fail(c, AFVM_ERR_BAD_ARG, msg[bad]);
    }
    h.nrm.resize(3 * (size_t)nF); h.du.resize(3 * (size_t)nF);
    h.lw.resize(2 * (size_t)nF); h.qw.resize(6 * (size_t)nF);
    h.area.assign(M->areas, M->areas + nF);
    h.dlt.assign(M->deltas, M->deltas + nF);
    // the viscous snGrad divides by deltas, and the face kernels double 1/deltas by raising its
    // exponent: every deltas must be a positive, finite number of ordinary size (a NaN fails
    // both comparisons)
    int badDelta = 0;
#pragma omp parallel for reduction(max : badDelta)
    for (int f = 0; f < nF; f++)
        if (!(h.dlt[f] >= 1e-30 && h.dlt[f] <= 1e30)) badDelta = 1;
    if (badDelta) return fail(c, AFVM_ERR_BAD_ARG, "deltas must lie in [1e-30, 1e30]");
    h.wts.assign(M->weights, M->weights + nF);
    c->volTotal = 0.0;
    for (int i = 0; i < nIC; i++) c->volTotal += M->volumes[i];
#pragma omp parallel for
    for (int f = 0; f < nF; f++) {
        for (int k = 0; k < 3; k++) {
            h.nrm[(size_t)k * nF + f] = M->normals[3 * (size_t)f + k];
            h.du[(size_t)k * nF + f] = M->deltasUnit[3 * (size_t)f + k];
        }
        for (int k = 0; k < 2; k++) h.lw[(size_t)k * nF + f] = M->linearWeights[2 * (size_t)f + k];
        for (int k = 0; k < 6; k++) h.qw[(size_t)k * nF + f] = M->quadraticWeights[6 * (size_t)f + k];
    }
    // patches (sorted order) -> boundary-face kinds, ghost sources and BC codes
    h.fkind.assign(nG, (uint8_t)FACE_BOUNDARY);
    h.gsrc.assign(nG, -1);
    h.gkind.assign(nG, 0);
    h.gval.assign(5 * (size_t)nG, 0.0);
    std::vector<int> rank(nF);
    std::iota(rank.begin(), rank.end(), 0);
    int pos = nIF;
    c->objStart = 0; c->objN = 0;
    for (int pi = 0; pi < M->nPatches; pi++) {
        const afvm_patch& p = M->patches[pi];
        const afvm_patch_bc& b = bcs[pi];
        if (p.nFaces < 0 || p.startFace < nIF || p.startFace + p.nFaces > nF)
            return fail(c, AFVM_ERR_BAD_ARG, "patch face range");
        if (p.kind == AFVM_PATCH_PROCESSOR) return fail(c, AFVM_ERR_UNSUPPORTED, "processor patch");
        auto isC = [](int k) { return k == AFVM_BC_CBC_UPT || k == AFVM_BC_CBC_TOTAL_PT; };
        bool cbc = isC(b.U) || isC(b.T) || isC(b.p);
        if (cbc && !(b.U == b.T && b.T == b.p))
            return fail(c, AFVM_ERR_BAD_ARG, "a characteristic BC must be set on U, T and p of a patch");
        bool totalpt = b.U == AFVM_BC_CBC_TOTAL_PT;
        bool cyclic = p.kind == AFVM_PATCH_CYCLIC;
        if (cyclic) {
            if (p.neighbourPatch < 0 || p.neighbourPatch >= M->nPatches ||
                M->patches[p.neighbourPatch].nFaces != p.nFaces)
                return fail(c, AFVM_ERR_BAD_ARG, "cyclic partner");
            if (b.U != AFVM_BC_CYCLIC || b.T != AFVM_BC_CYCLIC || b.p != AFVM_BC_CYCLIC)
                return fail(c, AFVM_ERR_BAD_ARG, "a cyclic patch needs cyclic BCs");
        }
        int cU = bc_code(b.U, true), cT = bc_code(b.T, false), cp = bc_code(b.p, false);
        if (cU < 0 || cT < 0 || cp < 0) return fail(c, AFVM_ERR_BAD_ARG, "unknown BC kind");
        for (int i = 0; i < p.nFaces; i++) {
            int f = p.startFace + i, g = f - nIF;
            h.fkind[g] = (uint8_t)(cyclic ? FACE_COUPLED : (cbc ? FACE_CHARACTERISTIC : FACE_BOUNDARY));
            h.gsrc[g] = cyclic ? h.own[M->patches[p.neighbourPatch].startFace + i] : h.own[f];
            h.gkind[g] = cU | (cT << 3) | (cp << 6);
            if (totalpt) {
                if (!b.T_value || !b.p_value) return fail(c, AFVM_ERR_BAD_ARG, "missing Tt or pt");
                for (int k = 0; k < 3; k++)
                    h.gval[(size_t)k * nG + g] = b.U_value ? b.U_value[3 * (size_t)i + k] : M->normals[3 * (size_t)f + k];
                h.gval[3 * (size_t)nG + g] = b.T_value[i];
                h.gval[4 * (size_t)nG + g] = b.p_value[i];
                if (!(b.T_value[i] > 0)) return fail(c, AFVM_ERR_BAD_ARG, "Tt must be positive");
                rank[f] = pos + i;
                continue;
            }
            if (cU == GK_FIXED) {
                if (!b.U_value) return fail(c, AFVM_ERR_BAD_ARG, "missing U value");
                for (int k = 0; k < 3; k++) h.gval[(size_t)k * nG + g] = b.U_value[3 * (size_t)i + k];
            }
            if (cT == GK_FIXED) {
                if (!b.T_value) return fail(c, AFVM_ERR_BAD_ARG, "missing T value");
                h.gval[3 * (size_t)nG + g] = b.T_value[i];
            }
            if (cp == GK_FIXED) {
                if (!b.p_value) return fail(c, AFVM_ERR_BAD_ARG, "missing p value");
                h.gval[4 * (size_t)nG + g] = b.p_value[i];
            }
            rank[f] = pos + i;
        }
        pos += p.nFaces;
        c->patchStart.push_back(p.startFace);
        c->patchN.push_back(p.nFaces);
        c->bcKinds.push_back(b.U); c->bcKinds.push_back(b.T); c->bcKinds.push_back(b.p);
        c->patchDirNormals.push_back(totalpt && !b.U_value ? 1 : 0);
        if (c->objective == AFVM_OBJ_DRAG && pi == c->objPatch) { c->objStart = p.startFace; c->objN = p.nFaces; }
    }
    if (pos != nF) return fail(c, AFVM_ERR_BAD_ARG, "patches do not cover the boundary faces");
    for (int g = 0; g < nG; g++)
        if (h.gsrc[g] < 0) return fail(c, AFVM_ERR_BAD_ARG, "boundary face outside every patch");
    if (c->objective == AFVM_OBJ_DRAG && (c->objPatch < 0 || c->objPatch >= M->nPatches))
        return fail(c, AFVM_ERR_BAD_ARG, "objective patch");

    // cells: gradient slots in cellFaces order (op.py:45-63)
    const size_t n = nIC;
    h.gnb.resize(6 * n); h.gw.resize(6 * n); h.gsn.resize(18 * n);
    h.rvol.resize(n); h.vol.assign(M->volumes, M->volumes + nIC);
    h.accf.resize(6 * n); h.accw.resize(6 * n);
    bad = 0;
#pragma omp parallel for reduction(max : bad)
    for (int ci = 0; ci < nIC; ci++) {
        if (!(M->volumes[ci] > 0)) { bad = std::max(bad, 1); continue; }
        h.rvol[ci] = 1.0 / M->volumes[ci];
        int fs[6] = {-1, -1, -1, -1, -1, -1};
        for (int s = 0; s < 6; s++) {
            int f = M->cellFaces[6 * (size_t)ci + s];
            int O = M->cellOwner[6 * (size_t)ci + s];
            int nb = M->cellNeighbours[6 * (size_t)ci + s];
            if (f < 0 || f >= nF || nb < 0 || nb >= nC || (O != 0 && O != 1)) { bad = std::max(bad, 2); f = -1; break; }
            if ((O == 1) != (h.own[f] == ci)) { bad = std::max(bad, 3); f = -1; break; }
            double Od = (double)O;
            double w = M->weights[f];
            double S = M->areas[f];
            h.gnb[s * n + ci] = nb;
            h.gw[s * n + ci] = (w + Od) - (2 * w) * Od;
            for (int k = 0; k < 3; k++) {
                double Nk = M->normals[3 * (size_t)f + k];
                h.gsn[(3 * s + k) * n + ci] = S * (((2 * Nk) * Od) - Nk);
            }
            fs[s] = f;
        }
        bool okc = true;
        for (int s = 0; s < 6; s++) okc = okc && fs[s] >= 0;
        if (!okc) continue;
        // collate order: internal faces by face id, then patches in sorted order
        std::sort(fs, fs + 6, [&](int a, int b2) { return rank[a] < rank[b2]; });
        for (int s = 0; s < 6; s++) {
            int f = fs[s];
            bool ownerSide = h.own[f] == ci;
            if (!ownerSide && f >= nIF) { bad = std::max(bad, 4); break; }
            h.accf[s * n + ci] = ownerSide ? f : ~f;
            h.accw[s * n + ci] = ownerSide ? M->areas[f] / M->volumesL[f] : M->areas[f] / M->volumesR[f];
        }
    }
    if (bad) {
        const char* msg[] = {"", "non-positive cell volume", "cell connectivity out of range",
                             "cellOwner disagrees with owner", "boundary face not owned by its cell"};
        return fail(c, AFVM_ERR_BAD_ARG, msg[bad]);
    }
    // adjoint tables: face weights, back-slot weights, ghosts grouped by source, ghost slots
    h.wpf.resize(nF); h.wnf.resize(std::max(nIF, 1));
    for (int f = 0; f < nF; f++) h.wpf[f] = M->areas[f] / M->volumesL[f];
    for (int f = 0; f < nIF; f++) h.wnf[f] = M->areas[f] / M->volumesR[f];
    h.gwb.assign(6 * n, 0.0);
    h.gslot.assign(std::max(nG, 1), -1);
#pragma omp parallel for
    for (int ci = 0; ci < nIC; ci++) {
        for (int s = 0; s < 6; s++) {
            int f = M->cellFaces[6 * (size_t)ci + s];
            int nb = M->cellNeighbours[6 * (size_t)ci + s];
            if (nb < nIC) {
                // the slot of f in nb's list has O' = 1 - O: w' = w + O' - 2 w O'
                double w = M->weights[f];
                double Ob = (double)(1 - M->cellOwner[6 * (size_t)ci + s]);
                h.gwb[s * n + ci] = (w + Ob) - (2 * w) * Ob;
            } else {
                h.gslot[nb - nIC] = s;
            }
        }
    }
    for (int g = 0; g < nG; g++)
        if (h.gslot[g] < 0) return fail(c, AFVM_ERR_BAD_ARG, "ghost without a gradient slot");
    // the cell's own share of the gradient transpose, sum_s (1 - w'_s) S N'_s (mesh-only): the
    // adjoint applies it once instead of slot by slot
    h.gA.assign(3 * n, 0.0);
    for (int ci = 0; ci < nIC; ci++)
        for (int k = 0; k < 3; k++) {
            double a = 0.0;
            for (int s = 0; s < 6; s++) a += (1.0 - h.gw[s * n + ci]) * h.gsn[(3 * s + k) * n + ci];
            h.gA[k * n + ci] = a;
        }
    // the same products with 1/V folded in, for the gradient gather and its transpose:
    //   grad phi_c = phi_c gA_c / V_c + sum_s phi_nb(s) w'_s S N'_s / V_c
    // and the neighbour slots' share of the transpose, -gwb_s S N'_s / V_nb(s)
    h.gws.assign(18 * n, 0.0);
    h.gAv.assign(3 * n, 0.0);
    h.gbs.assign(18 * n, 0.0);
    h.gcl.assign(3 * n, 0.0);
#pragma omp parallel for
    for (int ci = 0; ci < nIC; ci++) {
        for (int k = 0; k < 3; k++) {
            h.gAv[k * n + ci] = h.gA[k * n + ci] * h.rvol[ci];
            double a = 0.0;
            for (int s = 0; s < 6; s++) a += h.gsn[(3 * s + k) * n + ci];
            h.gcl[k * n + ci] = a * h.rvol[ci];
        }
        for (int s = 0; s < 6; s++) {
            int nb = h.gnb[s * n + ci];
            for (int k = 0; k < 3; k++) {
                double sn = h.gsn[(3 * s + k) * n + ci];
                h.gws[(3 * s + k) * n + ci] = (h.gw[s * n + ci] * sn) * h.rvol[ci];
                if (nb < nIC) h.gbs[(3 * s + k) * n + ci] = -(h.gwb[s * n + ci] * sn) * h.rvol[nb];
            }
        }
    }
    h.gsStart.assign(nIC + 1, 0);
    for (int g = 0; g < nG; g++) h.gsStart[h.gsrc[g] + 1]++;
    for (int ci = 0; ci < nIC; ci++) h.gsStart[ci + 1] += h.gsStart[ci];
    h.gsList.assign(std::max(nG, 1), 0);
    {
        std::vector<int32_t> fillp(h.gsStart.begin(), h.gsStart.end() - 1);
        for (int g = 0; g < nG; g++) h.gsList[fillp[h.gsrc[g]]++] = g;
    }
    return AFVM_OK;
}

// R: element type of the mesh tables, cell records and face fluxes; S: element type of the
// conservative state, its RK stages, sources and adjoints
template <typename R, typename S>
int alloc_work(Ctx* c) {
    int st;
    if ((st = dalloc(c, &c->rec, sizeof(R) * (size_t)c->nC * REC))) return st;
    if ((st = dalloc(c, &c->fflux, sizeof(R) * (size_t)c->nF * FREC))) return st;
    size_t n = c->nIC;
    size_t dims[3] = {1, 3, 1};
    for (int k = 0; k < 3; k++) {
        if ((st = dalloc(c, &c->u1[k], sizeof(S) * n * dims[k]))) return st;
        if ((st = dalloc(c, &c->u2[k], sizeof(S) * n * dims[k]))) return st;
    }
    if ((st = dalloc(c, &c->zeroS, sizeof(S) * n * 5))) return st;
    cudaMemset(c->zeroS, 0, sizeof(S) * n * 5);
    int np = (int)((std::max(c->nIC, c->nF) + BLOCK - 1) / BLOCK);
    c->nPartials = np;
    if ((st = dalloc(c, (void**)&c->partials, sizeof(double) * (size_t)np))) return st;
    if ((st = dalloc(c, (void**)&c->scal, sizeof(double) * 8))) return st;
    cudaMemset(c->scal, 0, sizeof(double) * 8);
    if ((st = dalloc(c, (void**)&c->dtcBits, sizeof(unsigned long long)))) return st;
    return AFVM_OK;
}

template <typename R, typename S>
int alloc_adjoint(Ctx* c) {
    if (c->fadj) return AFVM_OK;
    int64_t before = c->bytes;
    int st;
    size_t n = c->nIC;
    if ((st = dalloc(c, &c->fadj, sizeof(R) * (size_t)c->nF * 40))) return st;
    if ((st = dalloc(c, &c->cbar, sizeof(R) * n * 20))) return st;
    size_t dims[3] = {1, 3, 1};
    for (int k = 0; k < 3; k++) {
        if ((st = dalloc(c, &c->a1[k], sizeof(S) * n * dims[k]))) return st;
        if ((st = dalloc(c, &c->a2[k], sizeof(S) * n * dims[k]))) return st;
    }
    if ((st = dalloc(c, &c->sbar, sizeof(S) * n * 5))) return st;
    c->adjBytes = c->bytes - before;
    c->bytes = before;
    return AFVM_OK;
}

void release(Ctx* c) {
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    for (auto& e : c->profEntries) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    for (auto ev : c->eventPool) cudaEventDestroy(ev);
    c->profEntries.clear();
    c->eventPool.clear();
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
    if (c->sensScratch) cudaFree(c->sensScratch);
    c->sensScratch = nullptr;
    if (prev >= 0) cudaSetDevice(prev);
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// calls f(R{}, S{}) with the element types of the context's precision mode
template <typename F>
int dispatch(const Ctx* c, F&& f) {
    if (c->precision == AFVM_FP64) return f(double{}, double{});
    if (c->precision == AFVM_FP32) return f(float{}, float{});
    return f(float{}, double{});
}

// bytes of one state value (S) and of one mesh/record value (R)
inline size_t state_size(const Ctx* c) { return c->precision == AFVM_FP32 ? sizeof(float) : sizeof(double); }
inline size_t record_size(const Ctx* c) { return c->precision == AFVM_FP64 ? sizeof(double) : sizeof(float); }

int get_results(Ctx* c, double* dtc_out, double* obj_out, cudaStream_t s) {
    if (!dtc_out && !obj_out) return AFVM_OK;
    double tmp[2];
    cudaError_t e = cudaMemcpyAsync(tmp, c->scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "step results");
    if (dtc_out) *dtc_out = tmp[0];
    if (obj_out) *obj_out = tmp[1];
    if (!std::isfinite(tmp[0]) || !std::isfinite(tmp[1]))
        return fail(c, AFVM_ERR_NONFINITE, "non-finite CFL sum or objective");
    return AFVM_OK;
}

}  // namespace
}  // namespace afvm

namespace afvm {

// The gauge state of FP32 records (Phys): p, T and H rounded to floats, so that the FP32 face
// arithmetic holds exactly the values the records' offsets and the update's energy correction
// use (with float-exact Cp and T, H - Cp T is then exact as well).
static void set_gauge(Phys& P, double p, double T, double H) {
    P.gaugeP = (double)(float)p;
    P.gaugeT = (double)(float)T;
    P.gaugeH = (double)(float)H;
    finish_phys(P);
}

// the default gauge state: the mean fixed boundary pressure and temperature (the totals of
// CBC_TOTAL_PT patches) and the mean of Cp T + |U|^2/2 over the ghosts with fixed U and T (Cp T
// without any); zero where the boundary conditions fix none (a periodic box)
static void derive_gauge(const HostTables& h, Phys& P) {
    const size_t nG = h.gkind.size();
    double sp = 0, sT = 0, sH = 0;
    size_t np = 0, nT = 0, nH = 0;
    for (size_t g = 0; g < nG; g++) {
        int kind = h.gkind[g];
        int kU = kind & 7, kT = (kind >> 3) & 7, kp = (kind >> 6) & 7;
        double T = h.gval[3 * nG + g], p = h.gval[4 * nG + g];
        if (kU == GK_TOTALPT) {
            sT += T; nT++;
            sp += p; np++;
            sH += P.Cp * T; nH++;
            continue;
        }
        if (kT == GK_FIXED) {
            sT += T; nT++;
            if (kU == GK_FIXED) {
                double q = 0;
                for (int k = 0; k < 3; k++) q += h.gval[k * nG + g] * h.gval[k * nG + g];
                sH += P.Cp * T + 0.5 * q; nH++;
            }
        }
        if (kp == GK_FIXED) { sp += p; np++; }
    }
    double gp = np ? sp / np : 0.0, gT = nT ? sT / nT : 0.0;
    set_gauge(P, gp, gT, nH ? sH / nH : P.Cp * gT);
}

}  // namespace afvm

using namespace afvm;

extern "C" {

int afvm_ctx_create(const afvm_mesh_tensors* mesh, const afvm_patch_bc* bcs, const afvm_physics* phys,
                    int32_t precision, int32_t device, afvm_ctx** out) {
    if (!out) return AFVM_ERR_BAD_ARG;
    *out = nullptr;
    if (!mesh || !phys || (mesh->nPatches > 0 && (!bcs || !mesh->patches))) return AFVM_ERR_BAD_ARG;
    if (precision != AFVM_FP64 && precision != AFVM_FP32 && precision != AFVM_FP32_STATE64) return AFVM_ERR_BAD_ARG;
    if (phys->riemann != AFVM_RIEMANN_ROE && phys->riemann != AFVM_RIEMANN_LF) return AFVM_ERR_BAD_ARG;
    if (phys->boundary_riemann != AFVM_RIEMANN_ROE && phys->boundary_riemann != AFVM_RIEMANN_LF)
        return AFVM_ERR_BAD_ARG;
    if (phys->mu_model != AFVM_MU_CONSTANT && phys->mu_model != AFVM_MU_SUTHERLAND) return AFVM_ERR_BAD_ARG;
    if (phys->objective < AFVM_OBJ_NONE || phys->objective > AFVM_OBJ_VANE) return AFVM_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return AFVM_ERR_CUDA;
    }
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return AFVM_ERR_OOM;
    c->precision = precision;
    c->device = device;
    Phys& P = c->phys;
    P.gamma = phys->gamma;
    P.gm1 = phys->gamma - 1;
    P.Cp = phys->Cp;
    P.Cv = phys->Cp / phys->gamma;
    P.rCv = 1. / P.Cv;
    P.kFac = phys->Cp / phys->Pr;
    P.mu0 = phys->mu0;
    P.muAs = phys->mu_As;
    P.muTs = phys->mu_Ts;
    P.small = precision == AFVM_FP64 ? 1e-30 : 1e-9;   // adFVM/config.py:171-178
    P.muModel = phys->mu_model;
    P.riemann = phys->riemann;
    P.briemann = phys->boundary_riemann;
    finish_phys(P);
    c->objective = phys->objective;
    c->objPatch = phys->objective_patch;
    DeviceGuard dg(device);
    HostTables h;
    int st = build_tables(c, mesh, bcs, h);
    if (!st) derive_gauge(h, P);
    if (!st) st = (precision == AFVM_FP64) ? upload_mesh<double>(c, h, c->m64) : upload_mesh<float>(c, h, c->m32);
    if (!st)
        st = dispatch(c, [&](auto r, auto sv) { return alloc_work<decltype(r), decltype(sv)>(c); });
    if (!st) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_fail(c, e, "context set-up");
    }
    if (st) {
        release(c);
        delete c;
        return st;
    }
    *out = reinterpret_cast<afvm_ctx*>(c);
    return AFVM_OK;
}

int afvm_ctx_destroy(afvm_ctx* ctx) {
    if (!ctx) return AFVM_OK;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    release(c);
    delete c;
    return AFVM_OK;
}

const char* afvm_last_error(const afvm_ctx* ctx) {
    if (!ctx) return "null context";
    return reinterpret_cast<const Ctx*>(ctx)->err.c_str();
}

int afvm_profile(afvm_ctx* ctx, int32_t on) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    DeviceGuard dg(c->device);
    for (auto& e : c->profEntries) { c->eventPool.push_back(e.a); c->eventPool.push_back(e.b); }
    c->profEntries.clear();
    c->prof = on != 0;
    return AFVM_OK;
}

int afvm_profile_read(afvm_ctx* ctx, int32_t maxKernels, double* ms, int64_t* launches) {
    if (!ctx || !ms || !launches || maxKernels < KID_COUNT) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    DeviceGuard dg(c->device);
    for (int k = 0; k < KID_COUNT; k++) { ms[k] = 0; launches[k] = 0; }
    for (auto& e : c->profEntries) {
        cudaError_t err = cudaEventSynchronize(e.b);
        if (err != cudaSuccess) return cuda_fail(c, err, "profile read");
        float t = 0;
        cudaEventElapsedTime(&t, e.a, e.b);
        ms[e.id] += t;
        launches[e.id] += 1;
    }
    return AFVM_OK;
}

const char* afvm_profile_kernel_name(int32_t id) {
    return (id >= 0 && id < KID_COUNT) ? kKernelNames[id] : nullptr;
}

int afvm_ctx_precision(const afvm_ctx* ctx) {
    return ctx ? reinterpret_cast<const Ctx*>(ctx)->precision : -1;
}

int64_t afvm_ctx_device_bytes(const afvm_ctx* ctx) {
    if (!ctx) return 0;
    const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
    return c->bytes + c->adjBytes;
}

int afvm_set_objective_sink(afvm_ctx* ctx, void* prims) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    c->objSink = prims;
    return AFVM_OK;
}

int afvm_set_gauge(afvm_ctx* ctx, double p, double T, double H) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!std::isfinite(p) || !std::isfinite(T) || !std::isfinite(H))
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_gauge: the gauge state must be finite");
    set_gauge(c->phys, p, T, H);
    return AFVM_OK;
}

int afvm_get_gauge(const afvm_ctx* ctx, double* pTH) {
    if (!ctx || !pTH) return AFVM_ERR_BAD_ARG;
    const Phys& P = reinterpret_cast<const Ctx*>(ctx)->phys;
    pTH[0] = P.gaugeP; pTH[1] = P.gaugeT; pTH[2] = P.gaugeH;
    return AFVM_OK;
}

int afvm_set_objective_seed(afvm_ctx* ctx, const double* primBar) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    c->objSeed = primBar;
    return AFVM_OK;
}

int afvm_set_objective_vane(afvm_ctx* ctx, const afvm_objective_vane* v) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!v) return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: null description");
    if (c->objective != AFVM_OBJ_VANE) return fail(c, AFVM_ERR_BAD_ARG, "the context's objective is not AFVM_OBJ_VANE");
    if (v->nPlaneCells < 0 || (v->nPlaneCells > 0 && (!v->planeCells || !v->planeAreas)))
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: plane cells");
    if (v->nHeatPatches < 0 || (v->nHeatPatches > 0 && (!v->heatPatches || !v->heatWeights)))
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: heat patches");
    if (!(v->ptin != 0.0) || !std::isfinite(v->ptin) || !std::isfinite(v->Tw) || !std::isfinite(v->a) ||
        !std::isfinite(v->b))
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: constants");
    DeviceGuard dg(c->device);
    int np = v->nPlaneCells;
    std::vector<int32_t> cells(np > 0 ? np : 1), cellPlane(c->nIC, -1);
    std::vector<double> areas(np > 0 ? np : 1);
    for (int q = 0; q < np; q++) {
        int cc = v->planeCells[q];
        if (cc < 0 || cc >= c->nIC || cellPlane[cc] >= 0)
            return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: plane cell out of range or repeated");
        cells[q] = cc;
        areas[q] = v->planeAreas[q];
        cellPlane[cc] = q;
    }
    // heat-transfer coefficients k A w / delta from the context's mesh tables
    std::vector<double> A(c->nF), dl(c->nF);
    cudaError_t e;
    if (c->precision == AFVM_FP64) {
        e = cudaMemcpy(A.data(), c->m64.area, sizeof(double) * c->nF, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(dl.data(), c->m64.dlt, sizeof(double) * c->nF, cudaMemcpyDeviceToHost);
    } else {
        std::vector<float> a32(c->nF), d32(c->nF);
        e = cudaMemcpy(a32.data(), c->m32.area, sizeof(float) * c->nF, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(d32.data(), c->m32.dlt, sizeof(float) * c->nF, cudaMemcpyDeviceToHost);
        for (int f = 0; f < c->nF; f++) { A[f] = a32[f]; dl[f] = d32[f]; }
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "afvm_set_objective_vane: mesh tables");
    const Phys& P = c->phys;
    double mu = (P.muModel == AFVM_MU_SUTHERLAND) ? P.muAs * std::pow(v->Tw, 1.5) / (v->Tw + P.muTs) : P.mu0;
    double k = mu * P.kFac;
    std::vector<int32_t> hf;
    std::vector<double> hc, bhc(c->nG > 0 ? c->nG : 1, 0.0);
    double w2 = 0.0;
    for (int q = 0; q < v->nHeatPatches; q++) {
        int pi = v->heatPatches[q];
        if (pi < 0 || pi >= c->nPatches || !v->heatWeights[q])
            return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: heat patch index or weights");
        for (int i = 0; i < c->patchN[pi]; i++) {
            int f = c->patchStart[pi] + i;
            double w = v->heatWeights[q][i];
            w2 += A[f] * w;
            if (w == 0.0) continue;
            double cf = k * A[f] * w / dl[f];
            hf.push_back(f);
            hc.push_back(cf);
            bhc[f - c->nIF] += cf;
        }
    }
    int nh = (int)hf.size();
    if (hf.empty()) { hf.push_back(0); hc.push_back(0.0); }   // one placeholder, never read
    VaneDev d{};
    int st;
    if ((st = upload(c, &d.planeCells, cells))) return st;
    if ((st = upload(c, &d.planeArea, areas))) return st;
    if ((st = upload(c, &d.cellPlane, cellPlane))) return st;
    if ((st = upload(c, &d.heatFaces, hf))) return st;
    if ((st = upload(c, &d.heatCoef, hc))) return st;
    if ((st = upload(c, &d.bHeatCoef, bhc))) return st;
    int nb = nblocks((long long)np + nh);
    if (nb < 1) nb = 1;
    if ((st = dalloc(c, (void**)&c->vanePartials, sizeof(double) * 3 * (size_t)nb))) return st;
    if ((st = dalloc(c, (void**)&c->vaneSums, sizeof(double) * 4))) return st;
    cudaMemset(c->vaneSums, 0, sizeof(double) * 4);
    d.sums = c->vaneSums;
    d.nPlane = np;
    d.nHeat = nh;
    double nn = std::sqrt(v->normal[0] * v->normal[0] + v->normal[1] * v->normal[1] + v->normal[2] * v->normal[2]);
    if (!(nn > 0)) return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_objective_vane: zero normal");
    d.n0 = v->normal[0]; d.n1 = v->normal[1]; d.n2 = v->normal[2];
    d.ptin = v->ptin; d.Tw = v->Tw; d.a = v->a; d.b = v->b;
    d.rw2 = (w2 != 0.0) ? 1.0 / w2 : 0.0;
    c->vane = d;
    c->nVaneBlocks = nb;
    c->vaneSet = true;
    return AFVM_OK;
}

int afvm_set_bc_value(afvm_ctx* ctx, int32_t patch, int32_t field, const double* values) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (patch < 0 || patch >= c->nPatches || field < 0 || field > 2 || !values)
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_bc_value: bad patch/field/values");
    int kind = c->bcKinds[3 * patch + field];
    if (kind != AFVM_BC_FIXED_VALUE && kind != AFVM_BC_CBC_UPT && kind != AFVM_BC_CBC_TOTAL_PT)
        return fail(c, AFVM_ERR_BAD_ARG, "afvm_set_bc_value: the BC has no values");
    DeviceGuard dg(c->device);
    int g0 = c->patchStart[patch] - c->nIF, n = c->patchN[patch];
    int dims = field == 0 ? 3 : 1, comp0 = field == 0 ? 0 : (field == 1 ? 3 : 4);
    size_t es = c->precision == AFVM_FP64 ? sizeof(double) : sizeof(float);
    char* base = (char*)(c->precision == AFVM_FP64 ? (const void*)c->m64.gval : (const void*)c->m32.gval);
    std::vector<char> col(es * (size_t)n);
    for (int k = 0; k < dims; k++) {
        for (int i = 0; i < n; i++) {
            double v = values[(size_t)dims * i + k];
            if (es == sizeof(double)) memcpy(&col[es * i], &v, es);
            else { float fv = (float)v; memcpy(&col[es * i], &fv, es); }
        }
        cudaError_t e = cudaMemcpy(base + es * ((size_t)(comp0 + k) * c->nG + g0), col.data(), es * (size_t)n,
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "afvm_set_bc_value");
    }
    return AFVM_OK;
}

int64_t afvm_tape_elements(const afvm_ctx* ctx) {
    if (!ctx) return 0;
    return (int64_t)tape_elements(reinterpret_cast<const Ctx*>(ctx));
}

int afvm_primal_step_tape(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                          const void* S_rho, const void* S_rhoU, const void* S_rhoE, void* rhoN, void* rhoUN,
                          void* rhoEN, void* stages, void* tape, double* dtc_out, double* obj_out, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || !rhoN || !rhoUN || !rhoEN) return fail(c, AFVM_ERR_BAD_ARG, "null state pointer");
    if (!std::isfinite(dt)) return fail(c, AFVM_ERR_BAD_ARG, "non-finite dt");
    if (tape && !stages) return fail(c, AFVM_ERR_BAD_ARG, "a face tape is kept together with the stage states");
    if (((uintptr_t)tape & 15) != 0) return fail(c, AFVM_ERR_BAD_ARG, "the tape must be 16-byte aligned");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    int st = dispatch(c, [&](auto r, auto sv) {
        using R = decltype(r);
        using S = decltype(sv);
        return primal_step_dev<R, S>(c, (const S*)rho, (const S*)rhoU, (const S*)rhoE, dt, nullptr, (const S*)S_rho,
                                     (const S*)S_rhoU, (const S*)S_rhoE, (S*)rhoN, (S*)rhoUN, (S*)rhoEN, c->scal,
                                     c->scal + 1, s, (S*)stages, (R*)tape);
    });
    if (st) return st;
    return get_results(c, dtc_out, obj_out, s);
}

int afvm_primal_step_stages(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                            const void* S_rho, const void* S_rhoU, const void* S_rhoE, void* rhoN, void* rhoUN,
                            void* rhoEN, void* stages, double* dtc_out, double* obj_out, void* stream) {
    return afvm_primal_step_tape(ctx, rho, rhoU, rhoE, dt, S_rho, S_rhoU, S_rhoE, rhoN, rhoUN, rhoEN, stages, nullptr,
                                 dtc_out, obj_out, stream);
}

int afvm_primal_step(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                     const void* S_rho, const void* S_rhoU, const void* S_rhoE, void* rhoN, void* rhoUN, void* rhoEN,
                     double* dtc_out, double* obj_out, void* stream) {
    return afvm_primal_step_stages(ctx, rho, rhoU, rhoE, dt, S_rho, S_rhoU, S_rhoE, rhoN, rhoUN, rhoEN, nullptr,
                                   dtc_out, obj_out, stream);
}

int afvm_primal_step_host(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                          const void* S_rho, const void* S_rhoU, const void* S_rhoE, void* rhoN, void* rhoUN,
                          void* rhoEN, double* dtc_out, double* obj_out, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || !rhoN || !rhoUN || !rhoEN) return fail(c, AFVM_ERR_BAD_ARG, "null state pointer");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    size_t es = state_size(c);
    size_t n = c->nIC;
    // device staging, allocated on first use: state in (5n), state out (5n), sources (5n)
    if (!c->stageDev) {
        int st0 = dalloc(c, &c->stageDev, es * n * 15);
        if (st0) return st0;
    }
    int st = AFVM_OK;
    void* stage = c->stageDev;
    char* in = (char*)stage;
    char* outp = in + es * n * 5;
    char* src = outp + es * n * 5;
    void* dIn[3] = {in, in + es * n, in + es * n * 4};
    void* dOut[3] = {outp, outp + es * n, outp + es * n * 4};
    const void* hIn[3] = {rho, rhoU, rhoE};
    void* hOut[3] = {rhoN, rhoUN, rhoEN};
    size_t cnt[3] = {n, 3 * n, n};
    // pinned buffers are copied asynchronously; pageable ones through the pipelined host copy
    for (int k = 0; k < 3; k++) {
        st = host_copy(c->device, dIn[k], (int)es, hIn[k], (int)es, (int64_t)cnt[k], stream, true, false);
        if (st) return fail(c, st, "state upload");
    }
    const void* S[3] = {S_rho, S_rhoU, S_rhoE};
    void* dS[3] = {nullptr, nullptr, nullptr};
    void* sbuf[3] = {src, src + es * n, src + es * n * 4};
    for (int k = 0; k < 3; k++) {
        if (S[k]) {
            st = host_copy(c->device, sbuf[k], (int)es, S[k], (int)es, (int64_t)cnt[k], stream, true, false);
            if (st) return fail(c, st, "source upload");
            dS[k] = sbuf[k];
        }
    }
    st = afvm_primal_step(ctx, dIn[0], dIn[1], dIn[2], dt, dS[0], dS[1], dS[2], dOut[0], dOut[1], dOut[2], nullptr,
                          nullptr, stream);
    if (st) return st;
    for (int k = 0; k < 3; k++) {
        st = host_copy(c->device, hOut[k], (int)es, dOut[k], (int)es, (int64_t)cnt[k], stream, false, false);
        if (st) return fail(c, st, "state download");
    }
    if (!dtc_out && !obj_out) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(c, e, "host step");
        return AFVM_OK;
    }
    return get_results(c, dtc_out, obj_out, s);
}

int afvm_primal_run(afvm_ctx* ctx, void* rho, void* rhoU, void* rhoE, int32_t nSteps, double dt0, double CFL,
                    double stepFactor, int32_t fixed_dt, const void* S_rho, const void* S_rhoU, const void* S_rhoE,
                    double* dt_hist, double* dtc_hist, double* obj_hist, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || nSteps < 0) return fail(c, AFVM_ERR_BAD_ARG, "afvm_primal_run arguments");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    return dispatch(c, [&](auto r, auto sv) {
        using R = decltype(r);
        using S = decltype(sv);
        return primal_run_dev<R, S>(c, (S*)rho, (S*)rhoU, (S*)rhoE, nSteps, dt0, CFL, stepFactor, fixed_dt,
                                    (const S*)S_rho, (const S*)S_rhoU, (const S*)S_rhoE, dt_hist, dtc_hist, obj_hist,
                                    s);
    });
}

int afvm_adjoint_step_stages(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                             const void* S_rho, const void* S_rhoU, const void* S_rhoE, const void* stages,
                             const void* rhoNa, const void* rhoUNa, const void* rhoENa, double dtca, double obja,
                             void* rhoa, void* rhoUa, void* rhoEa, void* S_rhoa, void* S_rhoUa, void* S_rhoEa,
                             void* stream) {
    return afvm_adjoint_step_tape(ctx, rho, rhoU, rhoE, dt, S_rho, S_rhoU, S_rhoE, stages, nullptr, rhoNa, rhoUNa,
                                  rhoENa, dtca, obja, rhoa, rhoUa, rhoEa, S_rhoa, S_rhoUa, S_rhoEa, stream);
}

int afvm_adjoint_step_tape(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                           const void* S_rho, const void* S_rhoU, const void* S_rhoE, const void* stages,
                           const void* tape, const void* rhoNa, const void* rhoUNa, const void* rhoENa, double dtca,
                           double obja, void* rhoa, void* rhoUa, void* rhoEa, void* S_rhoa, void* S_rhoUa,
                           void* S_rhoEa, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || !rhoNa || !rhoUNa || !rhoENa || !rhoa || !rhoUa || !rhoEa)
        return fail(c, AFVM_ERR_BAD_ARG, "null pointer");
    if (dtca != 0.0) return fail(c, AFVM_ERR_UNSUPPORTED, "dtca != 0 (the CFL-sum output has no adjoint here)");
    if (tape && !stages) return fail(c, AFVM_ERR_BAD_ARG, "a face tape is read together with the stage states");
    if (((uintptr_t)tape & 15) != 0) return fail(c, AFVM_ERR_BAD_ARG, "the tape must be 16-byte aligned");
    if (!std::isfinite(dt) || !std::isfinite(obja)) return fail(c, AFVM_ERR_BAD_ARG, "non-finite dt or obja");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    return dispatch(c, [&](auto r, auto sv) {
        using R = decltype(r);
        using S = decltype(sv);
        int st = alloc_adjoint<R, S>(c);
        if (st) return st;
        return adjoint_step_dev<R, S>(c, (const S*)rho, (const S*)rhoU, (const S*)rhoE, dt, (const S*)S_rho,
                                      (const S*)S_rhoU, (const S*)S_rhoE, (const S*)rhoNa, (const S*)rhoUNa,
                                      (const S*)rhoENa, obja, (S*)rhoa, (S*)rhoUa, (S*)rhoEa, (S*)S_rhoa,
                                      (S*)S_rhoUa, (S*)S_rhoEa, s, (const S*)stages, (const R*)tape);
    });
}

int afvm_adjoint_step_params(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                             const void* S_rho, const void* S_rhoU, const void* S_rhoE, const void* stages,
                             const void* tape, const void* rhoNa, const void* rhoUNa, const void* rhoENa,
                             double dtca, double obja, void* rhoa, void* rhoUa, void* rhoEa, void* S_rhoa,
                             void* S_rhoUa, void* S_rhoEa, const afvm_param_grad* pg, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!pg) return fail(c, AFVM_ERR_BAD_ARG, "null parameter-gradient description");
    if (!rho || !rhoU || !rhoE || !rhoNa || !rhoUNa || !rhoENa || !rhoa || !rhoUa || !rhoEa)
        return fail(c, AFVM_ERR_BAD_ARG, "null pointer");
    if (c->precision != AFVM_FP64)
        return fail(c, AFVM_ERR_UNSUPPORTED, "mesh and boundary-input gradients need an AFVM_FP64 context");
    if (dtca != 0.0) return fail(c, AFVM_ERR_UNSUPPORTED, "dtca != 0 (the CFL-sum output has no adjoint here)");
    if (tape && !stages) return fail(c, AFVM_ERR_BAD_ARG, "a face tape is read together with the stage states");
    if (((uintptr_t)tape & 15) != 0) return fail(c, AFVM_ERR_BAD_ARG, "the tape must be 16-byte aligned");
    if (!std::isfinite(dt) || !std::isfinite(obja)) return fail(c, AFVM_ERR_BAD_ARG, "non-finite dt or obja");
    bool mesh = pg->areas || pg->volumesL || pg->volumesR || pg->weights || pg->deltas || pg->normals ||
                pg->deltasUnit || pg->linearWeights || pg->quadraticWeights || pg->volumes;
    if (mesh && c->objective == AFVM_OBJ_VANE && c->vane.b != 0.0)
        return fail(c, AFVM_ERR_UNSUPPORTED, "mesh gradient of the vane objective's heat-transfer term");
    ParamDev pd{};
    pd.areas = pg->areas; pd.volL = pg->volumesL; pd.volR = pg->volumesR; pd.wts = pg->weights;
    pd.dlt = pg->deltas; pd.nrm = pg->normals; pd.du = pg->deltasUnit; pd.lw = pg->linearWeights;
    pd.qw = pg->quadraticWeights; pd.vol = pg->volumes;
    int bcDims = 0;
    if (pg->bcPatch >= 0) {
        if (pg->bcPatch >= c->nPatches || pg->bcField < 0 || pg->bcField > 2 || !pg->bc)
            return fail(c, AFVM_ERR_BAD_ARG, "boundary input: patch, field or output");
        int kind = c->bcKinds[3 * pg->bcPatch + pg->bcField];
        if (kind != AFVM_BC_FIXED_VALUE && kind != AFVM_BC_CBC_UPT && kind != AFVM_BC_CBC_TOTAL_PT)
            return fail(c, AFVM_ERR_BAD_ARG, "boundary input: the field has no input on that patch");
        if (kind == AFVM_BC_CBC_TOTAL_PT && pg->bcField == 0 && c->patchDirNormals[pg->bcPatch])
            return fail(c, AFVM_ERR_BAD_ARG, "boundary input: that CBC_TOTAL_PT direction is the face normals");
        pd.bcStart = c->patchStart[pg->bcPatch];
        pd.bcN = c->patchN[pg->bcPatch];
        pd.bcField = pg->bcField;
        pd.bc = pg->bc;
        bcDims = pg->bcField == 0 ? 3 : 1;
    } else if (!mesh) {
        return fail(c, AFVM_ERR_BAD_ARG, "no parameter gradient asked for");
    }
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    int st = alloc_adjoint<double, double>(c);
    if (st) return st;
    // per ghost: the CBC_TOTAL_PT direction is the face normal (a mesh input then)
    if (!c->gdirn && c->nG > 0) {
        std::vector<uint8_t> h(c->nG, 0);
        for (int pi = 0; pi < c->nPatches; pi++)
            if (c->patchDirNormals[pi])
                for (int i = 0; i < c->patchN[pi]; i++) h[c->patchStart[pi] - c->nIF + i] = 1;
        void* p = nullptr;
        st = ctx_alloc(c, &p, h.size());
        if (st) return st;
        cudaError_t e = cudaMemcpy(p, h.data(), h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "ghost direction flags");
        c->gdirn = (uint8_t*)p;
    }
    pd.gdirn = c->gdirn;
    // the outputs are the step's gradients: cleared, then summed over the three stages
    const size_t nF = c->nF, nIF = c->nIF, nIC = c->nIC;
    const std::pair<double*, size_t> outs[] = {{pd.areas, nF}, {pd.volL, nF}, {pd.volR, nIF}, {pd.wts, nF},
                                               {pd.dlt, nF}, {pd.nrm, 3 * nF}, {pd.du, 3 * nF}, {pd.lw, 2 * nF},
                                               {pd.qw, 6 * nF}, {pd.vol, nIC},
                                               {pd.bc, (size_t)pd.bcN * bcDims}};
    for (const auto& o : outs) {
        if (!o.first || !o.second) continue;
        cudaError_t e = cudaMemsetAsync(o.first, 0, o.second * sizeof(double), s);
        if (e != cudaSuccess) return cuda_fail(c, e, "parameter gradient clear");
    }
    return adjoint_step_dev<double, double>(c, (const double*)rho, (const double*)rhoU, (const double*)rhoE, dt,
                                            (const double*)S_rho, (const double*)S_rhoU, (const double*)S_rhoE,
                                            (const double*)rhoNa, (const double*)rhoUNa, (const double*)rhoENa, obja,
                                            (double*)rhoa, (double*)rhoUa, (double*)rhoEa, (double*)S_rhoa,
                                            (double*)S_rhoUa, (double*)S_rhoEa, s, (const double*)stages,
                                            (const double*)tape, &pd);
}

int afvm_adjoint_step(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, double dt,
                      const void* S_rho, const void* S_rhoU, const void* S_rhoE, const void* rhoNa,
                      const void* rhoUNa, const void* rhoENa, double dtca, double obja, void* rhoa, void* rhoUa,
                      void* rhoEa, void* S_rhoa, void* S_rhoUa, void* S_rhoEa, void* stream) {
    return afvm_adjoint_step_stages(ctx, rho, rhoU, rhoE, dt, S_rho, S_rhoU, S_rhoE, nullptr, rhoNa, rhoUNa, rhoENa,
                                    dtca, obja, rhoa, rhoUa, rhoEa, S_rhoa, S_rhoUa, S_rhoEa, stream);
}

int afvm_adjoint_viscosity(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, int32_t kind,
                           double scaling, double dt, void* rhoa, void* rhoUa, void* rhoEa, double* M_out,
                           double* DT_out, int32_t* iterations_out, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || !rhoa || !rhoUa || !rhoEa) return fail(c, AFVM_ERR_BAD_ARG, "null pointer");
    if (kind < AFVM_VISC_UNIFORM || kind > AFVM_VISC_ABARBANEL) return fail(c, AFVM_ERR_BAD_ARG, "viscosity kind");
    if (!std::isfinite(scaling) || !std::isfinite(dt) || dt < 0) return fail(c, AFVM_ERR_BAD_ARG, "scaling or dt");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    int it = 0;
    int st = dispatch(c, [&](auto r, auto sv) {
        using R = decltype(r);
        using S = decltype(sv);
        return adjoint_viscosity_dev<R, S>(c, (const S*)rho, (const S*)rhoU, (const S*)rhoE, kind, scaling, dt,
                                           (S*)rhoa, (S*)rhoUa, (S*)rhoEa, M_out, DT_out, &it, s);
    });
    if (iterations_out) *iterations_out = it;
    return st;
}

int afvm_boundary_values(afvm_ctx* ctx, const void* rho, const void* rhoU, const void* rhoE, void* out,
                         void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    if (!rho || !rhoU || !rhoE || (!out && c->nG > 0)) return fail(c, AFVM_ERR_BAD_ARG, "null pointer");
    DeviceGuard dg(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (c->nG == 0) return AFVM_OK;
    size_t es = record_size(c);
    dispatch(c, [&](auto r, auto sv) {
        using R = decltype(r);
        using S = decltype(sv);
        launch_prim<R, S>(c, (const S*)rho, (const S*)rhoU, (const S*)rhoE, s);
        return 0;
    });
    // ghost rows of the cell record, columns U, T, p (FP32 records: the gauge offsets of T and p
    // made absolute)
    const char* src = (const char*)c->rec + es * REC * (size_t)c->nIC;
    cudaError_t e = cudaSuccess;
    if (c->precision == AFVM_FP64)
        e = cudaMemcpy2DAsync(out, es * 5, src, es * REC, es * 5, (size_t)c->nG, cudaMemcpyDeviceToDevice, s);
    else
        launch_abs_prims(c, (const float*)src, REC, c->nG, (float*)out, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "boundary values copy");
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "boundary values launch");
    return AFVM_OK;
}

int afvm_sensitivity(afvm_ctx* ctx, int32_t nArrays, const double* const* grad, const double* const* pert,
                     const int64_t* n, double* out, void* stream) {
    if (!ctx) return AFVM_ERR_BAD_ARG;
    Ctx* c = reinterpret_cast<Ctx*>(ctx);
    DeviceGuard dg(c->device);
    return sensitivity_dev(c, nArrays, grad, pert, n, out, (cudaStream_t)stream);
}

}  // extern "C"
