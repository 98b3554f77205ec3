// Bandwidth renumbering of a hex mesh's cells on the GPU: reverse Cuthill-McKee (Cuthill and
// McKee 1969; reversed as George 1971) over the cell graph whose edges are the internal faces
// and the cyclic patch face pairs, so that a mesh admitted in any cell order is laid out for
// coalesced gathers before its geometry is built (afvm_mesh_build_device).
//
// The order is the sequential Cuthill-McKee order with fixed tie rules, computed level by
// level without a sort:
//   * each connected component starts from the unvisited cell of least (degree, id), the
//     degree counting distinct neighbours other than the cell itself;
//   * a dequeued cell appends its unvisited neighbours in increasing (degree, id).
// A cell of level L+1 is appended by its level-L neighbour of least position (BFS queues
// finish a level before the next starts), so per level: every frontier cell claims its
// unvisited neighbours and offers its position (atomicMin: the parent is the least offer);
// each frontier cell counts the neighbours whose parent it is; an exclusive scan of the
// counts gives each parent its children's first position; each parent writes its children
// sorted by (degree, id). The result is the sequential order, position for position.
// New id = nInternalCells - 1 - position. The highest new id then goes to a cell owning a
// boundary face (an OpenFOAM reader counts cells as max(owner) + 1, adFVM/mesh.py:521): if
// the cell with id nIC - 1 owns none, it swaps ids with the boundary-owning cell of highest
// new id.
//
// Faces: an internal face whose new owner id exceeds its new neighbour id is flipped (owner
// and neighbour swapped, its points listed p2 p1 p0 p3); internal faces are then ordered by
// (new owner, new neighbour, old face id) - a bucket per owner cell (at most six faces) and
// an in-thread sort, no global sort. Boundary faces keep their positions and point lists.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>
#include <vector>
#include "afvm.h"

namespace {

constexpr int TB = 256;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_BLOCK = TB * SCAN_PER_THREAD;   // elements per block of the scan
constexpr int MAXDEG = 6;                          // a hex cell has six faces
enum : int { E_OWNER = 1, E_NEIGHBOUR = 2, E_DEGREE = 4, E_PLACE = 8, E_EMPTY = 16 };

struct DevPatch {
    int startFace, nFaces, partnerStart;   // partnerStart: start face of the cyclic partner, -1 otherwise
};

inline int nb(long long n) { return (int)((n + TB - 1) / TB); }

// ---- exclusive scan of non-negative int counts (block scans, a one-block scan of the block
// sums, then the add); in and out may be the same array
__global__ void k_scan_blocks(const int* in, int* out, int n, int* bsum) {
    __shared__ int sh[TB];
    int t = threadIdx.x;
    long long base = (long long)blockIdx.x * SCAN_BLOCK + (long long)SCAN_PER_THREAD * t;
    int v[SCAN_PER_THREAD];
    int s = 0;
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        long long i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    sh[t] = s;
    __syncthreads();
    for (int d = 1; d < TB; d <<= 1) {
        int x = t >= d ? sh[t - d] : 0;
        __syncthreads();
        sh[t] += x;
        __syncthreads();
    }
    int run = sh[t] - s;
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (t == TB - 1) bsum[blockIdx.x] = sh[t];
}

__global__ void k_scan_sums(int* bsum, int nBlocks, int* total) {
    __shared__ int sh[TB];
    int t = threadIdx.x;
    int carry = 0;
    for (int base = 0; base < nBlocks; base += TB) {
        int i = base + t;
        int v = i < nBlocks ? bsum[i] : 0;
        sh[t] = v;
        __syncthreads();
        for (int d = 1; d < TB; d <<= 1) {
            int x = t >= d ? sh[t - d] : 0;
            __syncthreads();
            sh[t] += x;
            __syncthreads();
        }
        if (i < nBlocks) bsum[i] = carry + sh[t] - v;
        carry += sh[TB - 1];
        __syncthreads();
    }
    if (t == 0) *total = carry;
}

__global__ void k_scan_add(int* out, int n, const int* bsum) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / SCAN_BLOCK];
}

void scan_exclusive(const int* in, int* out, int n, int* bsum, int* total, cudaStream_t s) {
    if (n <= 0) {
        cudaMemsetAsync(total, 0, sizeof(int), s);
        return;
    }
    int nBlocks = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    k_scan_blocks<<<nBlocks, TB, 0, s>>>(in, out, n, bsum);
    k_scan_sums<<<1, TB, 0, s>>>(bsum, nBlocks, total);
    k_scan_add<<<nb(n), TB, 0, s>>>(out, n, bsum);
}

// ---- graph
// range checks and the adjacency rows: internal faces add both directions, a cyclic face adds
// its owner -> its partner face's owner (the partner patch adds the reverse)
__global__ void k_adjacency(int nFaces, int nIF, int nIC, const int32_t* __restrict__ owner,
                            const int32_t* __restrict__ nbr, int nPatches, const DevPatch* __restrict__ patches,
                            int* __restrict__ fill, int32_t* __restrict__ adj, int* __restrict__ nfaces,
                            int* __restrict__ err) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    int p = owner[f];
    if (p < 0 || p >= nIC) {
        atomicOr(err, E_OWNER);
        return;
    }
    atomicAdd(nfaces + p, 1);
    int q = -1;
    if (f < nIF) {
        q = nbr[f];
        if (q < 0 || q >= nIC || q == p) {
            atomicOr(err, E_NEIGHBOUR);
            return;
        }
        atomicAdd(nfaces + q, 1);
    } else {
        for (int k = 0; k < nPatches; k++) {
            const DevPatch& P = patches[k];
            if (f >= P.startFace && f < P.startFace + P.nFaces) {
                if (P.partnerStart >= 0) {
                    int g = P.partnerStart + (f - P.startFace);   // range checked on the host
                    q = owner[g];
                    if (q < 0 || q >= nIC) {
                        atomicOr(err, E_OWNER);
                        return;
                    }
                }
                break;
            }
        }
        if (q < 0) return;
    }
    int s = atomicAdd(fill + p, 1);
    if (s < MAXDEG) adj[MAXDEG * (size_t)p + s] = q;
    else atomicOr(err, E_DEGREE);
    if (f < nIF) {
        s = atomicAdd(fill + q, 1);
        if (s < MAXDEG) adj[MAXDEG * (size_t)q + s] = p;
        else atomicOr(err, E_DEGREE);
    }
}

// a cell without faces is not a mesh cell (a wrong owner index leaves such cells behind)
__global__ void k_cells_have_faces(int nIC, const int* __restrict__ nfaces, int* __restrict__ err) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nIC && nfaces[c] == 0) atomicOr(err, E_EMPTY);
}

// each row sorted by id, duplicates and the cell itself dropped; deg = distinct neighbours
__global__ void k_rows(int nIC, const int* __restrict__ fill, int32_t* __restrict__ adj, int* __restrict__ deg) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC) return;
    int n = fill[c];
    if (n > MAXDEG) n = MAXDEG;
    int v[MAXDEG];
    for (int k = 0; k < n; k++) v[k] = adj[MAXDEG * (size_t)c + k];
    for (int i = 1; i < n; i++) {
        int x = v[i], j = i - 1;
        while (j >= 0 && v[j] > x) {
            v[j + 1] = v[j];
            j--;
        }
        v[j + 1] = x;
    }
    int m = 0;
    for (int k = 0; k < n; k++) {
        if (v[k] == c || (m > 0 && v[m - 1] == v[k])) continue;
        v[m++] = v[k];
    }
    for (int k = 0; k < m; k++) adj[MAXDEG * (size_t)c + k] = v[k];
    deg[c] = m;
}

// least (degree, id) over the unvisited cells
__global__ void k_seed(int nIC, const int* __restrict__ deg, const int* __restrict__ lev,
                       unsigned long long* __restrict__ best) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC || lev[c] >= 0) return;
    atomicMin(best, ((unsigned long long)deg[c] << 32) | (unsigned)c);
}

__global__ void k_start(const unsigned long long* __restrict__ best, int nIC, int pos, int level,
                        int32_t* __restrict__ order, int* __restrict__ lev, int* __restrict__ err) {
    unsigned long long k = *best;
    long long c = (long long)(k & 0xffffffffull);
    if (k == ~0ull || c >= nIC || pos < 0 || pos >= nIC) {
        atomicOr(err, E_PLACE);
        return;
    }
    order[pos] = (int32_t)c;
    lev[c] = level;
}

__global__ void k_claim(int fs, int fe, const int32_t* __restrict__ order, const int32_t* __restrict__ adj,
                        const int* __restrict__ deg, int* __restrict__ lev, int* __restrict__ ppos, int next) {
    int p = fs + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fe) return;
    int c = order[p];
    for (int k = 0; k < deg[c]; k++) {
        int j = adj[MAXDEG * (size_t)c + k];
        int old = atomicCAS(lev + j, -1, next);
        if (old == -1 || old == next) atomicMin(ppos + j, p);
    }
}

__global__ void k_count(int fs, int fe, const int32_t* __restrict__ order, const int32_t* __restrict__ adj,
                        const int* __restrict__ deg, const int* __restrict__ lev, const int* __restrict__ ppos,
                        int next, int* __restrict__ cnt) {
    int p = fs + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fe) return;
    int c = order[p];
    int n = 0;
    for (int k = 0; k < deg[c]; k++) {
        int j = adj[MAXDEG * (size_t)c + k];
        if (lev[j] == next && ppos[j] == p) n++;
    }
    cnt[p - fs] = n;
}

__global__ void k_place(int fs, int fe, int nIC, int32_t* __restrict__ order, const int32_t* __restrict__ adj,
                        const int* __restrict__ deg, const int* __restrict__ lev, const int* __restrict__ ppos,
                        int next, const int* __restrict__ off, int* __restrict__ err) {
    int p = fs + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= fe) return;
    int c = order[p];
    long long key[MAXDEG];
    int n = 0;
    for (int k = 0; k < deg[c]; k++) {
        int j = adj[MAXDEG * (size_t)c + k];
        if (lev[j] == next && ppos[j] == p) key[n++] = ((long long)deg[j] << 32) | (unsigned)j;
    }
    for (int i = 1; i < n; i++) {
        long long x = key[i];
        int j = i - 1;
        while (j >= 0 && key[j] > x) {
            key[j + 1] = key[j];
            j--;
        }
        key[j + 1] = x;
    }
    long long at = (long long)fe + off[p - fs];
    for (int k = 0; k < n; k++) {
        if (at + k >= nIC) {
            atomicOr(err, E_PLACE);
            return;
        }
        order[at + k] = (int32_t)(key[k] & 0xffffffffll);
    }
}

__global__ void k_new_ids(int nIC, const int32_t* __restrict__ order, int32_t* __restrict__ cellNew) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nIC) cellNew[order[p]] = nIC - 1 - p;
}

__global__ void k_boundary_max(int nFaces, int nIF, const int32_t* __restrict__ owner,
                               const int32_t* __restrict__ cellNew, int* __restrict__ mx) {
    int f = nIF + blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nFaces) atomicMax(mx, cellNew[owner[f]]);
}

// give id nIC-1 to the cell that has id mx, and mx to the cell that had nIC-1
__global__ void k_swap_last(int nIC, const int32_t* __restrict__ order, const int* __restrict__ mx,
                            int32_t* __restrict__ cellNew) {
    int m = *mx;
    if (m < 0 || m >= nIC - 1) return;
    int a = order[0];                 // new id nIC-1
    int b = order[nIC - 1 - m];       // new id m
    cellNew[a] = m;
    cellNew[b] = nIC - 1;
}

// ---- faces
__global__ void k_face_count(int nIF, const int32_t* __restrict__ owner, const int32_t* __restrict__ nbr,
                             const int32_t* __restrict__ cellNew, int* __restrict__ cnt) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nIF) return;
    int a = cellNew[owner[f]], b = cellNew[nbr[f]];
    atomicAdd(cnt + (a < b ? a : b), 1);
}

__global__ void k_face_bucket(int nIF, const int32_t* __restrict__ owner, const int32_t* __restrict__ nbr,
                              const int32_t* __restrict__ cellNew, const int* __restrict__ off,
                              int* __restrict__ fill, int32_t* __restrict__ bucket) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nIF) return;
    int a = cellNew[owner[f]], b = cellNew[nbr[f]];
    int o = a < b ? a : b;
    int s = atomicAdd(fill + o, 1);
    bucket[off[o] + s] = f;
}

// per new owner cell: its faces in (new neighbour, old face) order, written to their places
__global__ void k_face_write(int nIC, const int* __restrict__ off, const int* __restrict__ cnt,
                             const int32_t* __restrict__ bucket, const int32_t* __restrict__ faces,
                             const int32_t* __restrict__ owner, const int32_t* __restrict__ nbr,
                             const int32_t* __restrict__ cellNew, int32_t* __restrict__ facesOut,
                             int32_t* __restrict__ ownerOut, int32_t* __restrict__ nbrOut,
                             int32_t* __restrict__ faceOld, int* __restrict__ err) {
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nIC) return;
    int n = cnt[o];
    if (n > MAXDEG) {
        atomicOr(err, E_DEGREE);
        return;
    }
    long long key[MAXDEG];
    for (int k = 0; k < n; k++) {
        int f = bucket[off[o] + k];
        int a = cellNew[owner[f]], b = cellNew[nbr[f]];
        key[k] = ((long long)(a > b ? a : b) << 32) | (unsigned)f;
    }
    for (int i = 1; i < n; i++) {
        long long x = key[i];
        int j = i - 1;
        while (j >= 0 && key[j] > x) {
            key[j + 1] = key[j];
            j--;
        }
        key[j + 1] = x;
    }
    for (int k = 0; k < n; k++) {
        int f = (int)(key[k] & 0xffffffffll);
        int q = off[o] + k;
        int a = cellNew[owner[f]];
        bool flip = a != o;
        const int32_t* src = faces + 5 * (size_t)f;
        int32_t* dst = facesOut + 5 * (size_t)q;
        dst[0] = src[0];
        // a flipped face lists (p2, p1, p0, p3): the reversed cycle whose first three points
        // are the original first three reversed, so the normal the geometry takes from the
        // first three points (adFVM/cpp/cmesh.cpp:72-87) is exactly negated
        dst[1] = flip ? src[3] : src[1];
        dst[2] = src[2];
        dst[3] = flip ? src[1] : src[3];
        dst[4] = src[4];
        ownerOut[q] = o;
        nbrOut[q] = (int32_t)(key[k] >> 32);
        faceOld[q] = flip ? ~f : f;
    }
}

__global__ void k_boundary_faces(int nFaces, int nIF, const int32_t* __restrict__ faces,
                                 const int32_t* __restrict__ owner, const int32_t* __restrict__ cellNew,
                                 int32_t* __restrict__ facesOut, int32_t* __restrict__ ownerOut,
                                 int32_t* __restrict__ faceOld) {
    int f = nIF + blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces) return;
    for (int j = 0; j < 5; j++) facesOut[5 * (size_t)f + j] = faces[5 * (size_t)f + j];
    ownerOut[f] = cellNew[owner[f]];
    faceOld[f] = f;
}

// bandwidth: max |id(a) - id(b)| over the graph's edges, with ids as given (map NULL) or mapped
__global__ void k_bandwidth(int nIC, const int32_t* __restrict__ adj, const int* __restrict__ deg,
                            const int32_t* __restrict__ map, int* __restrict__ bw) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nIC) return;
    int a = map ? map[c] : c, m = 0;
    for (int k = 0; k < deg[c]; k++) {
        int j = adj[MAXDEG * (size_t)c + k];
        int b = map ? map[j] : j;
        int d = a > b ? a - b : b - a;
        if (d > m) m = d;
    }
    atomicMax(bw, m);
}

}  // namespace

extern "C" int afvm_mesh_reorder_device(const afvm_mesh_in* in, int32_t* facesOut, int32_t* ownerOut,
                                        int32_t* neighbourOut, int32_t* cellNew, int32_t* faceOld,
                                        int32_t* bandwidth, void* stream) {
    if (!in) return AFVM_ERR_BAD_ARG;
    const int nFaces = in->nFaces, nIF = in->nInternalFaces, nIC = in->nInternalCells;
    if (nFaces <= 0 || nIF < 0 || nIF > nFaces || nIC <= 0 || nIC > INT_MAX / MAXDEG - 1) return AFVM_ERR_BAD_ARG;
    if (!in->faces || !in->owner || (nIF > 0 && !in->neighbour) || (in->nPatches > 0 && !in->patches))
        return AFVM_ERR_BAD_ARG;
    if (!facesOut || !ownerOut || (nIF > 0 && !neighbourOut) || !cellNew || !faceOld) return AFVM_ERR_BAD_ARG;
    std::vector<DevPatch> pt(in->nPatches > 0 ? in->nPatches : 1, DevPatch{0, 0, -1});
    for (int q = 0; q < in->nPatches; q++) {
        const afvm_patch& P = in->patches[q];
        pt[q] = DevPatch{P.startFace, P.nFaces, -1};
        if (P.nFaces < 0 || (P.nFaces > 0 && (P.startFace < nIF || P.startFace + P.nFaces > nFaces)))
            return AFVM_ERR_BAD_ARG;
        if (P.kind == AFVM_PATCH_PROCESSOR && P.nFaces > 0) return AFVM_ERR_UNSUPPORTED;
        if (P.kind == AFVM_PATCH_CYCLIC) {
            int np = P.neighbourPatch;
            if (np < 0 || np >= in->nPatches || in->patches[np].nFaces != P.nFaces) return AFVM_ERR_BAD_ARG;
            const afvm_patch& Q = in->patches[np];
            if (P.nFaces > 0 && (Q.startFace < nIF || Q.startFace + Q.nFaces > nFaces)) return AFVM_ERR_BAD_ARG;
            pt[q].partnerStart = Q.startFace;
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)nIC;
    const int nScan = (nIC + SCAN_BLOCK - 1) / SCAN_BLOCK + 1;
    // the 64-bit seed key first (cudaMalloc's alignment keeps it 8-byte aligned for its
    // atomicMin), then ints: fill, deg, lev, ppos, order, cnt, off (n each); adj (6n); bucket
    // (nIF); scan block sums; small: err, total, mx, bw(2)
    const size_t keyBytes = 16;
    size_t nInts = 7 * n + 6 * n + (size_t)(nIF > 0 ? nIF : 1) + (size_t)nScan + 8;
    char* base = nullptr;
    DevPatch* dp = nullptr;
    cudaError_t e = cudaMalloc(&base, keyBytes + sizeof(int) * nInts);
    if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(DevPatch) * pt.size());
    if (e != cudaSuccess) {
        cudaFree(base);
        cudaFree(dp);
        cudaGetLastError();
        return AFVM_ERR_OOM;
    }
    unsigned long long* best = (unsigned long long*)base;
    int* ip = (int*)(base + keyBytes);
    int* fill = ip;
    int* deg = fill + n;
    int* lev = deg + n;
    int* ppos = lev + n;
    int32_t* order = ppos + n;
    int* cnt = order + n;
    int* off = cnt + n;
    int32_t* adj = off + n;
    int32_t* bucket = adj + 6 * n;
    int* bsum = bucket + (nIF > 0 ? nIF : 1);
    int* small = bsum + nScan;
    int* err = small;
    int* total = small + 1;
    int* mx = small + 2;
    int* bw = small + 3;          // [0] before, [1] after
    int status = AFVM_OK;
    int herr = 0;
    cudaMemcpyAsync(dp, pt.data(), sizeof(DevPatch) * pt.size(), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(fill, 0, sizeof(int) * n, s);
    cudaMemsetAsync(cnt, 0, sizeof(int) * n, s);               // faces per cell, for the check
    cudaMemsetAsync(small, 0, sizeof(int) * 8, s);
    cudaMemsetAsync(lev, 0xff, sizeof(int) * n, s);            // -1: unvisited
    cudaMemsetAsync(ppos, 0x7f, sizeof(int) * n, s);           // large
    k_adjacency<<<nb(nFaces), TB, 0, s>>>(nFaces, nIF, nIC, in->owner, in->neighbour, in->nPatches, dp, fill, adj,
                                          cnt, err);
    k_cells_have_faces<<<nb(nIC), TB, 0, s>>>(nIC, cnt, err);
    cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        status = AFVM_ERR_CUDA;
    } else if (herr & (E_OWNER | E_NEIGHBOUR | E_EMPTY)) {
        status = AFVM_ERR_BAD_ARG;
    } else if (herr) {
        status = AFVM_ERR_UNSUPPORTED;    // a cell with more than six faces
    }
    if (status == AFVM_OK) {
        k_rows<<<nb(nIC), TB, 0, s>>>(nIC, fill, adj, deg);
        k_bandwidth<<<nb(nIC), TB, 0, s>>>(nIC, adj, deg, nullptr, bw);
        int placed = 0, level = 0;
        while (placed < nIC && status == AFVM_OK) {
            cudaMemsetAsync(best, 0xff, sizeof(unsigned long long), s);
            k_seed<<<nb(nIC), TB, 0, s>>>(nIC, deg, lev, best);
            k_start<<<1, 1, 0, s>>>(best, nIC, placed, level, order, lev, err);
            int fs = placed, fe = placed + 1;
            while (fe > fs) {
                int nf = fe - fs, next = level + 1, ht = 0;
                k_claim<<<nb(nf), TB, 0, s>>>(fs, fe, order, adj, deg, lev, ppos, next);
                k_count<<<nb(nf), TB, 0, s>>>(fs, fe, order, adj, deg, lev, ppos, next, cnt);
                scan_exclusive(cnt, off, nf, bsum, total, s);
                k_place<<<nb(nf), TB, 0, s>>>(fs, fe, nIC, order, adj, deg, lev, ppos, next, off, err);
                cudaMemcpyAsync(&ht, total, sizeof(int), cudaMemcpyDeviceToHost, s);
                cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
                e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) {
                    status = AFVM_ERR_CUDA;
                    break;
                }
                if (herr || ht < 0 || ht > nIC - fe) {
                    status = AFVM_ERR_CUDA;      // cannot happen for a consistent graph
                    break;
                }
                fs = fe;
                fe += ht;
                level = next;
            }
            placed = fe;
            level += 1;
        }
    }
    if (status == AFVM_OK) {
        k_new_ids<<<nb(nIC), TB, 0, s>>>(nIC, order, cellNew);
        cudaMemsetAsync(mx, 0xff, sizeof(int), s);
        if (nFaces > nIF) {
            k_boundary_max<<<nb(nFaces - nIF), TB, 0, s>>>(nFaces, nIF, in->owner, cellNew, mx);
            k_swap_last<<<1, 1, 0, s>>>(nIC, order, mx, cellNew);
        }
        // internal faces by (new owner, new neighbour, old face)
        cudaMemsetAsync(cnt, 0, sizeof(int) * n, s);
        cudaMemsetAsync(fill, 0, sizeof(int) * n, s);
        if (nIF > 0) k_face_count<<<nb(nIF), TB, 0, s>>>(nIF, in->owner, in->neighbour, cellNew, cnt);
        scan_exclusive(cnt, off, nIC, bsum, total, s);
        if (nIF > 0) {
            k_face_bucket<<<nb(nIF), TB, 0, s>>>(nIF, in->owner, in->neighbour, cellNew, off, fill, bucket);
            k_face_write<<<nb(nIC), TB, 0, s>>>(nIC, off, cnt, bucket, in->faces, in->owner, in->neighbour, cellNew,
                                                facesOut, ownerOut, neighbourOut, faceOld, err);
        }
        if (nFaces > nIF)
            k_boundary_faces<<<nb(nFaces - nIF), TB, 0, s>>>(nFaces, nIF, in->faces, in->owner, cellNew, facesOut,
                                                             ownerOut, faceOld);
        k_bandwidth<<<nb(nIC), TB, 0, s>>>(nIC, adj, deg, cellNew, bw + 1);
        int hb[2] = {0, 0};
        cudaMemcpyAsync(hb, bw, sizeof(hb), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) status = AFVM_ERR_CUDA;
        else if (herr) status = AFVM_ERR_UNSUPPORTED;
        if (status == AFVM_OK && bandwidth) {
            bandwidth[0] = hb[0];
            bandwidth[1] = hb[1];
        }
    }
    cudaFree(dp);
    cudaFree(base);
    return status;
}
