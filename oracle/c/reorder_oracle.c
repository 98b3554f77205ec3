/*
 * Oracle (TEST INFRASTRUCTURE ONLY): sequential restatement of the cell renumbering that
 * afvm_mesh_reorder_device computes level-parallel. The product never links it.
 *
 * Reverse Cuthill-McKee (E. Cuthill and J. McKee, 1969; reversed as A. George, 1971) with
 * fixed tie rules, the textbook queue form:
 *   graph     cells; an edge across every internal face and every cyclic patch face pair
 *             (face i of a patch with face i of its neighbourPatch); repeated edges and
 *             edges of a cell to itself count once / not at all; degree = distinct
 *             neighbours;
 *   order     each component starts from the unvisited cell of least (degree, id); a cell
 *             taken from the queue appends its unvisited neighbours in increasing
 *             (degree, id);
 *   ids       new id = nInternalCells - 1 - queue position; then, if the cell with id
 *             nInternalCells - 1 owns no boundary face, it swaps ids with the boundary-owning
 *             cell of highest new id (an OpenFOAM reader counts cells as max(owner) + 1,
 *             adFVM/mesh.py:521);
 *   faces     internal faces get the new ids; one whose new owner id exceeds its new
 *             neighbour id is flipped (ids swapped, its points reordered p2 p1 p0 p3); internal
 *             faces are ordered by (new owner, new neighbour, old face id); boundary faces keep
 *             their positions and point lists. faceOld[new] = old face, or ~old if flipped.
 *   bandwidth max |id(a) - id(b)| over the graph's edges, before and after.
 * Returns 0, or 1 for an index out of range, a face between a cell and itself, a cell
 * without faces or a cell with more than six graph edges.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXDEG 6

/* point slots of a flipped face: (p2, p1, p0, p3), the reversed cycle started so that its
   first three points are the original first three in reverse order - the normal taken from
   the first three points (adFVM/cpp/cmesh.cpp:72-87) is then exactly negated */
static const int REV[5] = {0, 3, 2, 1, 4};

typedef struct {
    int64_t key;
    int32_t f;
} face_key;

static int cmp_face(const void* a, const void* b) {
    int64_t x = ((const face_key*)a)->key, y = ((const face_key*)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int oracle_mesh_reorder(int nIC, int nF, int nIF, const int32_t* faces, const int32_t* owner, const int32_t* nbr,
                        int nPatches, const int32_t* patchStart, const int32_t* patchN, const int32_t* partnerStart,
                        int32_t* facesOut, int32_t* ownerOut, int32_t* nbrOut, int32_t* cellNew, int32_t* faceOld,
                        int32_t* bandwidth) {
    int rc = 1;
    int32_t* adj = (int32_t*)malloc(sizeof(int32_t) * MAXDEG * (size_t)nIC);
    int* deg = (int*)calloc((size_t)nIC, sizeof(int));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)nIC);
    char* seen = (char*)calloc((size_t)nIC, 1);
    face_key* fk = (face_key*)malloc(sizeof(face_key) * (size_t)(nIF > 0 ? nIF : 1));
    if (!adj || !deg || !order || !seen || !fk) goto done;
    /* adjacency rows */
    for (int f = 0; f < nF; f++) {
        int p = owner[f], q = -1;
        if (p < 0 || p >= nIC) goto done;
        if (f < nIF) {
            q = nbr[f];
            if (q < 0 || q >= nIC || q == p) goto done;
        } else {
            for (int k = 0; k < nPatches; k++) {
                if (f >= patchStart[k] && f < patchStart[k] + patchN[k]) {
                    if (partnerStart[k] >= 0) q = owner[partnerStart[k] + (f - patchStart[k])];
                    break;
                }
            }
            if (q < 0) continue;
            if (q >= nIC) goto done;
        }
        if (deg[p] >= MAXDEG) goto done;
        adj[MAXDEG * (size_t)p + deg[p]++] = q;
        if (f < nIF) {
            if (deg[q] >= MAXDEG) goto done;
            adj[MAXDEG * (size_t)q + deg[q]++] = p;
        }
    }
    {   /* every cell has a face */
        char* has = seen;
        for (int f = 0; f < nF; f++) {
            has[owner[f]] = 1;
            if (f < nIF) has[nbr[f]] = 1;
        }
        for (int c = 0; c < nIC; c++)
            if (!has[c]) goto done;
        memset(seen, 0, (size_t)nIC);
    }
    for (int c = 0; c < nIC; c++) {   /* sort, drop repeats and the cell itself */
        int32_t* v = adj + MAXDEG * (size_t)c;
        int n = deg[c];
        for (int i = 1; i < n; i++)
            for (int j = i; j > 0 && v[j - 1] > v[j]; j--) { int32_t t = v[j]; v[j] = v[j - 1]; v[j - 1] = t; }
        int m = 0;
        for (int k = 0; k < n; k++) {
            if (v[k] == c || (m > 0 && v[m - 1] == v[k])) continue;
            v[m++] = v[k];
        }
        deg[c] = m;
    }
    int bw0 = 0;
    for (int c = 0; c < nIC; c++)
        for (int k = 0; k < deg[c]; k++) {
            int d = abs(c - adj[MAXDEG * (size_t)c + k]);
            if (d > bw0) bw0 = d;
        }
    /* Cuthill-McKee queue */
    int head = 0, tail = 0;
    while (tail < nIC) {
        int seed = -1;
        for (int c = 0; c < nIC; c++)
            if (!seen[c] && (seed < 0 || deg[c] < deg[seed])) seed = c;
        order[tail++] = seed;
        seen[seed] = 1;
        while (head < tail) {
            int c = order[head++];
            int first = tail;
            for (int k = 0; k < deg[c]; k++) {
                int j = adj[MAXDEG * (size_t)c + k];
                if (!seen[j]) { seen[j] = 1; order[tail++] = j; }
            }
            /* the appended cells in increasing (degree, id) */
            for (int i = first + 1; i < tail; i++)
                for (int j = i; j > first; j--) {
                    int a = order[j - 1], b = order[j];
                    if (deg[a] > deg[b] || (deg[a] == deg[b] && a > b)) { order[j - 1] = b; order[j] = a; }
                    else break;
                }
        }
    }
    for (int p = 0; p < nIC; p++) cellNew[order[p]] = nIC - 1 - p;
    if (nF > nIF) {
        int mx = -1;
        for (int f = nIF; f < nF; f++)
            if (cellNew[owner[f]] > mx) mx = cellNew[owner[f]];
        if (mx >= 0 && mx < nIC - 1) {
            int a = order[0], b = order[nIC - 1 - mx];
            cellNew[a] = mx;
            cellNew[b] = nIC - 1;
        }
    }
    /* faces */
    for (int f = 0; f < nIF; f++) {
        int a = cellNew[owner[f]], b = cellNew[nbr[f]];
        int lo = a < b ? a : b, hi = a < b ? b : a;
        fk[f].key = ((int64_t)lo << 32) | (int64_t)hi;
        fk[f].f = f;
    }
    /* ties in (owner, neighbour) keep the old face order: a stable order by sorting on the
       key and then on the face id */
    qsort(fk, (size_t)nIF, sizeof(face_key), cmp_face);
    for (int i = 0; i < nIF;) {
        int j = i;
        while (j < nIF && fk[j].key == fk[i].key) j++;
        for (int x = i + 1; x < j; x++)
            for (int y = x; y > i && fk[y - 1].f > fk[y].f; y--) { face_key t = fk[y]; fk[y] = fk[y - 1]; fk[y - 1] = t; }
        i = j;
    }
    for (int q = 0; q < nIF; q++) {
        int f = fk[q].f;
        int a = cellNew[owner[f]], b = cellNew[nbr[f]];
        int flip = a > b;
        facesOut[5 * (size_t)q] = faces[5 * (size_t)f];
        for (int j = 1; j < 5; j++) facesOut[5 * (size_t)q + j] = faces[5 * (size_t)f + (flip ? REV[j] : j)];
        ownerOut[q] = flip ? b : a;
        nbrOut[q] = flip ? a : b;
        faceOld[q] = flip ? ~f : f;
    }
    for (int f = nIF; f < nF; f++) {
        for (int j = 0; j < 5; j++) facesOut[5 * (size_t)f + j] = faces[5 * (size_t)f + j];
        ownerOut[f] = cellNew[owner[f]];
        faceOld[f] = f;
    }
    int bw1 = 0;
    for (int c = 0; c < nIC; c++)
        for (int k = 0; k < deg[c]; k++) {
            int d = abs(cellNew[c] - cellNew[adj[MAXDEG * (size_t)c + k]]);
            if (d > bw1) bw1 = d;
        }
    bandwidth[0] = bw0;
    bandwidth[1] = bw1;
    rc = 0;
done:
    free(adj);
    free(deg);
    free(order);
    free(seen);
    free(fk);
    return rc;
}
