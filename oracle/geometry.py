"""Mesh geometry and connectivity of a hex mesh in NumPy - TEST INFRASTRUCTURE ONLY.

A restatement of the reference's compiled mesh builder, cmesh.buildBeforeWrite and
cmesh.build (adFVM/cpp/cmesh.cpp:3-270), and of Mesh.createGhostCells (adFVM/mesh.py:758-819)
for one rank, vectorised over faces and cells with every element computed by the same
operations in the same order as cmesh.cpp (no contraction), so the results are those of the
reference bit for bit (tests/test_oracle_geometry.py against tests/golden/geometry.npz, which
the reference's own compiled cmesh made). bench.py's CPU baseline builds its meshes with it, so
that the timed reference arm uses no code of the library.
"""
import types

import numpy as np

CYCLIC = ('cyclic', 'slidingPeriodic1D')


def _cross(v1, v2):
    return np.stack([v1[:, 1] * v2[:, 2] - v1[:, 2] * v2[:, 1],
                     v1[:, 2] * v2[:, 0] - v1[:, 0] * v2[:, 2],
                     v1[:, 0] * v2[:, 1] - v1[:, 1] * v2[:, 0]], axis=1)


def _norm(v):
    return np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])


def build_mesh(meshData):
    """(points, faces (nF x 5: count + 4 point ids), owner, neighbour, boundary) -> an object
    with the reference Mesh's arrays and counts (nInternalCells = max(owner) + 1,
    adFVM/mesh.py:521; ghost cells appended, adFVM/mesh.py:758-819)."""
    points, faces, owner, neighbour, boundary = meshData
    points = np.asarray(points, np.float64)
    faces = np.asarray(faces, np.int64)
    owner = np.asarray(owner, np.int64).reshape(-1)
    neighbour = np.asarray(neighbour, np.int64).reshape(-1)
    nF, nIF = len(owner), len(neighbour)
    nIC = int(owner.max()) + 1
    # cellFaces: a cell's owned faces in face order, then the faces it neighbours (cmesh.cpp:3-19)
    nOwned = np.bincount(owner, minlength=nIC)
    cf = np.empty((nIC, 6), np.int64)
    fo = np.argsort(owner, kind='stable')
    start = np.concatenate([[0], np.cumsum(nOwned)[:-1]])
    slot = np.arange(nF) - start[owner[fo]]
    cf[owner[fo], slot] = fo
    fn = np.argsort(neighbour, kind='stable')
    nNb = np.bincount(neighbour, minlength=nIC)
    startN = np.concatenate([[0], np.cumsum(nNb)[:-1]])
    slotN = np.arange(nIF) - startN[neighbour[fn]] + nOwned[neighbour[fn]]
    cf[neighbour[fn], slotN] = fn

    # faces (cmesh.cpp:65-116)
    P = [points[faces[:, j]] for j in range(1, 5)]
    normals = _cross(P[0] - P[1], P[1] - P[2])
    normals = normals / _norm(normals)[:, None]
    fc = ((((0.0 + P[0]) + P[1]) + P[2]) + P[3]) / 4
    area = np.zeros(nF)
    sc = np.zeros((nF, 3))
    for j in range(4):
        pt, nx = P[j], P[(j + 1) % 4]
        avg = 0.0 + ((pt + nx) + fc) / 3
        Ns = _norm(_cross(nx - pt, fc - pt))
        area = area + Ns / 2
        sc = sc + (Ns[:, None] * avg) / 2
    faceCentres = sc / area[:, None]

    # cells (cmesh.cpp:121-152)
    cc = np.zeros((nIC, 3))
    for j in range(6):
        cc = cc + faceCentres[cf[:, j]]
    cc = cc / 6
    vol = np.zeros(nIC)
    scc = np.zeros((nIC, 3))
    for j in range(6):
        f = cf[:, j]
        fcj, A, N = faceCentres[f], area[f], normals[f]
        h = cc - fcj
        aN = A[:, None] * N
        v = ((0.0 + aN[:, 0] * h[:, 0]) + aN[:, 1] * h[:, 1]) + aN[:, 2] * h[:, 2]
        avgC = 3. / 4 * fcj + 1. / 4 * cc
        v = np.abs(v / 3)
        vol = vol + v
        scc = scc + v[:, None] * avgC
    cellCentres = scc / vol[:, None]

    # ghost cells (adFVM/mesh.py:758-819)
    nG = nF - nIF
    nbrFull = np.concatenate([neighbour, np.zeros(nG, np.int64)])
    ccFull = np.concatenate([cellCentres, np.zeros((nG, 3))])
    for name, b in boundary.items():
        s, n = int(b['startFace']), int(b['nFaces'])
        if n == 0:
            continue
        cs = s - nIF + nIC
        nbrFull[s:s + n] = np.arange(cs, cs + n)
        if b['type'] in CYCLIC:
            nb = boundary[b['neighbourPatch']]
            ns = int(nb['startFace'])
            transform = faceCentres[s] - faceCentres[ns]
            ccFull[cs:cs + n] = transform + cellCentres[owner[ns:ns + n]]
        else:
            ccFull[cs:cs + n] = faceCentres[s:s + n]

    # face weights (cmesh.cpp:166-223)
    Pc, Nc = ccFull[owner], ccFull[nbrFull]
    delta = Pc - Nc
    d = _norm(delta)
    deltasUnit = -delta / d[:, None]
    nFv = faceCentres - Nc
    pFv = faceCentres - Pc
    nD = np.abs(((0.0 + nFv[:, 0] * normals[:, 0]) + nFv[:, 1] * normals[:, 1]) + nFv[:, 2] * normals[:, 2])
    pD = np.abs(((0.0 + pFv[:, 0] * normals[:, 0]) + pFv[:, 1] * normals[:, 1]) + pFv[:, 2] * normals[:, 2])
    weights = nD / (nD + pD)
    w1 = ((0.0 + -delta[:, 0] * pFv[:, 0]) + -delta[:, 1] * pFv[:, 1]) + -delta[:, 2] * pFv[:, 2]
    w2 = ((0.0 + delta[:, 0] * nFv[:, 0]) + delta[:, 1] * nFv[:, 1]) + delta[:, 2] * nFv[:, 2]
    dd = ((0.0 + delta[:, 0] * delta[:, 0]) + delta[:, 1] * delta[:, 1]) + delta[:, 2] * delta[:, 2]
    w1 = w1 / dd
    w2 = w2 / dd
    lw = np.stack([w1 / 3, w2 / 3], axis=1)
    qw = np.stack([2. / 3 * pFv + 1. / 3 * (pFv + w1[:, None] * delta),
                   2. / 3 * nFv + 1. / 3 * (nFv - w2[:, None] * delta)], axis=1)

    # cell connectivity (cmesh.cpp:225-263)
    own_c = owner[cf]
    isOwn = own_c == np.arange(nIC)[:, None]
    cellOwner = isOwn.astype(np.int32)
    cellNeighbours = np.where(isOwn, nbrFull[cf], own_c)

    m = types.SimpleNamespace()
    m.boundary = {k: dict(v) for k, v in boundary.items()}
    m.sortedPatches = sorted(boundary.keys())
    m.nInternalCells, m.nInternalFaces, m.nFaces = nIC, nIF, nF
    m.nGhostCells = nG
    m.nCells = nIC + nG
    m.owner = owner.astype(np.int32)
    m.neighbour = nbrFull.astype(np.int32)
    m.normals, m.faceCentres, m.areas = normals, faceCentres, area.reshape(-1, 1)
    m.cellCentres, m.volumes = ccFull, vol.reshape(-1, 1)
    m.deltas, m.deltasUnit, m.weights = d.reshape(-1, 1), deltasUnit, weights.reshape(-1, 1)
    m.linearWeights, m.quadraticWeights = lw, qw
    m.cellFaces = cf.astype(np.int32)
    m.cellOwner = cellOwner
    m.cellNeighbours = cellNeighbours.astype(np.int32)
    m.volumesL = m.volumes[m.owner]
    m.volumesR = m.volumes[m.neighbour[:nIF]]
    return m
