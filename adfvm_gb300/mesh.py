"""Mesh container with the reference Mesh's attributes and tensor order.

``Mesh.build(meshData)`` mirrors adFVM/mesh.py:84-127: sizes (populateSizes, 517-523), patch
split and alphabetical ``sortedPatches`` (238-249, 100-101), the native geometry build
(``afvm_mesh_build``, restating adFVM/cpp/cmesh.cpp:3-270 and createGhostCells 758-819),
``volumesL/volumesR`` (108-109) and the counts nRemoteCells/nLocalFaces/nGhostCells
(110-112). ``getTensor()``/``getScalar()`` return the lists in the order the reference's
compiled step function takes them (mesh.py:27-37, 870-881).
"""
import copy
import ctypes as C

import numpy as np

from . import _lib as L

# patch types grouped as in adFVM/config.py:203-206
PROCESSOR_PATCHES = ['processor', 'processorCyclic']
CYCLIC_PATCHES = ['cyclic', 'slidingPeriodic1D']
COUPLED_PATCHES = CYCLIC_PATCHES + PROCESSOR_PATCHES
DEFAULT_PATCHES = COUPLED_PATCHES + ['symmetryPlane', 'empty']


class Mesh(object):
    intFields = ['owner', 'neighbour', 'cellFaces', 'cellNeighbours', 'cellOwner']
    gradFields = ['areas', 'volumesL', 'volumesR', 'weights', 'deltas', 'normals', 'deltasUnit',
                  'linearWeights', 'quadraticWeights', 'volumes']
    BCFields = ['startFace', 'nFaces', 'cellStartFace']
    constants = ['nCells', 'nFaces', 'nInternalCells', 'nInternalFaces',
                 'nLocalCells', 'nRemoteCells', 'nLocalFaces', 'nGhostCells']

    def __init__(self):
        self.boundary = {}

    @classmethod
    def create(cls, meshData, device=None):
        """device: None builds the geometry on the host (afvm_mesh_build, OpenMP); a CUDA
        ordinal builds it there (afvm_mesh_build_device) - the same bits either way."""
        self = cls()
        self.build(meshData, device)
        return self

    def build(self, meshData, device=None):
        points, faces, owner, neighbour, boundary = meshData
        self.points = np.ascontiguousarray(points, np.float64)
        self.faces = np.ascontiguousarray(faces, np.int32)
        self.owner = np.ascontiguousarray(owner, np.int32)
        neighbour = np.ascontiguousarray(neighbour, np.int32)
        self.boundary = copy.deepcopy(boundary)
        # sizes (adFVM/mesh.py:517-523)
        self.nInternalFaces = len(neighbour)
        self.nFaces = len(self.owner)
        self.nBoundaryFaces = self.nFaces - self.nInternalFaces
        self.nInternalCells = int(np.max(self.owner)) + 1
        self.nGhostCells = self.nBoundaryFaces
        self.nCells = self.nInternalCells + self.nGhostCells
        # patches (adFVM/mesh.py:238-249)
        patchIDs = sorted(self.boundary.keys(), key=lambda x: (self.boundary[x]['startFace'], self.boundary[x]['nFaces']))
        self.localPatches, self.remotePatches = [], []
        for patchID in patchIDs:
            b = self.boundary[patchID]
            b['cellStartFace'] = b['startFace'] - self.nInternalFaces + self.nInternalCells
            if b['type'] in PROCESSOR_PATCHES:
                self.remotePatches.append(patchID)
            else:
                self.localPatches.append(patchID)
        if self.remotePatches:
            raise NotImplementedError('processor patches: one partition per GPU is supported')
        self.patches = self.localPatches + self.remotePatches
        self.sortedPatches = sorted(self.localPatches)
        self.defaultBoundary = self.getDefaultBoundary()
        if device is None:
            self._geometry(neighbour)
        else:
            self._geometry_device(neighbour, device)
        self.volumesL = self.volumes[self.owner]
        self.volumesR = self.volumes[self.neighbour[:self.nInternalFaces]]
        self.nRemoteCells = self.nCells - self.nLocalCells
        self.nLocalFaces = self.nLocalCells - self.nInternalCells + self.nInternalFaces
        self.nGhostCells = self.nCells - self.nInternalCells
        return self

    def patchTable(self, order):
        """afvm_patch array for the given patch-name order (cyclic partners as indices)."""
        idx = {p: i for i, p in enumerate(order)}
        arr = (L.Patch * max(1, len(order)))()
        for i, p in enumerate(order):
            b = self.boundary[p]
            kind = L.AFVM_PATCH_CYCLIC if b['type'] in CYCLIC_PATCHES else (
                L.AFVM_PATCH_PROCESSOR if b['type'] in PROCESSOR_PATCHES else L.AFVM_PATCH_PLAIN)
            nb = idx[b['neighbourPatch']] if kind == L.AFVM_PATCH_CYCLIC else -1
            arr[i] = L.Patch(b['startFace'], b['nFaces'], kind, nb)
        return arr

    def _geometry(self, neighbour):
        nF, nIF, nIC, nC = self.nFaces, self.nInternalFaces, self.nInternalCells, self.nCells
        patches = self.patchTable(self.patches)
        mi = L.MeshIn(len(self.points), L.dptr(self.points), nF, L.iptr(self.faces), nIF,
                      L.iptr(self.owner), L.iptr(neighbour), nIC, len(self.patches), patches)
        self.normals = np.zeros((nF, 3))
        self.faceCentres = np.zeros((nF, 3))
        self.areas = np.zeros((nF, 1))
        self.cellCentres = np.zeros((nC, 3))
        self.volumes = np.zeros((nIC, 1))
        self.neighbour = np.zeros(nF, np.int32)
        self.deltas = np.zeros((nF, 1))
        self.deltasUnit = np.zeros((nF, 3))
        self.weights = np.zeros((nF, 1))
        self.linearWeights = np.zeros((nF, 2))
        self.quadraticWeights = np.zeros((nF, 2, 3))
        self.cellFaces = np.zeros((nIC, 6), np.int32)
        self.cellOwner = np.zeros((nIC, 6), np.int32)
        self.cellNeighbours = np.zeros((nIC, 6), np.int32)
        self.cellNeighboursMatOp = np.zeros((nIC, 6), np.int32)
        mo = L.MeshOut(L.dptr(self.normals), L.dptr(self.faceCentres), L.dptr(self.areas),
                       L.dptr(self.cellCentres), L.dptr(self.volumes), L.iptr(self.neighbour),
                       L.dptr(self.deltas), L.dptr(self.deltasUnit), L.dptr(self.weights),
                       L.dptr(self.linearWeights), L.dptr(self.quadraticWeights),
                       L.iptr(self.cellFaces), L.iptr(self.cellOwner), L.iptr(self.cellNeighbours),
                       L.iptr(self.cellNeighboursMatOp), 0)
        L.check(L.lib().afvm_mesh_build(mi, mo), what='afvm_mesh_build')
        self.nLocalCells = int(mo.nLocalCells)

    def getDefaultBoundary(self):
        """Boundary types of gradient fields (adFVM/mesh.py:702-711)."""
        boundary = {}
        for patchID in self.boundary:
            t = self.boundary[patchID]['type']
            boundary[patchID] = {'type': t if t in DEFAULT_PATCHES else 'zeroGradient'}
        return boundary

    def getTensor(self):
        return [getattr(self, a) for a in Mesh.gradFields] + [getattr(self, a) for a in Mesh.intFields]

    def getScalar(self):
        out = [getattr(self, a) for a in Mesh.constants]
        for patchID in self.sortedPatches:
            out.extend([self.boundary[patchID][a] for a in Mesh.BCFields])
        return out

    def cellRange(self, patchID):
        b = self.boundary[patchID]
        s = b['startFace'] - self.nInternalFaces + self.nInternalCells
        return s, s + b['nFaces']

    def tensorsStruct(self):
        """afvm_mesh_tensors view of this mesh (arrays must stay alive while in use)."""
        keep = {}
        for a in Mesh.gradFields:
            keep[a] = np.ascontiguousarray(getattr(self, a), np.float64)
        for a in Mesh.intFields:
            keep[a] = np.ascontiguousarray(getattr(self, a), np.int32)
        patches = self.patchTable(self.sortedPatches)
        mt = L.MeshTensors(*([L.dptr(keep[a]) for a in Mesh.gradFields] + [L.iptr(keep[a]) for a in Mesh.intFields]
                             + [getattr(self, a) for a in Mesh.constants] + [len(self.sortedPatches), patches]))
        return mt, (keep, patches)

    def _geometry_device(self, neighbour, device):
        import torch
        nF, nIF, nIC, nC = self.nFaces, self.nInternalFaces, self.nInternalCells, self.nCells
        dev = torch.device('cuda', device)
        up = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)
        points, faces, owner, nbr = up(self.points), up(self.faces), up(self.owner), up(neighbour)
        shapes = {'normals': ((nF, 3), torch.float64), 'faceCentres': ((nF, 3), torch.float64),
                  'areas': ((nF, 1), torch.float64), 'cellCentres': ((nC, 3), torch.float64),
                  'volumes': ((nIC, 1), torch.float64), 'neighbour': ((nF,), torch.int32),
                  'deltas': ((nF, 1), torch.float64), 'deltasUnit': ((nF, 3), torch.float64),
                  'weights': ((nF, 1), torch.float64), 'linearWeights': ((nF, 2), torch.float64),
                  'quadraticWeights': ((nF, 2, 3), torch.float64), 'cellFaces': ((nIC, 6), torch.int32),
                  'cellOwner': ((nIC, 6), torch.int32), 'cellNeighbours': ((nIC, 6), torch.int32),
                  'cellNeighboursMatOp': ((nIC, 6), torch.int32)}
        out = {k: torch.empty(s, dtype=t, device=dev) for k, (s, t) in shapes.items()}
        vp = lambda t: C.c_void_p(t.data_ptr())
        patches = self.patchTable(self.patches)
        mi = L.MeshIn(len(self.points), C.cast(vp(points), L._d), nF, C.cast(vp(faces), L._i), nIF,
                      C.cast(vp(owner), L._i), C.cast(vp(nbr), L._i), nIC, len(self.patches), patches)
        d = lambda k: C.cast(vp(out[k]), L._d)
        i = lambda k: C.cast(vp(out[k]), L._i)
        mo = L.MeshOut(d('normals'), d('faceCentres'), d('areas'), d('cellCentres'), d('volumes'), i('neighbour'),
                       d('deltas'), d('deltasUnit'), d('weights'), d('linearWeights'), d('quadraticWeights'),
                       i('cellFaces'), i('cellOwner'), i('cellNeighbours'), i('cellNeighboursMatOp'), 0)
        stream = torch.cuda.current_stream(dev).cuda_stream
        L.check(L.lib().afvm_mesh_build_device(mi, mo, C.c_void_p(stream)), what='afvm_mesh_build_device')
        for k, t in out.items():
            setattr(self, k, t.cpu().numpy())
        self.nLocalCells = int(mo.nLocalCells)


def reorder(meshData, device=0):
    """Bandwidth (reverse Cuthill-McKee) renumbering of a mesh's cells on the GPU
    (afvm_mesh_reorder_device), for meshes admitted in any cell order.

    meshData = (points, faces, owner, neighbour, boundary). Returns (meshData', cellNew,
    faceOld, (bandwidth before, after)): cellNew[old cell] = new id (a field ``x`` of the old
    mesh is ``x_new[cellNew] = x`` on the new one), faceOld[new face] = old face, ~old where
    the face was flipped. Points and boundary patches are unchanged."""
    import torch
    points, faces, owner, neighbour, boundary = meshData
    faces = np.ascontiguousarray(faces, np.int32)
    owner = np.ascontiguousarray(owner, np.int32).reshape(-1)
    neighbour = np.ascontiguousarray(neighbour, np.int32).reshape(-1)
    nF, nIF = len(owner), len(neighbour)
    nIC = int(owner.max()) + 1
    m = Mesh()
    m.boundary = copy.deepcopy(boundary)
    order = sorted(m.boundary.keys(), key=lambda x: (m.boundary[x]['startFace'], m.boundary[x]['nFaces']))
    patches = m.patchTable(order)
    dev = torch.device('cuda', device)
    up = lambda a: torch.as_tensor(a).to(dev)
    df, do, dn = up(faces), up(owner), up(neighbour if nIF > 0 else np.zeros(1, np.int32))
    fo = torch.empty_like(df)
    oo = torch.empty_like(do)
    no = torch.empty_like(dn)
    cn = torch.empty(nIC, dtype=torch.int32, device=dev)
    fold = torch.empty(nF, dtype=torch.int32, device=dev)
    ip = lambda t: C.cast(C.c_void_p(t.data_ptr()), L._i)
    mi = L.MeshIn(0, None, nF, ip(df), nIF, ip(do), ip(dn), nIC, len(order), patches)
    bw = (C.c_int32 * 2)()
    stream = torch.cuda.current_stream(dev).cuda_stream
    L.check(L.lib().afvm_mesh_reorder_device(mi, ip(fo), ip(oo), ip(no), ip(cn), ip(fold),
                                             C.cast(bw, L._i), C.c_void_p(stream)),
            what='afvm_mesh_reorder_device')
    out = (np.asarray(points), fo.cpu().numpy(), oo.cpu().numpy(), no.cpu().numpy()[:nIF], copy.deepcopy(boundary))
    return out, cn.cpu().numpy(), fold.cpu().numpy(), (int(bw[0]), int(bw[1]))
