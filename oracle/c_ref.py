"""ctypes driver of the C oracle (oracle/c/afvm_oracle.c). TEST INFRASTRUCTURE ONLY: used
by tests/test_oracle_c.py and as bench.py's timed CPU baseline.

The boundary tables it needs (face kinds, ghost sources, BC codes and values, the per-cell
collate order) are built here in numpy from the mesh and the boundary-condition dicts,
independently of the product's tables.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


class OracleMesh(C.Structure):
    _fields_ = [('nIC', C.c_int), ('nIF', C.c_int), ('nF', C.c_int), ('nG', C.c_int),
                ('own', C.c_void_p), ('nbr', C.c_void_p),
                ('nrm', C.c_void_p), ('area', C.c_void_p), ('dlt', C.c_void_p), ('du', C.c_void_p),
                ('lw', C.c_void_p), ('qw', C.c_void_p), ('wts', C.c_void_p), ('vol', C.c_void_p),
                ('cellFaces', C.c_void_p), ('cellNbr', C.c_void_p), ('cellOwn', C.c_void_p),
                ('fkind', C.c_void_p), ('gsrc', C.c_void_p), ('gkind', C.c_void_p), ('gval', C.c_void_p),
                ('accf', C.c_void_p),
                ('gamma', C.c_double), ('Cp', C.c_double), ('Pr', C.c_double),
                ('muModel', C.c_int), ('mu0', C.c_double), ('muAs', C.c_double), ('muTs', C.c_double),
                ('riemann', C.c_int), ('briemann', C.c_int),
                ('objective', C.c_int), ('objStart', C.c_int), ('objN', C.c_int),
                ('nPlane', C.c_int), ('planeCells', C.c_void_p), ('planeAreas', C.c_void_p),
                ('vn', C.c_double * 3), ('ptin', C.c_double), ('Tw', C.c_double), ('va', C.c_double),
                ('vb', C.c_double), ('nHeat', C.c_int), ('heatFaces', C.c_void_p), ('heatW', C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        from . import build
        path = build.build_c()
        L = C.CDLL(path)
        L.oracle_step.argtypes = [C.POINTER(OracleMesh)] + [C.c_void_p] * 3 + [C.c_double, C.c_void_p] + \
            [C.c_void_p] * 3 + [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]
        L.oracle_step.restype = None
        L.oracle_work_doubles.argtypes = [C.POINTER(OracleMesh)]
        L.oracle_work_doubles.restype = C.c_size_t
        L.oracle_mesh_reorder.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_int] + \
            [C.c_void_p] * 3 + [C.c_void_p] * 6
        L.oracle_mesh_reorder.restype = C.c_int
        L.oracle_adjoint_work_doubles.argtypes = [C.POINTER(OracleMesh)]
        L.oracle_adjoint_work_doubles.restype = C.c_size_t
        L.oracle_adjoint_step.argtypes = [C.POINTER(OracleMesh)] + [C.c_void_p] * 3 + [C.c_double] + \
            [C.c_void_p] * 4 + [C.c_double] + [C.c_void_p] * 5
        L.oracle_adjoint_step.restype = C.c_int
        _lib = L
    return _lib


class COracle(object):
    CYCLIC = ('cyclic', 'slidingPeriodic1D')

    def __init__(self, mesh, bc, config=None, objective='none'):
        cfg = {'Cp': 1004.5, 'gamma': 1.4, 'Pr': 0.7, 'riemannSolver': 'eulerRoe',
               'boundaryRiemannSolver': 'eulerRoe', 'mu': None}
        cfg.update(config or {})
        m = mesh
        nIC, nIF, nF = int(m.nInternalCells), int(m.nInternalFaces), int(m.nFaces)
        nG = nF - nIF
        owner = np.asarray(m.owner, np.int32).reshape(-1)
        fkind = np.full(nG, 3, np.uint8)
        gsrc = np.zeros(nG, np.int32)
        gkind = np.zeros(nG, np.int32)
        gval = np.zeros((nG, 5))
        rank = np.arange(nF, dtype=np.int64)
        pos = nIF
        objStart = objN = 0
        code = {'zeroGradient': 0, 'empty': 0, 'inletOutlet': 0, 'cyclic': 0, 'calculated': 0,
                'fixedValue': 1, 'CBC_UPT': 1, 'symmetryPlane': 2, 'slip': 2, 'CBC_TOTAL_PT': 3}
        for name in m.sortedPatches:
            b = m.boundary[name]
            s, n = int(b['startFace']), int(b['nFaces'])
            g = slice(s - nIF, s - nIF + n)
            kinds = {f: bc[f][name]['type'] for f in ('U', 'T', 'p')}
            char = 'CBC_UPT' in kinds.values() or 'CBC_TOTAL_PT' in kinds.values()
            if b['type'] in self.CYCLIC:
                nb = m.boundary[b['neighbourPatch']]
                gsrc[g] = owner[int(nb['startFace']):int(nb['startFace']) + n]
                fkind[g] = 1
            else:
                gsrc[g] = owner[s:s + n]
                fkind[g] = 2 if char else 3
            cU = code[kinds['U']]
            cT = 0 if kinds['T'] in ('symmetryPlane', 'slip') else code[kinds['T']]
            cp = 0 if kinds['p'] in ('symmetryPlane', 'slip') else code[kinds['p']]
            gkind[g] = cU | (cT << 3) | (cp << 6)
            if kinds['p'] == 'CBC_TOTAL_PT':
                cb = bc['p'][name]
                gval[g, 0:3] = (np.asarray(cb['direction']).reshape(-1, 3) if 'direction' in cb
                                else np.asarray(m.normals).reshape(-1, 3)[s:s + n])
                gval[g, 3] = np.asarray(cb['Tt']).reshape(-1)
                gval[g, 4] = np.asarray(cb['pt']).reshape(-1)
            elif char:
                cb = bc['p'][name]
                gval[g, 0:3] = np.asarray(cb['U0']).reshape(-1, 3)
                gval[g, 3] = np.asarray(cb['T0']).reshape(-1)
                gval[g, 4] = np.asarray(cb['p0']).reshape(-1)
            else:
                for f, cols in (('U', slice(0, 3)), ('T', slice(3, 4)), ('p', slice(4, 5))):
                    if kinds[f] == 'fixedValue':
                        gval[g, cols] = np.asarray(bc[f][name]['value']).reshape(n, -1)
            rank[s:s + n] = pos + np.arange(n)
            pos += n
            if objective == 'drag:' + name:
                objStart, objN = s, n
        cf = np.asarray(m.cellFaces, np.int64).reshape(-1, 6)
        order = np.argsort(rank[cf], axis=1, kind='stable')
        accF = np.take_along_axis(cf, order, axis=1)
        own = owner[accF] == np.arange(nIC)[:, None]
        accf = np.where(own, accF, ~accF).astype(np.int32)
        vane = objective if isinstance(objective, dict) else None
        if vane is not None:
            obj = 4
        else:
            obj = {'none': 0, 'kinetic_energy': 1, 'sum_T': 3}.get(objective, 2 if objective.startswith('drag:') else 0)
        mu = cfg['mu']
        keep = dict(own=owner, nbr=np.asarray(m.neighbour, np.int32).reshape(-1),
                    nrm=np.ascontiguousarray(m.normals, np.float64), area=np.ascontiguousarray(m.areas, np.float64),
                    dlt=np.ascontiguousarray(m.deltas, np.float64), du=np.ascontiguousarray(m.deltasUnit, np.float64),
                    lw=np.ascontiguousarray(m.linearWeights, np.float64),
                    qw=np.ascontiguousarray(m.quadraticWeights, np.float64),
                    wts=np.ascontiguousarray(m.weights, np.float64), vol=np.ascontiguousarray(m.volumes, np.float64),
                    cellFaces=np.ascontiguousarray(m.cellFaces, np.int32),
                    cellNbr=np.ascontiguousarray(m.cellNeighbours, np.int32),
                    cellOwn=np.ascontiguousarray(m.cellOwner, np.int32),
                    fkind=fkind, gsrc=gsrc, gkind=gkind, gval=np.ascontiguousarray(gval), accf=np.ascontiguousarray(accf))
        self.keep = keep
        ptr = lambda k: C.c_void_p(keep[k].ctypes.data)
        self.M = OracleMesh(nIC, nIF, nF, nG, *[ptr(k) for k in ('own', 'nbr', 'nrm', 'area', 'dlt', 'du', 'lw', 'qw',
                                                                 'wts', 'vol', 'cellFaces', 'cellNbr', 'cellOwn',
                                                                 'fkind', 'gsrc', 'gkind', 'gval', 'accf')],
                            float(cfg['gamma']), float(cfg['Cp']), float(cfg['Pr']),
                            1 if mu is None else 0, 0.0 if mu is None else float(mu), 1.4792e-06, 116.,
                            0 if cfg['riemannSolver'] == 'eulerRoe' else 1,
                            0 if cfg['boundaryRiemannSolver'] == 'eulerRoe' else 1, obj, objStart, objN)
        if vane is not None:
            hf, hw = [], []
            # heat faces in the order of objectives/vane.py's patch list
            for name in [p for p in ('pressure', 'suction') if p in vane['heat']] + \
                    [p for p in vane['heat'] if p not in ('pressure', 'suction')]:
                b = m.boundary[name]
                s, n = int(b['startFace']), int(b['nFaces'])
                hf.append(np.arange(s, s + n, dtype=np.int32))
                hw.append(np.asarray(vane['heat'][name], np.float64).reshape(-1))
            keep['planeCells'] = np.ascontiguousarray(vane['planeCells'], np.int32).reshape(-1)
            keep['planeAreas'] = np.ascontiguousarray(vane['planeAreas'], np.float64).reshape(-1)
            keep['heatFaces'] = np.ascontiguousarray(np.concatenate(hf) if hf else np.zeros(1, np.int32), np.int32)
            keep['heatW'] = np.ascontiguousarray(np.concatenate(hw) if hw else np.zeros(1), np.float64)
            M = self.M
            M.nPlane = len(keep['planeCells'])
            M.planeCells, M.planeAreas = ptr('planeCells'), ptr('planeAreas')
            M.vn = (C.c_double * 3)(*[float(x) for x in vane['normal']])
            M.ptin, M.Tw, M.va, M.vb = float(vane['ptin']), float(vane['Tw']), float(vane['a']), float(vane['b'])
            M.nHeat = int(sum(len(h) for h in hf))
            M.heatFaces, M.heatW = ptr('heatFaces'), ptr('heatW')
        self.nIC = nIC
        self.work = np.zeros(lib().oracle_work_doubles(C.byref(self.M)))

    def step(self, rho, rhoU, rhoE, dt, S=None):
        n = self.nIC
        x = [np.ascontiguousarray(a, np.float64).reshape(n, d) for a, d in zip((rho, rhoU, rhoE), (1, 3, 1))]
        out = [np.empty((n, d)) for d in (1, 3, 1)]
        Sp = None if S is None else np.ascontiguousarray(np.concatenate([np.asarray(s).reshape(n, -1) for s in S], 1))
        dtc = C.c_double()
        obj = C.c_double()
        v = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
        lib().oracle_step(C.byref(self.M), v(x[0]), v(x[1]), v(x[2]), float(dt), v(Sp), v(out[0]), v(out[1]),
                          v(out[2]), C.byref(dtc), C.byref(obj), v(self.work))
        return out[0], out[1], out[2], dtc.value, obj.value


def _adjoint_step(self, rho, rhoU, rhoE, dt, seeds, S=None, obja=1.0):
    """The host adjoint baseline (oracle/c/adjoint_host.cpp): VJP of one FP64 step with dt held
    fixed. Returns (rhoa, rhoUa, rhoEa, S_a (nIC x 5))."""
    n = self.nIC
    if not hasattr(self, 'awork'):
        self.awork = np.zeros(lib().oracle_adjoint_work_doubles(C.byref(self.M)))
    x = [np.ascontiguousarray(a, np.float64).reshape(n, d) for a, d in zip((rho, rhoU, rhoE), (1, 3, 1))]
    sd = [np.ascontiguousarray(a, np.float64).reshape(n, d) for a, d in zip(seeds, (1, 3, 1))]
    out = [np.empty((n, d)) for d in (1, 3, 1)]
    Sa = np.empty((n, 5))
    Sp = None if S is None else np.ascontiguousarray(np.concatenate([np.asarray(s).reshape(n, -1) for s in S], 1))
    v = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
    st = lib().oracle_adjoint_step(C.byref(self.M), v(x[0]), v(x[1]), v(x[2]), float(dt), v(Sp), v(sd[0]), v(sd[1]),
                                   v(sd[2]), float(obja), v(out[0]), v(out[1]), v(out[2]), v(Sa), v(self.awork))
    if st != 0:
        raise ValueError('oracle_adjoint_step: objective not supported by the host adjoint')
    return out[0], out[1], out[2], Sa


COracle.adjoint_step = _adjoint_step


def mesh_reorder(meshData):
    """Reverse Cuthill-McKee renumbering of a mesh's cells (oracle/c/reorder_oracle.c).

    meshData = (points, faces, owner, neighbour, boundary) as read from a polyMesh. Returns
    ((points, faces', owner', neighbour', boundary), cellNew, faceOld, (bandwidth before,
    after)); cellNew[old cell] = new id, faceOld[new face] = old face (~old where flipped)."""
    points, faces, owner, neighbour, boundary = meshData
    faces = np.ascontiguousarray(faces, np.int32)
    owner = np.ascontiguousarray(owner, np.int32).reshape(-1)
    neighbour = np.ascontiguousarray(neighbour, np.int32).reshape(-1)
    nF, nIF = len(owner), len(neighbour)
    nIC = int(owner.max()) + 1
    names = list(boundary.keys())
    start = np.array([int(boundary[p]['startFace']) for p in names], np.int32)
    count = np.array([int(boundary[p]['nFaces']) for p in names], np.int32)
    partner = np.array([int(boundary[boundary[p]['neighbourPatch']]['startFace'])
                        if boundary[p]['type'] in COracle.CYCLIC else -1 for p in names], np.int32)
    fo = np.empty_like(faces)
    oo = np.empty_like(owner)
    no = np.empty_like(neighbour)
    cn = np.empty(nIC, np.int32)
    fold = np.empty(nF, np.int32)
    bw = np.zeros(2, np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = lib().oracle_mesh_reorder(nIC, nF, nIF, p(faces), p(owner), p(neighbour), len(names), p(start), p(count),
                                   p(partner), p(fo), p(oo), p(no), p(cn), p(fold), p(bw))
    if rc != 0:
        raise ValueError('oracle_mesh_reorder: index out of range or a cell with more than six edges')
    return (points, fo, oo, no, boundary), cn, fold, (int(bw[0]), int(bw[1]))
