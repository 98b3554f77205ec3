"""Set-up of the turbine-vane design objective (adFVM/objectives/vane.py): a pressure loss over
the cells cut by a plane plus a weighted wall heat transfer,

    J = a * sum_c (ptin - pt_c) rhoUn_c A_c / ptin / sum_c rhoUn_c A_c
      + b * sum_f k (Tw - T_own(f)) / delta_f A_f w_f / sum_f A_f w_f

with rho = p/(Cv T (gamma-1)), rhoUn = rho U.n, M^2 = |U|^2/c^2, c^2 = gamma p/rho,
pt = p (1 + (gamma-1)/2 M^2)^(gamma/(gamma-1)) and k = Cp mu(Tw)/Pr (vane.py:7-60, 118-131).
The device evaluates J and its gradient (afvm_set_objective_vane); this module computes the
mesh-only inputs the reference's ``getPlane``/``getWeights`` put in ``solver.extraArgs``
(vane.py:23-37, 68-80): the cut cells with their cut areas, and the wall weights.

The cut cells and areas are computed here geometrically (the polygon in which the plane meets
each cell); the reference obtains them from ``compat.intersectPlane``, a compiled helper
(adFVM/compat/cfuncs.pyx:20-107). A host that has that helper passes its output instead
(``plane=(cells, areas)``), as the reference's input list does.
"""
import numpy as np

# the constants of adFVM/objectives/vane.py
POINT = (0.052641, -0.1, 0.005)          # getPlane (vane.py:26)
NORMAL = (1.0, 0.0, 0.0)                 # vane.py:27, 41, 53
PTIN = 175158.0                          # objectivePressureLoss (vane.py:51)
TW = 300.0                               # objectiveHeatTransfer (vane.py:17)
A_PL, B_HT = 0.4, 0.0                    # objective (vane.py:118-120)
HEAT_PATCHES = ('pressure', 'suction')   # vane.py:66
# getWeights (vane.py:72-77): faces with centre x >= x_min and y <= y_max count
WEIGHT_BOX = {'pressure': (0.033757, 0.04692), 'suction': (0.035241, 0.044337)}


def plane_cells(mesh, point=POINT, normal=NORMAL, tol=0.0):
    """Internal cells the plane through ``point`` with ``normal`` cuts, and the area of each
    cut (the polygon where the plane meets the cell), as (cells int32 (n,), areas (n, 1))."""
    point = np.asarray(point, np.float64)
    nrm = np.asarray(normal, np.float64)
    nrm = nrm / np.linalg.norm(nrm)
    P = np.asarray(mesh.points, np.float64)
    d = (P - point) @ nrm
    faces = np.asarray(mesh.faces)[:, 1:5]
    nIC = int(mesh.nInternalCells)
    cf = np.asarray(mesh.cellFaces)[:nIC]
    fpts = faces[cf]                                    # (nIC, 6, 4) point ids
    dc = d[fpts.reshape(nIC, -1)]
    cut = np.where((dc.max(axis=1) > tol) & (dc.min(axis=1) < -tol))[0]
    # an orthonormal basis of the plane for the polygon area
    e1 = np.cross(nrm, [1.0, 0.0, 0.0] if abs(nrm[0]) < 0.9 else [0.0, 1.0, 0.0])
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(nrm, e1)
    areas = np.zeros(len(cut))
    for n, c in enumerate(cut):
        q = fpts[c]                                     # (6, 4)
        a, b = q.reshape(-1), np.roll(q, -1, axis=1).reshape(-1)   # the 24 face edges
        da, db = d[a], d[b]
        hit = (da * db) < 0
        t = da[hit] / (da[hit] - db[hit])
        X = P[a[hit]] + t[:, None] * (P[b[hit]] - P[a[hit]])
        on = P[np.unique(np.concatenate([a[da == 0], b[db == 0]]))]
        X = np.concatenate([X, on]) if len(on) else X
        uv = np.stack([(X - point) @ e1, (X - point) @ e2], axis=1)
        uv = np.unique(np.round(uv, 15), axis=0)
        if len(uv) < 3:
            continue
        ctr = uv.mean(axis=0)
        ang = np.arctan2(uv[:, 1] - ctr[1], uv[:, 0] - ctr[0])
        uv = uv[np.argsort(ang)]
        x, y = uv[:, 0], uv[:, 1]
        areas[n] = 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))
    keep = areas > 0
    return cut[keep].astype(np.int32), areas[keep].reshape(-1, 1)


def heat_weights(mesh, patches=HEAT_PATCHES, box=WEIGHT_BOX):
    """{patch: weights (nFaces, 1)} of getWeights (vane.py:68-80); patches absent from the
    mesh are skipped."""
    out = {}
    for p in patches:
        if p not in mesh.boundary:
            continue
        b = mesh.boundary[p]
        s, n = int(b['startFace']), int(b['nFaces'])
        cen = np.asarray(mesh.faceCentres)[s:s + n]
        xmin, ymax = box[p]
        out[p] = (np.logical_and(cen[:, 0] >= xmin, cen[:, 1] <= ymax) * 1.0).reshape(-1, 1)
    return out


def options(mesh, plane=None, point=POINT, normal=NORMAL, ptin=PTIN, Tw=TW, a=A_PL, b=B_HT, heat=None):
    """The full objective description: {'kind': 'vane', 'planeCells', 'planeAreas', 'normal',
    'ptin', 'heat' {patch: weights}, 'Tw', 'a', 'b'}."""
    cells, areas = plane if plane is not None else plane_cells(mesh, point, normal)
    return {'kind': 'vane', 'planeCells': np.asarray(cells, np.int32).reshape(-1),
            'planeAreas': np.asarray(areas, np.float64).reshape(-1, 1),
            'normal': np.asarray(normal, np.float64).reshape(3), 'ptin': float(ptin),
            'heat': heat if heat is not None else heat_weights(mesh), 'Tw': float(Tw), 'a': float(a), 'b': float(b)}
