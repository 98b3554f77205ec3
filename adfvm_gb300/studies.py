"""Precision study of the FP32 and mixed forms (the cylinder workload).

Cylinder O-grid 256x128 extruded one cell, inflow Mach 0.3, T = 300 K, p = 1e5 Pa, viscous
no-slip wall, characteristic far field; 2000 steps. FP32 storage and flux/gradient
arithmetic with FP64 objective and sensitivity accumulation ('fp32'), and the same face
arithmetic with the state, RK stages and adjoints in FP64 ('mixed'), against the FP64 run: the
time-averaged drag (templates/cylinder_test.py:9-37) and its sensitivity to a source
perturbation near the cylinder (the perturbation of templates/cylinder_test.py:45-55, scaled
to this mesh) by the checkpointed adjoint sweep.
"""
import time

import numpy as np

from . import cases
from .adjoint import Adjoint
from .solver import RCF


def source_near_cylinder(mesh):
    cc = mesh.cellCentres[:mesh.nInternalCells]
    mid = np.array([-0.6, 0.0, cc[:, 2].mean()])
    G = 1e-3 * np.exp(-np.sum((cc - mid) ** 2, axis=1, keepdims=True) / 0.05 ** 2)
    rhoU = np.zeros((len(cc), 3))
    rhoU[:, 0] = 100 * G[:, 0]
    return (G, rhoU, 2e5 * G)


def precision_study(n_theta=256, n_r=128, nSteps=2000, writeInterval=100, device=0):
    case = cases.cylinder(n_theta, n_r, objective='drag:cylinder')
    mesh = case.build_mesh()
    fields = cases.conservative(case)
    pert = source_near_cylinder(mesh)
    out = {'workload': 'cylinder %dx%d, %d steps, dt %.3e s' % (n_theta, n_r, nSteps, case.dt)}
    res = {}
    for prec in ('fp64', 'fp32', 'mixed'):
        rcf = RCF(mesh, case.bc, objective=case.objective, precision=prec, device=device, **case.config)
        adj = Adjoint(rcf)
        t0 = time.perf_counter()
        sens, a0, rec = adj.run(fields, nSteps, case.dt, writeInterval, perturbations=[pert])
        el = time.perf_counter() - t0
        drag = float(np.mean([float(o) for o in rec['objective']]))
        res[prec] = {'drag': drag, 'sensitivity': sens[0], 'seconds': round(el, 2)}
        rcf.close()
    out.update(res)
    for prec in ('fp32', 'mixed'):
        out['%s_drag_rel_err' % prec] = abs(res[prec]['drag'] - res['fp64']['drag']) / abs(res['fp64']['drag'])
        out['%s_sensitivity_rel_err' % prec] = (abs(res[prec]['sensitivity'] - res['fp64']['sensitivity'])
                                                / abs(res['fp64']['sensitivity']))
    return out
