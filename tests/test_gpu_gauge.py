"""The gauge state of FP32 cell records ('fp32' and 'mixed' contexts): records hold p - p_g and
T - T_g and the face fluxes leave out p_g N and H_g times the mass flux (afvm_set_gauge).

* the default gauge is the far field's p, T and total enthalpy (afvm_ctx_create);
* over 50 steps of the cylinder the mixed form with the gauge is much closer to FP64 than with
  a zero gauge (the form FP32 records had before), and both are within 1e-5;
* what leaves the records - the boundary map, the objective-stage primitives handed to an
  objective function - is absolute: the same as the FP64 context's to FP32 rounding.
"""
import math

import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from adfvm_gb300.solver import RCF
from tests import objective_fns as O

pytestmark = pytest.mark.gpu


def _cyl():
    case = cases.cylinder(64, 32, objective='drag:cylinder')
    mesh = case.build_mesh()
    x = [torch.as_tensor(np.asarray(a).reshape(mesh.nInternalCells, -1)) for a in cases.conservative(case)]
    return case, mesh, x


def test_default_gauge_is_the_far_field():
    case, mesh, _ = _cyl()
    r = RCF(mesh, case.bc, objective=case.objective, precision='mixed', **case.config)
    U0 = 0.3 * math.sqrt(cases.GAMMA * cases.R_GAS * 300.0)
    H = float(np.float32(1004.5 * 300.0 + 0.5 * U0 * U0))
    assert r.gauge == (1e5, 300.0, H), r.gauge
    box = cases.box(8)
    rb = RCF(box.build_mesh(), box.bc, objective=box.objective, precision='fp32', **box.config)
    assert rb.gauge == (0.0, 0.0, 0.0)          # a periodic box fixes no boundary value
    rb.close()
    r.close()


def _run(case, mesh, x, precision, gauge=None, n=50):
    r = RCF(mesh, case.bc, objective=case.objective, precision=precision, gauge=gauge, **case.config)
    td = torch.float32 if r.dtype == np.float32 else torch.float64
    y = [t.to(td).cuda() for t in x]
    for _ in range(n):
        y = list(r.step(y[0], y[1], y[2], case.dt)[:3])
    out = [t.double().cpu().numpy() for t in y]
    r.close()
    return out


def test_gauge_brings_mixed_closer_to_fp64():
    case, mesh, x = _cyl()
    ref = _run(case, mesh, x, 'fp64')
    g = _run(case, mesh, x, 'mixed')
    z = _run(case, mesh, x, 'mixed', gauge=(0.0, 0.0, 0.0))
    for i, name in enumerate(('rho', 'rhoU', 'rhoE')):
        scale = np.abs(ref[i]).max()
        eg = np.abs(g[i] - ref[i]).max() / scale
        ez = np.abs(z[i] - ref[i]).max() / scale
        assert eg <= 1e-5 and ez <= 1e-5, (name, eg, ez)
        assert eg < 0.75 * ez, '%s: gauge %.3e, no gauge %.3e' % (name, eg, ez)


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_gauge_on_warped_faces(precision):
    """The jittered periodic box, whose warped faces leave each cell's sum of A N nonzero (the
    reference takes a face's normal from three of its points): with the gauge of its initial
    field, 20 steps and an adjoint step stay as close to FP64 as without one."""
    case = cases.box(16, objective='kinetic_energy')
    mesh = case.build_mesh()
    x = [torch.as_tensor(np.asarray(a).reshape(mesh.nInternalCells, -1)) for a in cases.conservative(case)]

    def run(prec, gauge):
        r = RCF(mesh, case.bc, objective=case.objective, precision=prec, gauge=gauge, **case.config)
        td = torch.float32 if r.dtype == np.float32 else torch.float64
        y = [t.to(td).cuda() for t in x]
        for _ in range(20):
            y = list(r.step(y[0], y[1], y[2], case.dt)[:3])
        a = r.adjoint_step(y[0], y[1], y[2], case.dt, [torch.ones_like(t) for t in y], obja=1.0)
        out = [t.double().cpu().numpy() for t in y] + [t.double().cpu().numpy() for t in a[:3]]
        r.close()
        return out

    ref = run('fp64', None)
    g = run(precision, cases.gauge(case))
    assert cases.gauge(case)[0] > 1e5
    for i in range(6):
        e = np.abs(g[i] - ref[i]).max() / np.abs(ref[i]).max()
        assert e <= 1e-5, 'field %d: rel err %.3e' % (i, e)


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_values_leaving_the_records_are_absolute(precision):
    case, mesh, x = _cyl()
    a = RCF(mesh, case.bc, objective=case.objective, **case.config)
    b = RCF(mesh, case.bc, objective=O.drag('cylinder'), precision=precision, **case.config)
    td = torch.float32 if b.dtype == np.float32 else torch.float64
    xa = [t.cuda() for t in x]
    xb = [t.to(td).cuda() for t in x]
    ga = a.boundary_values(*xa).double().cpu().numpy()
    gb = b.boundary_values(*xb).double().cpu().numpy()
    err = np.abs(gb - ga).max(axis=0) / np.abs(ga).max(axis=0).clip(1.0)
    assert (err < 1e-6).all(), err
    oa = float(a.step(*xa, case.dt)[4])
    ob = float(b.step(*xb, case.dt)[4])
    assert abs(ob - oa) <= 1e-5 * abs(oa), (oa, ob)
    a.close()
    b.close()


def test_gauge_and_tape_arguments_are_checked():
    """afvm_set_gauge rejects a non-finite gauge state; a tape that is not 16-byte aligned is
    rejected before any launch (the tape's cell records are read with 16-byte loads)."""
    from adfvm_gb300 import _lib as L
    case, mesh, x = _cyl()
    r = RCF(mesh, case.bc, objective=case.objective, precision='fp64', **case.config)
    assert L.lib().afvm_set_gauge(r._ctx, float('nan'), 300.0, 3e5) == L.AFVM_ERR_BAD_ARG
    assert L.lib().afvm_set_gauge(r._ctx, 1e5, float('inf'), 3e5) == L.AFVM_ERR_BAD_ARG
    xd = [t.cuda() for t in x]
    st = r.stage_buffer()
    tape = r.tape_buffer()
    shifted = torch.empty(tape.numel() + 1, dtype=tape.dtype, device=tape.device)[1:]
    with pytest.raises(L.AfvmError) as ei:
        r.step(xd[0], xd[1], xd[2], case.dt, stages=st, tape=shifted)
    assert ei.value.status == L.AFVM_ERR_BAD_ARG
    r.step(xd[0], xd[1], xd[2], case.dt, stages=st, tape=tape)     # the aligned one runs
    r.close()
