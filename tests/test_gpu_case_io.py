"""Case directories on the GPU path: RCF.fromCase / readFields / run with writes / status.pkl
resume, and the boundary map (afvm_boundary_values) against the oracle's ghost rows.

Tolerances: the ghost values are FP64 and within 1e-13 relative of the oracle's; a run resumed
from the written files matches an uninterrupted run within 1e-10 relative (the files hold the
primitive fields, so a resume goes through one primitive -> conservative round trip).
"""
import os

import numpy as np
import pytest
import torch

from adfvm_gb300 import cases, foam
from adfvm_gb300.solver import RCF
from oracle import torch_ref

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _write_case(d, case):
    foam.write_mesh(d, case.meshData)
    for name, val in (('U', case.U), ('T', case.T), ('p', case.p)):
        foam.write_field(os.path.join(d, '0'), name, val, case.bc[name])


@pytest.mark.parametrize('make', [lambda: cases.cylinder(32, 16), lambda: cases.duct(40), lambda: cases.box(8),
                                  lambda: cases.sod(60, side='symmetryPlane')])
def test_boundary_values_match_oracle(make):
    case = make()
    m = case.build_mesh()
    rcf = RCF(m, case.bc, objective=case.objective, **case.config)
    x = cases.conservative(case)
    rng = np.random.default_rng(1)
    x = [a * (1 + 0.01 * rng.standard_normal(a.shape)) for a in x]       # a non-uniform state
    xd = [torch.as_tensor(np.ascontiguousarray(a), device='cuda') for a in x]
    ghost = rcf.boundary_values(*xd).cpu().numpy()
    prob = torch_ref.Problem(m, case.bc, case.config, case.objective)
    U, T, p = prob.primitive(*[torch.as_tensor(a) for a in x])
    gU, gT, gp = [t.numpy()[m.nInternalCells:] for t in prob.ghosts(U, T, p)]
    assert ghost.shape == (m.nGhostCells, 5)
    assert _rel(ghost[:, 0:3], gU) < 1e-13 and _rel(ghost[:, 3:4], gT) < 1e-13 and _rel(ghost[:, 4:5], gp) < 1e-13


def test_run_writes_and_resumes(tmp_path):
    d = str(tmp_path)
    case = cases.cylinder(32, 16)
    _write_case(d, case)
    rcf = RCF.fromCase(d, objective=case.objective, **case.config)
    fields = rcf.readFields(0.0)
    x0 = cases.conservative(case)
    for a, b in zip(fields, x0):
        assert _rel(a, b) < 1e-15
    nW, nS = 5, 10
    result, record = rcf.run(fields, nS, case.dt, writeInterval=nW)
    st = rcf.readStatusFile()
    assert st[0] == nS and st[3] == result
    t5 = 0.0
    for _ in range(nW):
        t5 = round(t5 + case.dt, 12)          # the loop's time update (solver.py:355-358)
    assert os.path.exists(os.path.join(d, foam.time_name(t5), 'U'))
    for name in ('rho', 'rhoU', 'rhoE', 'U', 'T', 'p'):
        assert os.path.exists(os.path.join(d, foam.time_name(st[1]), name)), name
    # the patch values written are the ghost cells of the written state
    m = rcf.mesh
    internal = {}
    bnd = {}
    for name in ('U', 'T', 'p'):
        internal[name], bnd[name] = foam.read_field(os.path.join(d, foam.time_name(st[1])), name, m.boundary,
                                                    m.nInternalCells)
    prob = torch_ref.Problem(m, case.bc, case.config, case.objective)
    gU, gT, gp = [t.numpy() for t in prob.ghosts(*[torch.as_tensor(internal[k]) for k in ('U', 'T', 'p')])]
    s = m.boundary['farfield']['startFace'] - m.nInternalFaces + m.nInternalCells
    n = m.boundary['farfield']['nFaces']
    assert bnd['p']['farfield']['type'] == 'CBC_UPT'
    assert _rel(bnd['p']['farfield']['value'], gp[s:s + n]) < 1e-12
    assert 'value' in bnd['U']['cylinder'] and np.all(bnd['U']['cylinder']['value'] == 0.0)
    # resume from the files at step 5 and run on to step 10
    rcf2 = RCF.fromCase(d, objective=case.objective, **case.config)
    f5 = rcf2.readFields(t5)
    res2, _ = rcf2.run(f5, nS, case.dt, startTime=t5, startIndex=nW, result=sum(r[2] for r in record[:nW]))
    sols_ref, _ = rcf.run(x0, nS, case.dt, mode='forward')
    assert abs(res2 - result) <= 1e-10 * abs(result)
    final = rcf2.readFields(st[1])
    for a, b in zip(final, sols_ref[-1]):
        assert _rel(a, b) < 1e-10
