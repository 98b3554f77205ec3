"""The oracle restatement against trajectories of the reference's own solver code."""
import hashlib

import numpy as np
import pytest
import torch

from oracle import torch_ref
from tests import golden_cases as G

torch.set_num_threads(min(8, torch.get_num_threads()))


def digest(md):
    h = hashlib.sha256()
    for a in md[:4]:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize('name', G.available())
def test_mesh_generator_matches_fixture(name):
    case, g = G.load(name)
    assert digest(case.meshData) == str(g['mesh_digest'])


@pytest.mark.parametrize('name', G.available())
def test_oracle_trajectory_matches_reference(name):
    case, g = G.load(name)
    mesh = case.build_mesh()
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    rho = torch.as_tensor(g['rho_init']).reshape(-1, 1)
    rhoU = torch.as_tensor(g['rhoU_init']).reshape(-1, 3)
    rhoE = torch.as_tensor(g['rhoE_init']).reshape(-1, 1)
    rec = g['record']
    S = None
    if bool(g['with_source']):
        from adfvm_gb300 import cases
        S = [torch.as_tensor(s) for s in cases.source_field(mesh)]
    nSteps = int(g['nSteps'])
    cfl = case.config.get('CFL', 1.2)
    sf = case.config.get('stepFactor', 1.2)
    fixed = case.config.get('fixedTimeStep', False)
    states, record = torch_ref.run(prob, rho, rhoU, rhoE, nSteps, float(g['dt0']), CFL=cfl,
                                   stepFactor=sf, fixed=fixed, S=S)
    record = np.array(record)
    # 1e-12 relative: the tolerance of the plain FP64 path
    for k in range(3):
        assert G.rel_err(record[:, k], rec[:, k]) < 1e-12, (k, record[:4, k], rec[:4, k])
    for s in g['steps']:
        for i, nm in enumerate(['rho', 'rhoU', 'rhoE']):
            e = G.rel_err(states[s][i].numpy(), g['%s_%d' % (nm, s)])
            assert e < 1e-12, (nm, s, e)


def test_oracle_sharp_sod_goes_nonfinite_like_reference():
    """One-cell Sod jump: the reference's first step gives a non-finite CFL sum and a state that
    is non-finite in the cells around the jump; the oracle's step gives the same non-finite
    cells and the same values elsewhere."""
    case, g = G.load_sharp_sod()
    assert digest(case.meshData) == str(g['mesh_digest'])
    mesh = case.build_mesh()
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    x = [torch.as_tensor(g[k + '_init']).reshape(mesh.nInternalCells, -1) for k in ('rho', 'rhoU', 'rhoE')]
    out = prob.step(x[0], x[1], x[2], float(g['dt0']))
    assert not np.isfinite(float(g['dtc'])) and not np.isfinite(float(out[3]))
    for i, nm in enumerate(['rho', 'rhoU', 'rhoE']):
        same, e = G.nonfinite_parity(out[i].numpy(), g[nm + '_1'])
        assert same, nm
        assert e < 1e-12, (nm, e)
