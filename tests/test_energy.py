"""Adjoint energy (cmesh.computeEnergy): the oracle restatement against the reference's own
compiled function (tests/golden/energy.npz), and the GPU kernel against both."""
import numpy as np
import pytest

from adfvm_gb300 import cases
from oracle import torch_ref

GOLD = np.load(__import__('os').path.join(__import__('os').path.dirname(__file__), 'golden', 'energy.npz'))
CASES = {'box6': lambda: cases.box(6, objective='kinetic_energy'), 'cyl16x8': lambda: cases.cylinder(16, 8)}


def _fields(name):
    return [GOLD[name + '/' + k] for k in ('rhoa', 'rhoUa', 'rhoEa', 'rho', 'rhoU', 'rhoE')]


@pytest.mark.parametrize('name', list(CASES))
def test_oracle_energy_matches_reference(name):
    mesh = CASES[name]().build_mesh()
    e = torch_ref.adjoint_energy(mesh.volumes, 1.4, *_fields(name))
    assert abs(e - float(GOLD[name + '/energy'])) <= 1e-12 * abs(float(GOLD[name + '/energy']))


@pytest.mark.gpu
@pytest.mark.parametrize('name', list(CASES))
def test_gpu_energy_matches_reference(name):
    import torch
    from adfvm_gb300.solver import RCF
    case = CASES[name]()
    rcf = RCF(case.build_mesh(), case.bc, objective=case.objective, **case.config)
    f = [torch.as_tensor(a).cuda() for a in _fields(name)]
    e = rcf.adjoint_energy(f[:3], f[3:])
    assert abs(e - float(GOLD[name + '/energy'])) <= 1e-12 * abs(float(GOLD[name + '/energy']))
