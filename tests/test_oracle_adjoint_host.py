"""The host adjoint baseline (oracle/c/adjoint_host.cpp: the CPU adjoint step bench.py times)
against torch autograd of the oracle, the exact VJP of the same discrete step: within 1e-12
(max|x-ref|/max|ref| per field) on the golden cases and the tiny meshes."""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from oracle import torch_ref
from oracle.c_ref import COracle
from tests import golden_cases as G
from tests.test_gpu_adjoint import _seeds, _setup

torch.set_num_threads(min(8, torch.get_num_threads()))


def _check(case, mesh, x, S, dt, label, seed=7):
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, seed)
    St = None if S is None else [torch.as_tensor(s) for s in S]
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], dt, St, seeds, obja=1.0)
    co = COracle(mesh, case.bc, case.config, case.objective)
    a = co.adjoint_step(*[t.numpy() for t in x], dt, [t.numpy() for t in seeds],
                        S=None if S is None else [np.asarray(s) for s in S], obja=1.0)
    for i in range(3):
        e = G.rel_err(a[i], ref[i].numpy())
        assert e < 1e-12, '%s field %d: rel err %.3e' % (label, i, e)
    e = G.rel_err(a[3], ref[3].numpy())
    assert e < 1e-12, '%s source: rel err %.3e' % (label, e)


@pytest.mark.parametrize('name', ['box8', 'cyl32x16', 'sod200_sym_lf', 'box6_inviscid_sumT', 'sod1000',
                                  'duct100_totalpt', 'duct60_totalpt_normals'])
def test_host_adjoint_matches_autograd(name):
    case, mesh, x, S, dt = _setup(name)
    _check(case, mesh, x, S, dt, name)


def test_host_adjoint_on_the_benchmark_recipe():
    case = cases.box(16, objective='kinetic_energy')
    mesh = case.build_mesh()
    x = [torch.as_tensor(a) for a in cases.conservative(case)]
    _check(case, mesh, x, None, case.dt, 'box16')
