"""Objectives given as functions (tests/objective_fns.py) in the oracle: the same values and
the same autograd adjoints as the built-in kinds they restate."""
import torch

from oracle import torch_ref
from tests import golden_cases as G
from tests import objective_fns as O
from tests.test_gpu_adjoint import _seeds, _setup


def test_function_objectives_equal_built_ins():
    for name, fn in (('box8', O.kinetic_energy), ('cyl32x16', O.drag('cylinder'))):
        case, mesh, x, S, dt = _setup(name)
        St = None if S is None else [torch.as_tensor(s) for s in S]
        a = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
        b = torch_ref.Problem(mesh, case.bc, case.config, fn)
        ra, rb = a.step(x[0], x[1], x[2], dt, St), b.step(x[0], x[1], x[2], dt, St)
        assert abs(float(ra[4]) - float(rb[4])) <= 1e-13 * abs(float(ra[4])), name
        seeds = _seeds(x, 7)
        ga = torch_ref.vjp_step(a, x[0], x[1], x[2], dt, St, seeds, 1.0)
        gb = torch_ref.vjp_step(b, x[0], x[1], x[2], dt, St, seeds, 1.0)
        for i in range(3):
            assert G.rel_err(gb[i].numpy(), ga[i].numpy()) < 1e-13, (name, i)
