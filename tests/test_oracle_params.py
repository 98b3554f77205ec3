"""The oracle's parameter gradients (torch_ref.vjp_step_params: autograd with the mesh tensors
or one boundary input as leaves, the oracle of the GPU's afvm_adjoint_step_params) against
central finite differences of the oracle's own step, so that every use of a parameter in the
restated residual is seen by the leaves."""
import numpy as np
import pytest
import torch

from oracle import torch_ref
from tests.test_gpu_adjoint import _seeds, _setup

torch.set_num_threads(min(8, torch.get_num_threads()))


def _J(P, x, dt, S, seeds, obja):
    with torch.no_grad():
        o = P.step(x[0], x[1], x[2], dt, S)
        return float(sum((oi * si).sum() for oi, si in zip(o[:3], seeds)) + obja * o[4])


@pytest.mark.parametrize('name,params', [('box8', 'mesh'), ('cyl32x16', 'mesh'), ('sod200_sym_lf', 'mesh'),
                                         ('duct60_totalpt_normals', 'mesh'),
                                         ('cyl32x16', ('BCs', 'p', 'farfield', 'p0')),
                                         ('cyl32x16', ('BCs', 'U', 'cylinder', 'value')),
                                         ('duct100_totalpt', ('BCs', 'p', 'left', 'Tt')),
                                         ('duct100_totalpt', ('BCs', 'p', 'left', 'direction'))])
def test_oracle_parameter_gradient_matches_central_differences(name, params):
    case, mesh, x, S, dt = _setup(name)
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, 7)
    St = None if S is None else torch.cat([torch.as_tensor(s).reshape(len(x[0]), -1) for s in S], dim=1)
    obja = 1e-3
    r = torch_ref.vjp_step_params(prob, x[0], x[1], x[2], dt, St, seeds, obja, params)
    grads = [g.numpy() for g in r[4]]
    base = [t.detach().numpy() for t in torch_ref.with_parameter_leaves(prob, params)[1]]
    rng = np.random.default_rng(41)
    v = [rng.standard_normal(b.shape) * (np.abs(b).max() if b.size and np.abs(b).max() > 0 else 1.0) for b in base]
    h = 1e-6

    def J(sign):
        P, _ = torch_ref.with_parameter_leaves(prob, params, [b + sign * h * vi for b, vi in zip(base, v)])
        return _J(P, x, dt, St, seeds, obja)
    fd = (J(1) - J(-1)) / (2 * h)
    ad = sum(float((g * vi).sum()) for g, vi in zip(grads, v))
    scale = sum(float(np.abs(g * vi).sum()) for g, vi in zip(grads, v))
    assert scale > 0
    assert abs(fd - ad) <= 1e-6 * scale, (fd, ad, scale)
