"""GPU discrete adjoint of one step through the C ABI against torch autograd of the oracle
(the exact VJP of the same discrete arithmetic), and against central finite differences."""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from adfvm_gb300.solver import RCF
from oracle import torch_ref
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _setup(name):
    case, g = G.load(name)
    mesh = case.build_mesh()
    x = [torch.as_tensor(np.asarray(g[k + '_init'])).reshape(mesh.nInternalCells, -1)
         for k in ('rho', 'rhoU', 'rhoE')]
    S = cases.source_field(mesh) if bool(g['with_source']) else None
    return case, mesh, x, S, float(g['dt0'])


def _seeds(x, seed):
    rng = np.random.default_rng(seed)
    return [torch.as_tensor(rng.normal(size=tuple(t.shape)) / np.abs(t.numpy()).max()) for t in x]


@pytest.mark.parametrize('name', ['box8', 'cyl32x16', 'sod200_sym_lf', 'box6_inviscid_sumT', 'sod1000'])
def test_adjoint_step_matches_autograd(name):
    case, mesh, x, S, dt = _setup(name)
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, 7)
    St = None if S is None else [torch.as_tensor(s) for s in S]
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], dt, St, seeds, obja=1.0)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).cuda() for s in S]
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, [t.cuda() for t in seeds], obja=1.0, S=Sd)
    # FP64 adjoint within 1e-11 of the autograd VJP (max|x-ref|/max|ref| per field)
    for i in range(3):
        e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
        assert e < 1e-11, (name, i, e)
    sg = torch.cat([t.reshape(len(t), -1) for t in a[3]], dim=1).cpu().numpy()
    e = G.rel_err(sg, ref[3].numpy())
    assert e < 1e-11, (name, 'source', e)


def test_adjoint_deterministic_and_aliasing():
    case, mesh, x, S, dt = _setup('cyl32x16')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    seeds = [t.cuda() for t in _seeds(x, 3)]
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, obja=0.5)
    b = rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, obja=0.5)
    for i in range(3):
        assert torch.equal(a[i], b[i])
    # outputs may alias the seeds
    s2 = [t.clone() for t in seeds]
    c = rcf.adjoint_step(d[0], d[1], d[2], dt, s2, obja=0.5, out=s2)
    for i in range(3):
        assert torch.equal(c[i], a[i])


def test_adjoint_matches_central_differences():
    """<seed, d step(u + h v)/dh> by central differences vs <adjoint, v> (FD step 1e-6,
    relative to the state scale), on several seeded directions."""
    case, mesh, x, S, dt = _setup('box8')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    seeds = [t.cuda() for t in _seeds(x, 5)]
    obja = 1e-3
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, obja=obja)
    rng = np.random.default_rng(9)
    for k in range(4):
        v = [torch.as_tensor(rng.normal(size=tuple(t.shape))).cuda() * t.abs().max() for t in d]
        h = 1e-6

        def J(sign):
            y = [t + sign * h * vv for t, vv in zip(d, v)]
            o = rcf.step(y[0], y[1], y[2], dt)
            return sum(float((oi * si).sum()) for oi, si in zip(o[:3], seeds)) + obja * o[4]
        fd = (J(1) - J(-1)) / (2 * h)
        ad = sum(float((ai * vi).sum()) for ai, vi in zip(a[:3], v))
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30), (k, fd, ad)
