"""Gradients of the adjoint step with respect to the mesh tensors and the boundary inputs
(afvm_adjoint_step_params; the reference's Adjoint(parameters='mesh') and
Adjoint(parameters=('BCs', field, patch, key)), apps/adjoint.py:101-126) against torch autograd
of the oracle with those tensors as leaves, and against central finite differences of the
GPU step itself.

Tolerance: 1e-12 relative (max|x-ref|/max|ref| per tensor) for the autograd comparisons;
finite differences (step 1e-6 relative to each tensor's scale) within 1e-6 of the sum of
|gradient| |direction|. The state and source adjoints of the call are bitwise those of the
plain adjoint step.
"""
import copy

import numpy as np
import pytest
import torch

from adfvm_gb300.solver import RCF
from oracle import torch_ref
from tests import golden_cases as G
from tests.test_gpu_adjoint import _seeds, _setup

pytestmark = pytest.mark.gpu

MESH_CASES = ['box8', 'cyl32x16', 'sod200_sym_lf', 'box6_inviscid_sumT', 'duct100_totalpt', 'duct60_totalpt_normals',
              'sod1000']


def _run(name, params, taped=False):
    case, mesh, x, S, dt = _setup(name)
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, 7)
    St = None if S is None else [torch.as_tensor(s) for s in S]
    ref = torch_ref.vjp_step_params(prob, x[0], x[1], x[2], dt, St, seeds, 1.0, params)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).cuda() for s in S]
    sd = [t.cuda() for t in seeds]
    kw = {}
    if taped:
        kw = {'stages': rcf.stage_buffer(), 'tape': rcf.tape_buffer()}
        rcf.step(d[0], d[1], d[2], dt, S=Sd, **kw)
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, params=params, **kw)
    plain = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, **kw)
    for i in range(3):
        assert torch.equal(a[i], plain[i]), 'state adjoint %d changed by the parameter gradients' % i
    for u, v in zip(a[3], plain[3]):
        assert torch.equal(u, v)
    return a, ref, rcf


@pytest.mark.parametrize('taped', [False, True])
@pytest.mark.parametrize('name', MESH_CASES)
def test_mesh_gradient_matches_autograd(name, taped):
    a, ref, rcf = _run(name, 'mesh', taped)
    assert [tuple(t.shape) for t in a[4]] == [tuple(t.shape) for t in ref[4]]
    for k, field in enumerate(RCF.MESH_GRAD_FIELDS):
        e = G.rel_err(a[4][k].cpu().numpy(), ref[4][k].numpy())
        assert e < 1e-12, '%s d/d%s: rel err %.3e' % (name, field, e)
    rcf.close()


BC_PARAMS = [('cyl32x16', ('BCs', 'p', 'farfield', 'p0')),        # templates/cylinder.py:92
             ('cyl32x16', ('BCs', 'p', 'farfield', 'U0')),
             ('cyl32x16', ('BCs', 'p', 'farfield', 'T0')),
             ('cyl32x16', ('BCs', 'U', 'farfield', 'U0')),        # a copy the step never reads: zero
             ('cyl32x16', ('BCs', 'U', 'cylinder', 'value')),
             ('duct100_totalpt', ('BCs', 'p', 'left', 'pt')),
             ('duct100_totalpt', ('BCs', 'p', 'left', 'Tt')),
             ('duct100_totalpt', ('BCs', 'p', 'left', 'direction')),
             ('duct100_totalpt', ('BCs', 'p', 'right', 'p0')),
             ('duct60_totalpt_normals', ('BCs', 'p', 'left', 'pt'))]


@pytest.mark.parametrize('name,params', BC_PARAMS)
def test_boundary_input_gradient_matches_autograd(name, params):
    a, ref, rcf = _run(name, params)
    g, r = a[4][0].cpu().numpy(), ref[4][0].numpy()
    assert g.shape == r.shape
    if params[1] == 'U' and params[3] == 'U0':
        assert not g.any() and not r.any()
    else:
        assert np.abs(r).max() > 0
    e = G.rel_err(g, r)
    assert e < 1e-12, '%s %s: rel err %.3e' % (name, params, e)
    rcf.close()


def test_parameter_errors():
    case, mesh, x, S, dt = _setup('cyl32x16')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    sd = [t.cuda() for t in _seeds(x, 7)]
    for bad in [('BCs', 'p', 'cylinder', 'value'), ('BCs', 'p', 'front', 'value'), ('BCs', 'p', 'nowhere', 'p0'),
                ('BCs', 'U', 'cylinder', 'U0'), 'source', ('mesh',)]:
        with pytest.raises(ValueError):
            rcf.adjoint_step(d[0], d[1], d[2], dt, sd, params=bad)
    c32 = RCF(mesh, case.bc, objective=case.objective, precision='fp32', **case.config)
    from adfvm_gb300 import _lib as L
    with pytest.raises(L.AfvmError) as ei:
        c32.adjoint_step(*[t.float() for t in d], dt, [t.float() for t in sd], params='mesh')
    assert ei.value.status == L.AFVM_ERR_UNSUPPORTED


def _J(rcf, d, sd, dt, S, obja):
    o = rcf.step(d[0], d[1], d[2], dt, S=S)
    return sum(float((oi * si).sum()) for oi, si in zip(o[:3], sd)) + obja * o[4]


@pytest.mark.parametrize('name', ['box8', 'cyl32x16'])
def test_mesh_gradient_matches_central_differences(name):
    """<grad, v> against (J(mesh + h v) - J(mesh - h v)) / 2h, J = <seeds, step outputs> +
    obja obj, over a seeded direction v in all ten tensors at once (each scaled to its own
    magnitude), each side a context built on the perturbed tensors."""
    case, mesh, x, S, dt = _setup(name)
    d = [t.cuda() for t in x]
    sd = [t.cuda() for t in _seeds(x, 7)]
    Sd = None if S is None else [torch.as_tensor(s).cuda() for s in S]
    obja = 1e-3
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    grads = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=obja, S=Sd, params='mesh')[4]
    rng = np.random.default_rng(31)
    v = {}
    for k in RCF.MESH_GRAD_FIELDS:
        a = np.asarray(getattr(mesh, k))
        v[k] = rng.standard_normal(a.shape) * (np.abs(a).max() if a.size else 1.0)
    h = 1e-6

    def J(sign):
        m2 = copy.copy(mesh)
        for k in RCF.MESH_GRAD_FIELDS:
            setattr(m2, k, np.asarray(getattr(mesh, k)) + sign * h * v[k])
        r = RCF(m2, case.bc, objective=case.objective, **case.config)
        out = _J(r, d, sd, dt, Sd, obja)
        r.close()
        return out
    fd = (J(1) - J(-1)) / (2 * h)
    ad = sum(float((g.cpu().numpy() * v[k].reshape(g.shape)).sum()) for g, k in zip(grads, RCF.MESH_GRAD_FIELDS))
    scale = sum(float(np.abs(g.cpu().numpy() * v[k].reshape(g.shape)).sum()) for g, k in zip(grads, RCF.MESH_GRAD_FIELDS))
    assert abs(fd - ad) <= 1e-6 * scale, (fd, ad, scale)


def test_boundary_input_gradient_matches_central_differences():
    """The far-field p0 of the cylinder (the parameter of templates/cylinder.py:92)."""
    case, mesh, x, S, dt = _setup('cyl32x16')
    d = [t.cuda() for t in x]
    sd = [t.cuda() for t in _seeds(x, 7)]
    obja = 1e-3
    params = ('BCs', 'p', 'farfield', 'p0')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    g = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=obja, params=params)[4][0].cpu().numpy()
    p0 = np.asarray(case.bc['p']['farfield']['p0'], np.float64).reshape(-1, 1)
    v = np.random.default_rng(33).standard_normal(p0.shape) * np.abs(p0).max()
    h = 1e-6

    def J(sign):
        bc = {f: {p: dict(e) for p, e in case.bc[f].items()} for f in ('U', 'T', 'p')}
        bc['p']['farfield']['p0'] = p0 + sign * h * v
        r = RCF(mesh, bc, objective=case.objective, **case.config)
        out = _J(r, d, sd, dt, None, obja)
        r.close()
        return out
    fd = (J(1) - J(-1)) / (2 * h)
    ad = float((g * v).sum())
    assert abs(fd - ad) <= 1e-6 * float(np.abs(g * v).sum()), (fd, ad)


def test_adjoint_map_returns_mesh_gradients_in_reference_order():
    """Adjoint(parameters='mesh').map: the reference's input list in, [rhoa, rhoUa, rhoEa] and
    the ten Mesh.gradFields gradients out (apps/adjoint.py:108-110, 124-126), host arrays."""
    from adfvm_gb300.adjoint import Adjoint
    from adfvm_gb300.mesh import Mesh
    case, mesh, x, S, dt = _setup('box8')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    seeds = [t.numpy() for t in _seeds(x, 7)]
    host = [t.numpy() for t in x]
    src = [np.asarray(s) for s in S] if S is not None else None
    inputs = rcf.mapInputs(*host, dt, src) + seeds + [np.zeros((1, 1)), np.ones((1, 1)), np.zeros((1, 1))]
    out = Adjoint(rcf, parameters='mesh').map(*inputs)
    assert len(out) == 3 + len(Mesh.gradFields)
    for o, k in zip(out[3:], Mesh.gradFields):
        assert o.shape == np.shape(getattr(mesh, k)), k
    d = [t.cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).cuda() for s in S]
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, [torch.as_tensor(s).cuda() for s in seeds], obja=1.0, S=Sd,
                         params='mesh')
    for o, t in zip(out, list(a[:3]) + list(a[4])):
        e = G.rel_err(o, t.cpu().numpy().reshape(o.shape))
        assert e < 1e-13, e


def test_adjoint_sweep_boundary_sensitivity_matches_finite_differences():
    """Adjoint(parameters=('BCs', 'U', 'cylinder', 'value')).run over 4 fixed steps with
    checkpoints every 2: the time-averaged drag's sensitivity to a perturbation of the wall
    velocity against central differences of the primal runs. (The far-field inputs of the
    templates reach the wall only after many more steps than these 4.)"""
    from adfvm_gb300.adjoint import Adjoint
    case, mesh, x, S, dt = _setup('cyl32x16')
    cfg = dict(case.config, fixedTimeStep=True)
    rcf = RCF(mesh, case.bc, objective=case.objective, **cfg)
    uw = np.asarray(case.bc['U']['cylinder']['value'], np.float64).reshape(-1, 3)
    v = np.random.default_rng(35).standard_normal(uw.shape)
    host = [t.numpy() for t in x]
    nSteps = 4
    sens, _, _ = Adjoint(rcf, parameters=('BCs', 'U', 'cylinder', 'value')).run(host, nSteps, dt, 2,
                                                                                 perturbations=[(v,)])
    assert abs(sens[0]) > 0
    h = 1e-4

    def J(sign):
        bc = {f: {p: dict(e) for p, e in case.bc[f].items()} for f in ('U', 'T', 'p')}
        bc['U']['cylinder']['value'] = uw + sign * h * v
        r = RCF(mesh, bc, objective=case.objective, **cfg)
        res, _ = r.run([a.copy() for a in host], nSteps, dt)
        r.close()
        return res / nSteps
    fd = (J(1) - J(-1)) / (2 * h)
    assert abs(fd - sens[0]) <= 1e-6 * abs(sens[0]), (fd, sens[0])
