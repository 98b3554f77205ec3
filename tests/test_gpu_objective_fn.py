"""Objectives given as torch functions objective([U, T, p], solver), the form of a reference
case file's objective (adFVM/density.py:354-357), through the GPU solver: evaluated in FP64
on the objective-stage primitives the step copies out (afvm_set_objective_sink), their adjoint
seed by torch autograd (afvm_set_objective_seed).

* restating the built-in kinetic energy and drag: the same objective values and the same
  state, source and mesh adjoints as the built-in kernels, within 1e-12;
* a made-up objective that reads ghost cells, volumes and areas: state adjoint, mesh gradient
  and boundary-input gradient against autograd of the oracle running the same function,
  within 1e-12; through Adjoint.map and with kept stages and tapes.
"""
import numpy as np
import pytest
import torch

from adfvm_gb300.solver import RCF
from oracle import torch_ref
from tests import golden_cases as G
from tests import objective_fns as O
from tests.test_gpu_adjoint import _seeds, _setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name,fn', [('box8', O.kinetic_energy), ('cyl32x16', O.drag('cylinder'))])
def test_function_objective_equals_built_in(name, fn):
    case, mesh, x, S, dt = _setup(name)
    d = [t.cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).cuda() for s in S]
    sd = [t.cuda() for t in _seeds(x, 7)]
    a = RCF(mesh, case.bc, objective=case.objective, **case.config)
    b = RCF(mesh, case.bc, objective=fn, **case.config)
    ra, rb = a.step(d[0], d[1], d[2], dt, S=Sd), b.step(d[0], d[1], d[2], dt, S=Sd)
    for i in range(3):
        assert torch.equal(ra[i], rb[i])
    e = abs(rb[4] - ra[4]) / abs(ra[4])
    assert e < 1e-12, '%s objective: rel err %.3e' % (name, e)
    ga = a.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, params='mesh')
    gb = b.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, params='mesh')
    for i in range(3):
        e = G.rel_err(gb[i].cpu().numpy(), ga[i].cpu().numpy())
        assert e < 1e-12, '%s adjoint %d: rel err %.3e' % (name, i, e)
    for k, f in enumerate(RCF.MESH_GRAD_FIELDS):
        e = G.rel_err(gb[4][k].cpu().numpy(), ga[4][k].cpu().numpy())
        assert e < 1e-12, '%s d/d%s: rel err %.3e' % (name, f, e)


@pytest.mark.parametrize('params', [None, 'mesh', ('BCs', 'p', 'farfield', 'p0')])
@pytest.mark.parametrize('taped', [False, True])
def test_function_objective_against_oracle(params, taped):
    case, mesh, x, S, dt = _setup('cyl32x16')
    fn = O.pressure_mix('farfield')
    prob = torch_ref.Problem(mesh, case.bc, case.config, fn)
    seeds = _seeds(x, 7)
    if params is None:
        ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], dt, None, seeds, 1.0)
        ref_obj = float(prob.step(x[0], x[1], x[2], dt)[4])
    else:
        ref = torch_ref.vjp_step_params(prob, x[0], x[1], x[2], dt, None, seeds, 1.0, params)
    rcf = RCF(mesh, case.bc, objective=fn, **case.config)
    d = [t.cuda() for t in x]
    sd = [t.cuda() for t in seeds]
    kw = {}
    if taped:
        kw = {'stages': rcf.stage_buffer(), 'tape': rcf.tape_buffer()}
    r = rcf.step(d[0], d[1], d[2], dt, **kw)
    if params is None:
        e = abs(r[4] - ref_obj) / abs(ref_obj)
        assert e < 1e-12, 'objective: rel err %.3e' % e
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, params=params, **kw)
    for i in range(3):
        e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
        assert e < 1e-12, 'adjoint %d: rel err %.3e' % (i, e)
    if params is not None:
        for k, (g, gr) in enumerate(zip(a[4], ref[4])):
            e = G.rel_err(g.cpu().numpy(), gr.numpy())
            assert e < 1e-12, 'parameter gradient %d: rel err %.3e' % (k, e)


def test_function_objective_through_the_reference_maps():
    """RCF.map returns the function's value as its obj output, and Adjoint.map's adjoint seeds
    it: the same as the device calls."""
    from adfvm_gb300.adjoint import Adjoint
    case, mesh, x, S, dt = _setup('cyl32x16')
    fn = O.pressure_mix('farfield')
    rcf = RCF(mesh, case.bc, objective=fn, **case.config)
    host = [t.numpy() for t in x]
    out = rcf.map(*rcf.mapInputs(*host, dt))
    d = [t.cuda() for t in x]
    r = rcf.step(d[0], d[1], d[2], dt)
    assert abs(float(out[4][0, 0]) - r[4]) <= 1e-14 * abs(r[4])
    seeds = [t.numpy() for t in _seeds(x, 7)]
    inputs = rcf.mapInputs(*host, dt) + seeds + [np.zeros((1, 1)), np.ones((1, 1)), np.zeros((1, 1))]
    am = Adjoint(rcf).map(*inputs)
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, [torch.as_tensor(s).cuda() for s in seeds], obja=1.0)
    for i in range(3):
        e = G.rel_err(am[i], a[i].cpu().numpy())
        assert e < 1e-13, 'Adjoint.map field %d: rel err %.3e' % (i, e)
