"""Parity on the benchmarked workloads themselves, not only on the small golden meshes.

* the throughput workload - the periodic 128^3 box, node coordinates jittered, cells shuffled
  and then renumbered (2,097,152 cells, 6,340,608 faces), Roe, Sutherland viscosity - three
  FP64 steps through the C ABI against the C oracle (oracle/c), state, CFL sum and objective
  within 1e-12 after every step;
* one FP64 adjoint step of the same recipe on a 32^3 box against torch autograd of the oracle
  (the exact VJP of the same discrete step) within 1e-12;
* the adjoint workload's mesh (64^3 box, kinetic-energy objective) through the
  torch.autograd.Function with checkpoints and tapes, against autograd of a chain of oracle
  steps, within 1e-12.

Relative error = max|x - ref| / max|ref| per field (the measure of the reference's own tests,
tests/test_op.py:15-18); every assertion message carries the measured error.
"""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from adfvm_gb300.solver import RCF
from oracle import torch_ref
from tests import golden_cases as G

pytestmark = pytest.mark.gpu

NAMES = ('rho', 'rhoU', 'rhoE')


def test_box128_fp64_three_steps_match_c_oracle():
    from oracle.c_ref import COracle
    case = cases.box(128, objective='kinetic_energy')
    mesh = case.build_mesh()
    assert mesh.nInternalCells == 128 ** 3 and mesh.nFaces == 3 * 128 ** 3 + 3 * 128 ** 2
    co = COracle(mesh, case.bc, case.config, case.objective)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    x = [np.asarray(a) for a in cases.conservative(case)]
    d = [torch.as_tensor(a).cuda() for a in x]
    for step in range(3):
        ref = co.step(x[0], x[1], x[2], case.dt)
        out = rcf.step(d[0], d[1], d[2], case.dt)
        for i in range(3):
            e = G.rel_err(out[i].cpu().numpy(), ref[i])
            assert e < 1e-12, ('box128 step %d %s: rel err %.3e' % (step + 1, NAMES[i], e))
        e_dtc = abs(out[3] - ref[3]) / abs(ref[3])
        e_obj = abs(out[4] - ref[4]) / abs(ref[4])
        assert e_dtc < 1e-12, ('box128 step %d dtc: rel err %.3e' % (step + 1, e_dtc))
        assert e_obj < 1e-12, ('box128 step %d objective: rel err %.3e' % (step + 1, e_obj))
        x = list(ref[:3])
        d = list(out[:3])
    rcf.close()


def test_box32_fp64_adjoint_step_matches_autograd():
    case = cases.box(32, objective='kinetic_energy')
    mesh = case.build_mesh()
    x = [torch.as_tensor(a) for a in cases.conservative(case)]
    rng = np.random.default_rng(17)
    seeds = [torch.as_tensor(rng.normal(size=tuple(t.shape))) / float(t.abs().max()) for t in x]
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], case.dt, None, seeds, obja=1.0)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    sd = [t.cuda() for t in seeds]
    # the recomputing adjoint step and the one reading the primal step's stages and tape
    st, tp = rcf.stage_buffer(), rcf.tape_buffer()
    rcf.step(d[0], d[1], d[2], case.dt, stages=st, tape=tp)
    for label, kw in (('recomputed', {}), ('taped', {'stages': st, 'tape': tp})):
        a = rcf.adjoint_step(d[0], d[1], d[2], case.dt, sd, obja=1.0, **kw)
        for i in range(3):
            e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
            assert e < 1e-12, ('box32 adjoint (%s) %sa: rel err %.3e' % (label, NAMES[i], e))
        sg = torch.cat([t.reshape(len(t), -1) for t in a[3]], dim=1).cpu().numpy()
        e = G.rel_err(sg, ref[3].numpy())
        assert e < 1e-12, ('box32 adjoint (%s) source gradient: rel err %.3e' % (label, e))
    rcf.close()


def test_box64_autograd_solve_matches_oracle_chain():
    """The adjoint workload's 64^3 box and kinetic-energy objective: J = sum_n w_n obj_n + a
    terminal term over a two-step chain with a checkpoint every step (so the backward
    recomputes from checkpoints and reads kept stages and tapes), gradient with respect to the
    initial state and the sources."""
    from adfvm_gb300.autograd import solve
    case = cases.box(64, objective='kinetic_energy')
    mesh = case.build_mesh()
    x = [torch.as_tensor(a) for a in cases.conservative(case)]
    nSteps = 2
    w = torch.tensor([0.75, 1.25], dtype=torch.float64)
    rng = np.random.default_rng(23)
    term = [torch.as_tensor(rng.normal(size=tuple(t.shape))) / float(t.abs().max()) for t in x]
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    xs = [t.clone().requires_grad_(True) for t in x]
    St = [torch.zeros_like(t).requires_grad_(True) for t in x]
    y = xs
    objs = []
    for n in range(nSteps):
        o = prob.step(y[0], y[1], y[2], case.dt, torch.cat(St, dim=1))
        objs.append(o[4])
        y = o[:3]
    Jref = (torch.stack(objs) * w).sum() + sum((yi * ti).sum() for yi, ti in zip(y, term))
    gref = torch.autograd.grad(Jref, xs + St)
    del y, objs
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    xd = [t.cuda().requires_grad_(True) for t in x]
    Sd = [torch.zeros_like(t).cuda().requires_grad_(True) for t in x]
    r = solve(rcf, xd[0], xd[1], xd[2], Sd, nSteps=nSteps, dt=case.dt, checkpoint_every=1)
    J = (r[3] * w.cuda()).sum() + sum((yi * ti.cuda()).sum() for yi, ti in zip(r[:3], term))
    eJ = abs(float(J) - float(Jref)) / abs(float(Jref))
    assert eJ < 1e-12, ('box64 objective: rel err %.3e' % eJ)
    g = torch.autograd.grad(J, xd + Sd)
    labels = ['rhoa', 'rhoUa', 'rhoEa', 'S_rhoa', 'S_rhoUa', 'S_rhoEa']
    for i in range(6):
        e = G.rel_err(g[i].cpu().numpy(), gref[i].numpy())
        assert e < 1e-12, ('box64 autograd %s: rel err %.3e' % (labels[i], e))
    rcf.close()
