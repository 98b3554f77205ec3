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
    return [torch.as_tensor(rng.normal(size=tuple(t.shape)) / max(np.abs(t.numpy()).max(), 1.0)) for t in x]


# (the vane channel's golden state is uniform, which puts every wall-parallel face exactly at
# |U.n| = 0, the kink of the Roe entropy fix: there the VJP is decided by roundoff of the
# face velocity, in the reference as here, and no two evaluation orders agree; the vane channel
# is compared at a perturbed state in test_vane_objective_adjoint_with_heat_term)
@pytest.mark.parametrize('name', ['box8', 'cyl32x16', 'sod200_sym_lf', 'box6_inviscid_sumT', 'sod1000',
                                  'duct100_totalpt', 'duct60_totalpt_normals'])
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
    # FP64 adjoint within 1e-12 of the autograd VJP (max|x-ref|/max|ref| per field)
    for i in range(3):
        e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
        assert e < 1e-12, '%s field %d: rel err %.3e' % (name, i, e)
    sg = torch.cat([t.reshape(len(t), -1) for t in a[3]], dim=1).cpu().numpy()
    e = G.rel_err(sg, ref[3].numpy())
    assert e < 1e-12, '%s source gradient: rel err %.3e' % (name, e)


@pytest.mark.parametrize('precision,tol', [('fp32', 1e-4), ('mixed', 1e-6)])
@pytest.mark.parametrize('name', ['box8', 'cyl32x16', 'duct100_totalpt'])
def test_reduced_precision_adjoint_against_fp64_autograd(name, precision, tol):
    """FP32 contexts and mixed ones (FP32 records and face arithmetic, FP64 state, stages and
    adjoints) against the FP64 autograd VJP of one step: max|x-ref|/max|ref| per field."""
    case, mesh, x, S, dt = _setup(name)
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, 7)
    St = None if S is None else [torch.as_tensor(s) for s in S]
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], dt, St, seeds, obja=1.0)
    rcf = RCF(mesh, case.bc, objective=case.objective, precision=precision, **case.config)
    td = torch.float32 if precision == 'fp32' else torch.float64
    d = [t.to(td).cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).to(td).cuda() for s in S]
    a = rcf.adjoint_step(d[0], d[1], d[2], dt, [t.to(td).cuda() for t in seeds], obja=1.0, S=Sd)
    for i in range(3):
        assert a[i].dtype == td
        e = G.rel_err(a[i].double().cpu().numpy(), ref[i].numpy())
        assert e < tol, '%s %s field %d: rel err %.3e' % (name, precision, i, e)


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


def test_sensitivity_dot_product():
    case, mesh, x, S, dt = _setup('box8')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    rng = np.random.default_rng(1)
    arrays = [rng.normal(size=n) for n in (1000, 3 * 512, 7, 300000)]
    perts = [rng.normal(size=a.size) for a in arrays]
    ref = sum(float(np.dot(a, p)) for a, p in zip(arrays, perts))
    g = [torch.as_tensor(a).cuda() for a in arrays]
    p = [torch.as_tensor(b).cuda() for b in perts]
    v1 = rcf.sensitivity(g, p)
    v2 = rcf.sensitivity(g, p)
    assert v1 == v2                                   # fixed reduction order
    assert abs(v1 - ref) <= 1e-12 * sum(float(np.abs(a * b).sum()) for a, b in zip(arrays, perts))


def test_autograd_solve_matches_oracle_and_fd():
    """torch.autograd.Function over 6 steps with checkpoints every 4: gradient of a weighted
    objective time series plus a terminal term, against autograd of the oracle (6 chained
    oracle steps) and central differences."""
    from adfvm_gb300.autograd import solve
    case, mesh, x, S, dt = _setup('cyl32x16')
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    nSteps = 6
    w = torch.linspace(0.5, 1.5, nSteps, dtype=torch.float64)
    term = [t for t in _seeds(x, 21)]
    xs = [t.clone().requires_grad_(True) for t in x]
    St = [torch.zeros_like(t).requires_grad_(True) for t in x]
    # oracle chain
    y = xs
    objs = []
    for n in range(nSteps):
        o = prob.step(y[0], y[1], y[2], dt, torch.cat(St, dim=1))
        objs.append(o[4])
        y = o[:3]
    Jref = (torch.stack(objs) * w).sum() + sum((yi * ti).sum() for yi, ti in zip(y, term))
    gref = torch.autograd.grad(Jref, xs + St)
    # GPU
    xd = [t.cuda().requires_grad_(True) for t in x]
    Sd = [torch.zeros_like(t).cuda().requires_grad_(True) for t in x]
    r = solve(rcf, xd[0], xd[1], xd[2], Sd, nSteps=nSteps, dt=dt, checkpoint_every=4)
    J = (r[3] * w.cuda()).sum() + sum((yi * ti.cuda()).sum() for yi, ti in zip(r[:3], term))
    assert abs(float(J) - float(Jref)) <= 1e-12 * abs(float(Jref))
    g = torch.autograd.grad(J, xd + Sd)
    for i in range(6):
        e = G.rel_err(g[i].cpu().numpy(), gref[i].numpy())
        assert e < 1e-12, 'autograd chain input %d: rel err %.3e' % (i, e)


@pytest.mark.parametrize('name,precision', [('box8', 'fp64'), ('cyl32x16', 'fp64'), ('duct100_totalpt', 'fp64'),
                                            ('box8', 'fp32'), ('cyl32x16', 'mixed')])
def test_kept_stages_give_the_same_adjoint(name, precision):
    """afvm_primal_step_stages / afvm_adjoint_step_stages: the adjoint on the stage states the
    primal step kept is bitwise the adjoint that recomputes them, and the primal step itself is
    unchanged by keeping them."""
    case, mesh, x, S, dt = _setup(name)
    rcf = RCF(mesh, case.bc, objective=case.objective, precision=precision, **case.config)
    td = torch.float32 if precision == 'fp32' else torch.float64
    d = [t.to(td).cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).to(td).cuda() for s in S]
    seeds = [t.to(td).cuda() for t in _seeds(x, 3)]
    st = rcf.stage_buffer()
    p0 = rcf.step(d[0], d[1], d[2], dt, S=Sd)
    p1 = rcf.step(d[0], d[1], d[2], dt, S=Sd, stages=st)
    for u, v in zip(p0[:3], p1[:3]):
        assert torch.equal(u, v)
    assert p0[3:] == p1[3:]
    a0 = rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, obja=1.0, S=Sd)
    a1 = rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, obja=1.0, S=Sd, stages=st)
    for u, v in zip(a0[:3], a1[:3]):
        assert torch.equal(u, v)
    for u, v in zip(a0[3], a1[3]):
        assert torch.equal(u, v)
    with pytest.raises(ValueError):
        rcf.adjoint_step(d[0], d[1], d[2], dt, seeds, S=Sd, stages=st[:10])


@pytest.mark.parametrize('nx,ny,b,ref', [(24, 10, 0.0, False), (24, 10, 1e-5, False), (32, 12, 0.0, True)])
def test_vane_objective_adjoint_with_heat_term(nx, ny, b, ref):
    """The turbine-vane objective, with its heat-transfer term switched on (the reference's own
    file has b = 0) and with the reference's own constants on the golden mesh: value and VJP
    against the oracle and its autograd, FP64, at a perturbed state."""
    case = cases.vane_channel(nx, ny, reference_constants=True) if ref else cases.vane_channel(nx, ny, b=b)
    mesh = case.build_mesh()
    x = [torch.as_tensor(a) for a in cases.conservative(case)]
    rng = np.random.default_rng(5)
    x = [t * (1 + 0.01 * torch.as_tensor(rng.standard_normal(tuple(t.shape)))) for t in x]
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    ref_step = prob.step(x[0], x[1], x[2], case.dt)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    d = [t.cuda() for t in x]
    r = rcf.step(d[0], d[1], d[2], case.dt)
    assert abs(r[4] - float(ref_step[4])) <= 1e-12 * abs(float(ref_step[4]))
    seeds = _seeds(x, 9)
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], case.dt, None, seeds, obja=1.0)
    a = rcf.adjoint_step(d[0], d[1], d[2], case.dt, [t.cuda() for t in seeds], obja=1.0)
    for i in range(3):
        e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
        assert e < 1e-12, 'vane field %d: rel err %.3e' % (i, e)
    # the objective's own gradient (no state seeds) is the part that changes with b
    z = [torch.zeros_like(t) for t in seeds]
    ref0 = torch_ref.vjp_step(prob, x[0], x[1], x[2], case.dt, None, z, obja=1.0)
    a0 = rcf.adjoint_step(d[0], d[1], d[2], case.dt, [t.cuda() for t in z], obja=1.0)
    for i in range(3):
        e = G.rel_err(a0[i].cpu().numpy(), ref0[i].numpy())
        assert e < 1e-12, 'vane objective gradient field %d: rel err %.3e' % (i, e)


@pytest.mark.parametrize('name', ['sod1', 'box1', 'box2', 'vane2x1', 'cyl4x2'])
def test_tiny_meshes_adjoint_matches_autograd(name):
    """The adjoint step on the smallest meshes (one cell cyclic to itself, ...) within 1e-12 of
    the oracle's autograd VJP."""
    from tests.test_oracle_c import TINY
    case = TINY[name]()
    mesh = case.build_mesh()
    x = [torch.as_tensor(np.asarray(a)) for a in cases.conservative(case)]
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    seeds = _seeds(x, 11)
    ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], case.dt, None, seeds, obja=1.0)
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    a = rcf.adjoint_step(*[t.cuda() for t in x], case.dt, [t.cuda() for t in seeds], obja=1.0)
    for i in range(3):
        e = G.rel_err(a[i].cpu().numpy(), ref[i].numpy())
        if name == 'box1' and i == 2:
            # one cell cyclic to itself: its rhoE adjoint is the seed (~1e-6) plus the kinetic
            # energy's derivative, which is exactly zero (0.5 |rhoU|^2 V / rho does not depend on
            # rhoE) but is evaluated, through p and T, as two terms of size |U|^2 V / (2 Cv T)
            # that cancel: their rounding is measured against that size (measured 7e-16)
            rho, rhoE = float(x[0].reshape(-1)[0]), float(x[2].reshape(-1)[0])
            U = (x[1] / x[0]).numpy().ravel()
            Cv = 1004.5 / 1.4
            T = (rhoE / rho - 0.5 * float(np.dot(U, U))) / Cv
            term = 0.5 * float(np.dot(U, U)) * float(np.asarray(mesh.volumes).ravel()[0]) / (Cv * T)
            err = float(np.abs(a[i].cpu().numpy() - ref[i].numpy()).max())
            assert err <= 1e-14 * term, 'box1 rhoE: error %.3e against terms of %.3e' % (err, term)
            continue
        assert e < 1e-12, '%s field %d: rel err %.3e' % (name, i, e)


@pytest.mark.parametrize('name,precision', [('box8', 'fp64'), ('cyl32x16', 'fp64'), ('sod200_sym_lf', 'fp64'),
                                            ('duct100_totalpt', 'fp64'), ('box6_inviscid_sumT', 'fp64'),
                                            ('box8', 'fp32'), ('cyl32x16', 'mixed')])
def test_taped_adjoint_matches(name, precision):
    """afvm_primal_step_tape / afvm_adjoint_step_tape: the adjoint that reads the forward's face
    tape agrees with the one that re-evaluates the forward (to the rounding of FMA contraction
    in the two kernels) and, in FP64, with the autograd VJP within 1e-12; the primal step is the
    same with and without the tape."""
    case, mesh, x, S, dt = _setup(name)
    rcf = RCF(mesh, case.bc, objective=case.objective, precision=precision, **case.config)
    td = torch.float32 if precision == 'fp32' else torch.float64
    d = [t.to(td).cuda() for t in x]
    Sd = None if S is None else [torch.as_tensor(s).to(td).cuda() for s in S]
    seeds = _seeds(x, 5)
    sd = [t.to(td).cuda() for t in seeds]
    st1, st2, tp = rcf.stage_buffer(), rcf.stage_buffer(), rcf.tape_buffer()
    p1 = rcf.step(d[0], d[1], d[2], dt, S=Sd, stages=st1)
    p2 = rcf.step(d[0], d[1], d[2], dt, S=Sd, stages=st2, tape=tp)
    for u, v in zip(p1[:3], p2[:3]):
        assert G.rel_err(v.double().cpu().numpy(), u.double().cpu().numpy()) <= 1e-15
    a1 = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, stages=st1)
    a2 = rcf.adjoint_step(d[0], d[1], d[2], dt, sd, obja=1.0, S=Sd, stages=st2, tape=tp)
    tol = 1e-5 if precision == 'fp32' else (1e-6 if precision == 'mixed' else 1e-13)
    for i in range(3):
        e = G.rel_err(a2[i].double().cpu().numpy(), a1[i].double().cpu().numpy())
        assert e <= tol, (name, precision, i, e)
    if precision == 'fp64':
        prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
        St = None if S is None else [torch.as_tensor(s) for s in S]
        ref = torch_ref.vjp_step(prob, x[0], x[1], x[2], dt, St, seeds, obja=1.0)
        for i in range(3):
            e = G.rel_err(a2[i].cpu().numpy(), ref[i].numpy())
            assert e < 1e-12, '%s taped field %d: rel err %.3e' % (name, i, e)
    with pytest.raises(ValueError):
        rcf.step(d[0], d[1], d[2], dt, S=Sd, tape=tp)
