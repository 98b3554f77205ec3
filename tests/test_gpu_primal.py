"""GPU primal step through the C ABI against the reference's own trajectories and the oracle.

Tolerances: FP64 within 1e-12 relative (max|x-ref|/max|ref| per field, the measure of the
reference's tests, tests/test_op.py:15-18); FP32 against the FP64 oracle within the bound
stated in each test.
"""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from adfvm_gb300.solver import RCF
from oracle import torch_ref
from tests import golden_cases as G
from tests.test_oracle_c import TINY

pytestmark = pytest.mark.gpu


def _solver(case, precision='fp64'):
    return RCF(case.build_mesh(), case.bc, objective=case.objective, precision=precision, **case.config)


def _init(g):
    return [np.asarray(g['rho_init']).reshape(-1, 1), np.asarray(g['rhoU_init']).reshape(-1, 3),
            np.asarray(g['rhoE_init']).reshape(-1, 1)]


@pytest.mark.parametrize('name', G.available())
def test_fp64_trajectory_matches_reference(name):
    case, g = G.load(name)
    rcf = _solver(case)
    src = None
    if bool(g['with_source']):
        from adfvm_gb300 import cases
        src = cases.source_field(case.build_mesh())
    sols, record = rcf.run(_init(g), int(g['nSteps']), float(g['dt0']), mode='forward', source=src)
    record = np.array(record)
    for k in range(3):
        assert G.rel_err(record[:, k], g['record'][:, k]) < 1e-12, (name, k)
    for s in g['steps']:
        for i, nm in enumerate(['rho', 'rhoU', 'rhoE']):
            e = G.rel_err(sols[s][i], g['%s_%d' % (nm, s)])
            assert e < 1e-12, (name, nm, s, e)


@pytest.mark.parametrize('name', ['box8', 'cyl32x16', 'sod200_sym_lf'])
def test_device_step_matches_oracle_one_step(name):
    case, g = G.load(name)
    mesh = case.build_mesh()
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    x = [torch.as_tensor(a) for a in _init(g)]
    ref = prob.step(x[0], x[1], x[2], float(g['dt0']))
    rcf = _solver(case)
    d = [a.cuda() for a in x]
    out = rcf.step(d[0], d[1], d[2], float(g['dt0']))
    for i in range(3):
        assert G.rel_err(out[i].cpu().numpy(), ref[i].numpy()) < 1e-13
    assert abs(out[3] - float(ref[3])) <= 1e-13 * abs(float(ref[3]))
    assert abs(out[4] - float(ref[4])) <= 1e-12 * max(1.0, abs(float(ref[4])))


def test_device_run_matches_step_loop_and_is_deterministic():
    case, g = G.load('sod1000')
    rcf = _solver(case)
    x = [torch.as_tensor(a).cuda() for a in _init(g)]
    a = [t.clone() for t in x]
    hist = rcf.run_device(a[0], a[1], a[2], 20, float(g['dt0']))
    b = [t.clone() for t in x]
    hist2 = rcf.run_device(b[0], b[1], b[2], 20, float(g['dt0']))
    torch.cuda.synchronize()
    for i in range(3):
        assert torch.equal(a[i], b[i])          # bitwise reproducible (no atomics in sums)
    assert torch.equal(hist, hist2)
    # same as the host loop of the reference time-step rule
    sols, record = rcf.run(_init(g), 20, float(g['dt0']), mode='forward')
    for i in range(3):
        assert G.rel_err(a[i].cpu().numpy(), sols[20][i]) < 1e-13
    assert G.rel_err(hist[0].cpu().numpy(), np.array(record)[:, 0]) < 1e-13


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
@pytest.mark.parametrize('name', ['box8', 'cyl32x16'])
def test_fp32_against_fp64_oracle(name, precision):
    case, g = G.load(name)
    mesh = case.build_mesh()
    prob = torch_ref.Problem(mesh, case.bc, case.config, case.objective)
    x = [torch.as_tensor(a) for a in _init(g)]
    ref = prob.step(x[0], x[1], x[2], float(g['dt0']))
    rcf = _solver(case, precision)
    td = torch.float32 if precision == 'fp32' else torch.float64
    d = [a.to(td).cuda() for a in x]
    out = rcf.step(d[0], d[1], d[2], float(g['dt0']))
    assert out[0].dtype == td
    # FP32 records and flux arithmetic: one step stays within 1e-5 of FP64 per field; with
    # the state in FP64 ('mixed') only the step's increment carries FP32 rounding: 1e-6
    tol = 1e-5 if precision == 'fp32' else 1e-6
    for i in range(3):
        e = G.rel_err(out[i].double().cpu().numpy(), ref[i].numpy())
        assert e < tol, (i, e)
    assert abs(out[4] - float(ref[4])) <= 1e-5 * max(1.0, abs(float(ref[4])))


def test_map_signature_matches_reference_inputs():
    case, g = G.load('cyl32x16')
    rcf = _solver(case)
    inputs = rcf.mapInputs(*_init(g), float(g['dt0']))
    out = rcf.map(*inputs)
    assert [o.shape for o in out] == [(case.build_mesh().nInternalCells, 1), (case.build_mesh().nInternalCells, 3),
                                      (case.build_mesh().nInternalCells, 1), (1, 1), (1, 1)]
    # changing a BC tensor input changes the result (the values are per-call inputs)
    bct = rcf.getBoundaryTensor(1)
    pos = 4 + 15 + len(case.build_mesh().getScalar()) + 3
    inputs2 = list(inputs)
    inputs2[pos + len(bct) - 1] = bct[-1] * 1.01    # far-field p0
    out2 = rcf.map(*inputs2)
    assert not np.array_equal(out[2], out2[2])
    out3 = rcf.map(*inputs)
    assert np.array_equal(out[2], out3[2])


@pytest.mark.parametrize('name', sorted(TINY))
def test_tiny_meshes_against_oracle(name):
    """One cell (no internal face; a periodic cube cyclic to itself), two cells, a one-cell-thick
    channel, the smallest O-grid: FP64 within 1e-12 of the oracle; FP32 and mixed run and stay
    within their one-step bounds."""
    case = TINY[name]()
    mesh = case.build_mesh()
    x = [np.asarray(a) for a in cases.conservative(case)]
    ref = torch_ref.Problem(mesh, case.bc, case.config, case.objective).step(
        *[torch.as_tensor(a) for a in x], case.dt)
    for precision, tol in (('fp64', 1e-12), ('fp32', 1e-5), ('mixed', 1e-6)):
        rcf = RCF(mesh, case.bc, objective=case.objective, precision=precision, **case.config)
        td = torch.float32 if precision == 'fp32' else torch.float64
        d = [torch.as_tensor(a).to(td).cuda() for a in x]
        out = rcf.step(d[0], d[1], d[2], case.dt)
        for i in range(3):
            e = G.rel_err(out[i].double().cpu().numpy(), ref[i].numpy())
            assert e < tol, (name, precision, i, e)
        assert abs(out[3] - float(ref[3])) <= max(tol, 1e-12) * abs(float(ref[3])), (name, precision)
        rcf.close()


def test_sharp_sod_nonfinite_like_reference():
    """One-cell Sod jump (the reference's own shock-tube set-up): the reference's first step
    returns a non-finite CFL sum and a state non-finite around the jump, and its solver stops
    there (Field.info -> MPI Abort). Through the C ABI the same step returns
    AFVM_ERR_NONFINITE, leaves non-finite values in exactly the same entries, and matches the
    reference elsewhere within 1e-12."""
    from adfvm_gb300 import _lib as L
    case, g = G.load_sharp_sod()
    rcf = _solver(case)
    n = case.build_mesh().nInternalCells
    d = [torch.as_tensor(g[k + '_init']).reshape(n, -1).cuda() for k in ('rho', 'rhoU', 'rhoE')]
    out = [torch.empty_like(t) for t in d]
    with pytest.raises(L.AfvmError) as ei:
        rcf.step(d[0], d[1], d[2], float(g['dt0']), out=out)
    assert ei.value.status == L.AFVM_ERR_NONFINITE
    for i, nm in enumerate(['rho', 'rhoU', 'rhoE']):
        same, e = G.nonfinite_parity(out[i].cpu().numpy(), g[nm + '_1'])
        assert same, '%s: non-finite entries differ from the reference' % nm
        assert e < 1e-12, '%s finite entries: rel err %.3e' % (nm, e)
    # the same state through the reference-facing map: the error reaches the caller
    inputs = rcf.mapInputs(*[g[k + '_init'] for k in ('rho', 'rhoU', 'rhoE')], float(g['dt0']))
    with pytest.raises(L.AfvmError):
        rcf.map(*inputs)
