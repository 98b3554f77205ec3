"""Adjoint stabilisation on the GPU (afvm_adjoint_viscosity) against the reference's own
postpro.computeAdjointViscosity / viscositySolver (tests/golden/viscosity.npz).

Tolerances: the viscosity and its face values within 1e-12 relative in FP64 (the largest
eigenvalue comes from Jacobi rotations here and LAPACK there); the smoothed adjoint within
1e-10 (CG to a relative residual of 1e-13 here, a direct solve there); FP32 contexts (whose
mesh tables and state are FP32) and mixed ones (FP32 mesh tables and records, FP64 state)
within 1e-5."""
import numpy as np
import pytest
import torch

from adfvm_gb300.solver import RCF
from tests import golden_cases as G
from tests.test_viscosity import CASES, PATH

pytestmark = pytest.mark.gpu


def _setup(name, precision='fp64'):
    g = np.load(PATH)
    case = CASES[name]()
    m = case.build_mesh()
    rcf = RCF(m, case.bc, objective=case.objective, precision=precision, **case.config)
    td = torch.float32 if precision == 'fp32' else torch.float64
    x = [torch.as_tensor(g['%s/%s' % (name, k)]).to(td).cuda() for k in ('rho', 'rhoU', 'rhoE')]
    return g, m, rcf, x, td


@pytest.mark.parametrize('name', list(CASES))
@pytest.mark.parametrize('kind', ['turkel', 'abarbanel', 'uniform'])
def test_viscosity_fields_match_reference(name, kind):
    g, m, rcf, x, td = _setup(name)
    s = float(g['%s/%s/scaling' % (name, kind)])
    a = [torch.zeros_like(t) for t in x]
    it, M, DT = rcf.adjoint_viscosity(x[0], x[1], x[2], a, 1e-6, kind, s, want_fields=True)
    assert G.rel_err(M.cpu().numpy()[:m.nInternalCells], g['%s/%s/M' % (name, kind)][:m.nInternalCells]) < 1e-12
    assert G.rel_err(DT.cpu().numpy(), g['%s/%s/DT' % (name, kind)]) < 1e-12
    for t in a:
        assert torch.count_nonzero(t) == 0          # zero stays zero


@pytest.mark.parametrize('name', list(CASES))
@pytest.mark.parametrize('precision', ['fp64', 'fp32', 'mixed'])
def test_smoother_matches_reference(name, precision):
    g, m, rcf, x, td = _setup(name, precision)
    dt = float(g['%s/smooth/dt' % name])
    a = [torch.as_tensor(g['%s/smooth/in_%s' % (name, k)]).to(td).cuda() for k in ('rhoa', 'rhoUa', 'rhoEa')]
    it = rcf.adjoint_viscosity(x[0], x[1], x[2], a, dt, 'abarbanel', float(g['%s/abarbanel/scaling' % name]))
    tol = 1e-10 if precision == 'fp64' else 1e-5
    for k, nm in enumerate(['rhoa', 'rhoUa', 'rhoEa']):
        assert G.rel_err(a[k].double().cpu().numpy(), g['%s/smooth/out_%s' % (name, nm)]) < tol, (nm, it)
    assert 0 < it < 500


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_viscosity_fields_with_a_gauge_on_warped_faces(precision):
    """The jittered box (cells whose face area vectors do not close) with FP32 records holding
    gauge offsets: the pressure gradient of the viscosity puts the gauge pressure times each
    cell's sum of A/V N back, so the viscosity field matches the reference's as without a gauge."""
    from adfvm_gb300 import cases
    name = 'box6'
    g = np.load(PATH)
    case = CASES[name]()
    m = case.build_mesh()
    ref = g['%s/turkel/M' % name][:m.nInternalCells]
    s = float(g['%s/turkel/scaling' % name])
    errs = []
    for gauge in (None, cases.gauge(case)):
        rcf = RCF(m, case.bc, objective=case.objective, precision=precision, gauge=gauge, **case.config)
        td = torch.float32 if precision == 'fp32' else torch.float64
        x = [torch.as_tensor(g['%s/%s' % (name, k)]).to(td).cuda() for k in ('rho', 'rhoU', 'rhoE')]
        a = [torch.zeros_like(t) for t in x]
        _, M, _ = rcf.adjoint_viscosity(x[0], x[1], x[2], a, 1e-6, 'turkel', s, want_fields=True)
        errs.append(G.rel_err(M.cpu().numpy()[:m.nInternalCells], ref))
        rcf.close()
    assert max(errs) < 1e-4, errs
