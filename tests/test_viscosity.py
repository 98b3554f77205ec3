"""Adjoint stabilisation (artificial viscosity) of the oracle against the reference's own
postpro.computeAdjointViscosity / viscositySolver (tests/golden/viscosity.npz, made by
tests/golden/make_golden.py through the adpy stand-in), on the host.

Tolerances: the viscosity M and face values DT within 1e-12 relative (max|x-ref|/max|ref|);
the smoothed adjoint within 1e-10 (both sides solve the sparse system, by different
factorisations)."""
import os

import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from oracle import torch_ref
from tests import golden_cases as G

PATH = os.path.join(G.HERE, 'viscosity.npz')
CASES = {'cyl16x8': lambda: cases.cylinder(16, 8), 'box6': lambda: cases.box(6),
         'vane16x8': lambda: cases.vane_channel(16, 8)}


def _load(name):
    g = np.load(PATH)
    case = CASES[name]()
    m = case.build_mesh()
    prob = torch_ref.Problem(m, case.bc, case.config, case.objective)
    x = [g['%s/%s' % (name, k)] for k in ('rho', 'rhoU', 'rhoE')]
    return g, case, prob, x


@pytest.mark.parametrize('name', list(CASES))
@pytest.mark.parametrize('kind', ['turkel', 'abarbanel', 'uniform'])
def test_oracle_viscosity_matches_reference(name, kind):
    g, case, prob, x = _load(name)
    s = float(g['%s/%s/scaling' % (name, kind)])
    M, DT = torch_ref.adjoint_viscosity(prob, x[0], x[1], x[2], kind, s)
    assert G.rel_err(M, g['%s/%s/M' % (name, kind)][:len(M)]) < 1e-12
    assert G.rel_err(DT, g['%s/%s/DT' % (name, kind)]) < 1e-12


@pytest.mark.parametrize('name', list(CASES))
def test_oracle_smoother_matches_reference(name):
    g, case, prob, x = _load(name)
    dt = float(g['%s/smooth/dt' % name])
    a = [g['%s/smooth/in_%s' % (name, k)] for k in ('rhoa', 'rhoUa', 'rhoEa')]
    out = torch_ref.viscosity_solve(prob, g['%s/abarbanel/DT' % name], dt, *a)
    for k, nm in enumerate(['rhoa', 'rhoUa', 'rhoEa']):
        assert G.rel_err(out[k], g['%s/smooth/out_%s' % (name, nm)]) < 1e-10, nm
    # the smoothing is not the identity at this dt
    assert G.rel_err(out[0], a[0]) > 1e-3 or name == 'vane16x8'
