"""The C restatement (timed CPU baseline) against the reference's own trajectories."""
import numpy as np
import pytest

from oracle.c_ref import COracle
from tests import golden_cases as G


@pytest.mark.parametrize('name', G.available())
def test_c_oracle_matches_reference_trajectory(name):
    case, g = G.load(name)
    mesh = case.build_mesh()
    co = COracle(mesh, case.bc, case.config, case.objective)
    x = [np.asarray(g[k + '_init']) for k in ('rho', 'rhoU', 'rhoE')]
    S = None
    if bool(g['with_source']):
        from adfvm_gb300 import cases
        S = cases.source_field(mesh)
    dt = float(g['dt0'])
    cfl = case.config.get('CFL', 1.2)
    sf = case.config.get('stepFactor', 1.2)
    fixed = case.config.get('fixedTimeStep', False)
    rec = []
    keep = set(int(s) for s in g['steps'])
    for n in range(1, int(g['nSteps']) + 1):
        r = co.step(x[0], x[1], x[2], dt, S)
        rec.append((dt, r[3], r[4]))
        x = list(r[:3])
        if n in keep:
            for i, nm in enumerate(['rho', 'rhoU', 'rhoE']):
                assert G.rel_err(x[i], g['%s_%d' % (nm, n)]) < 1e-12, (nm, n)
        if not fixed:
            dt = min(2 * cfl / r[3], dt * sf)
    rec = np.array(rec)
    for k in range(3):
        assert G.rel_err(rec[:, k], g['record'][:, k]) < 1e-12
