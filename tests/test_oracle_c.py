"""The C restatement (timed CPU baseline) against the reference's own trajectories."""
import numpy as np
import pytest

from adfvm_gb300 import cases
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


# edge cases of the mesh: one cell (no internal face; a periodic cube whose six faces are cyclic
# to itself), two cells, a one-cell-thick channel, the smallest O-grid
TINY = {'sod1': lambda: cases.sod(1), 'sod2': lambda: cases.sod(2), 'box1': lambda: cases.box(1),
        'box2': lambda: cases.box(2), 'vane2x1': lambda: cases.vane_channel(2, 1),
        'cyl4x2': lambda: cases.cylinder(4, 2)}


@pytest.mark.parametrize('name', sorted(TINY))
def test_tiny_meshes_c_oracle_equals_torch_oracle(name):
    """Both oracles agree to 1e-12 on the smallest meshes."""
    import torch
    from oracle import torch_ref
    case = TINY[name]()
    mesh = case.build_mesh()
    x = [np.asarray(a) for a in cases.conservative(case)]
    r0 = torch_ref.Problem(mesh, case.bc, case.config, case.objective).step(
        *[torch.as_tensor(a) for a in x], case.dt)
    r1 = COracle(mesh, case.bc, case.config, case.objective).step(x[0], x[1], x[2], case.dt, None)
    for i in range(3):
        assert G.rel_err(r1[i], r0[i].numpy()) < 1e-12, (name, i)
    assert abs(r1[3] - float(r0[3])) <= 1e-12 * abs(float(r0[3]))
    assert abs(r1[4] - float(r0[4])) <= 1e-12 * max(1.0, abs(float(r0[4])))
