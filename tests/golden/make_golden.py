"""Generate the golden trajectories in tests/golden/*.npz from the REFERENCE solver itself.

Runs the reference's own RCF residual, SSP-RK3 stepper and time loop (adFVM/density.py,
interp.py, riemann.py, op.py, timestep.py, BCs.py, solver.py) and its own mesh builder
(adFVM/cpp/cmesh.cpp, compiled by oracle/build.py), through the adpy/mpi4py stand-ins of
oracle/refshim, on meshes from adfvm_gb300.meshgen. Needs the reference checkout, so it runs
in the development container only; the .npz files it writes are committed.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py sod1000    # one case
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from adfvm_gb300 import cases  # noqa: E402
from oracle import refrun  # noqa: E402


def mesh_digest(md):
    h = hashlib.sha256()
    for a in md[:4]:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def objective_fn(kind, rcf_cfg):
    """Objectives written in the adpy style of the reference's case files."""
    from adpy.tensor import Kernel, Zeros, ExternalFunctionOp
    if kind == 'none':
        return None
    if kind == 'kinetic_energy':
        def objective(fields, solver):
            U, T, p = fields
            mesh = solver.mesh.symMesh

            def _ke(U, T, p, volumes):
                rho = p / ((solver.Cv * T) * (solver.gamma - 1))
                return (0.5 * rho * U.magSqr() * volumes).sum()
            return Kernel(_ke)(mesh.nInternalCells)(U, T, p, mesh.volumes)
        return objective
    if kind == 'sum_T':
        def objective(fields, solver):
            U, T, p = fields
            mesh = solver.mesh.symMesh
            return Kernel(lambda T: (T * 1).sum())(mesh.nInternalCells)(T)
        return objective
    if kind.startswith('drag:'):
        patch_name = kind.split(':', 1)[1]

        # templates/cylinder_test.py:9-37
        def objectiveDrag(U, T, p, *mesh, **options):
            from adFVM.mesh import Mesh
            solver = options['solver']
            mesh = Mesh.container(mesh)
            U0 = U.extract(mesh.neighbour)[0]
            U0i = U.extract(mesh.owner)[0]
            p0 = p.extract(mesh.neighbour)
            T0 = T.extract(mesh.neighbour)
            nx = mesh.normals[0]
            mungUx = solver.mu(T0) * (U0 - U0i) / mesh.deltas
            drag = (p0 * nx - mungUx) * mesh.areas
            return drag.sum()

        def objective(fields, solver):
            U, T, p = fields
            mesh = solver.mesh.symMesh
            patch = mesh.boundary[patch_name]
            startFace, nFaces = patch['startFace'], patch['nFaces']
            meshArgs = [x[startFace] for x in mesh.getTensor()]
            drag = Zeros((1, 1))
            drag = Kernel(objectiveDrag)(nFaces, (drag,))(U, T, p, *meshArgs, solver=solver)
            (drag,) = ExternalFunctionOp('mpi_allreduce', (drag,), (drag,)).outputs
            return drag
        return objective
    raise ValueError(kind)


def reference_config(case):
    """(RCF options, hook run before the step function is compiled)."""
    cfg = dict(case.config)
    if 'mu' in cfg and not callable(cfg['mu']):
        v = float(cfg['mu'])
        cfg['mu'] = lambda T, v=v: v
    if isinstance(case.objective, dict):
        # the reference's own turbine-vane objective (adFVM/objectives/vane.py) with its own
        # getPlane/getWeights; the compiled compat.intersectPlane it calls is replaced by the
        # plane cells and areas of adfvm_gb300.vane (the only input not computed by that file)
        import adFVM.objectives.vane as V
        cells = np.asarray(case.objective['planeCells'], np.int32)
        areas = np.asarray(case.objective['planeAreas'], np.float64).reshape(-1, 1)
        V.intersectPlane = lambda mesh, point, normal: (cells, areas)
        cfg['objective'] = V.objective

        def hook(rcf):
            V.getPlane(rcf)
            V.getWeights(rcf)
        return cfg, hook
    obj = objective_fn(case.objective, cfg)
    if obj is not None:
        cfg['objective'] = obj
    return cfg, None


def run_case(case, nSteps, keep_steps, with_source=False):
    refrun.load()
    md = case.meshData
    with tempfile.TemporaryDirectory() as d:
        cfg, hook = reference_config(case)
        rcf, cons = refrun.make_rcf(md, d, case.bc, case.U, case.T, case.p, before_compile=hook, **cfg)
        src = None
        if with_source:
            S = cases.source_field(case.build_mesh())
            src = lambda fields, mesh, t: [x.copy() for x in S]
        sols, record = refrun.run_forward(rcf, nSteps, case.dt, source=src)
    out = {
        'mesh_digest': np.array(mesh_digest(md)),
        'nSteps': np.array(nSteps),
        'dt0': np.array(case.dt),
        'with_source': np.array(with_source),
        'record': np.array(record),   # per step: dt, dtc (stage-1 max), obj (stage-1)
        'steps': np.array(keep_steps),
        'U0': case.U, 'T0': case.T, 'p0': case.p,
    }
    for k, name in enumerate(['rho', 'rhoU', 'rhoE']):
        out[name + '_init'] = np.asarray(cons[k].field)
        for s in keep_steps:
            out['%s_%d' % (name, s)] = np.asarray(sols[s][k].field)
    return out


CASES = {
    'sod1000': lambda: (cases.sod(1000), 200, [1, 2, 10, 50, 100, 200], False),
    'sod200_sym_lf': lambda: (cases.sod(200, side='symmetryPlane', riemann='eulerLaxFriedrichs'), 60, [1, 20, 60], False),
    'box8': lambda: (cases.box(8, objective='kinetic_energy'), 5, [1, 2, 5], True),
    'box6_inviscid_sumT': lambda: (cases.box(6, objective='sum_T', viscous=False), 3, [1, 3], False),
    'cyl32x16': lambda: (cases.cylinder(32, 16, objective='drag:cylinder'), 5, [1, 2, 5], False),
    'duct100_totalpt': lambda: (cases.duct(100), 40, [1, 10, 40], False),
    'duct60_totalpt_normals': lambda: (cases.duct(60, direction=False, U0=-20.0), 20, [1, 20], False),
    'vane32x12': lambda: (cases.vane_channel(32, 12, reference_constants=True), 20, [1, 5, 20], False),
}


GEOMETRY_FIELDS = ['normals', 'faceCentres', 'areas', 'cellCentres', 'volumes', 'neighbour', 'deltas',
                   'deltasUnit', 'weights', 'linearWeights', 'quadraticWeights', 'cellFaces', 'cellOwner',
                   'cellNeighbours', 'volumesL', 'volumesR']
GEOMETRY_MESHES = {
    'sod50': lambda: cases.meshgen.sod_tube(50),
    'box6': lambda: cases.meshgen.periodic_box(6),
    'cyl16x8': lambda: cases.meshgen.cylinder_ogrid(16, 8),
}


def make_geometry():
    """Mesh arrays from the reference's own Mesh.build (adFVM/mesh.py:84-127): its compiled
    cmesh.cpp and its createGhostCells."""
    refrun.load()
    out = {}
    for name, fn in GEOMETRY_MESHES.items():
        md = fn()
        with tempfile.TemporaryDirectory() as d:
            m = refrun.build_mesh(md, d)
        out[name + '/digest'] = np.array(mesh_digest(md))
        out[name + '/sortedPatches'] = np.array(m.sortedPatches)
        for a in GEOMETRY_FIELDS + ['nLocalCells', 'nCells', 'nGhostCells', 'nLocalFaces', 'nRemoteCells']:
            out[name + '/' + a] = np.asarray(getattr(m, a))
    path = os.path.join(HERE, 'geometry.npz')
    np.savez_compressed(path, **out)
    print('geometry ->', path, os.path.getsize(path), 'bytes')


def make_energy():
    """cmesh.computeEnergy (adFVM/cpp/cmesh.cpp:342-425), the reference's compiled adjoint
    energy, on seeded adjoint fields over box6 and cyl16x8 states."""
    refrun.load()
    from oracle.refrun import load
    ns = load()
    import adFVM.mesh as rmesh
    out = {}
    for name, mk in [('box6', lambda: cases.box(6, objective='kinetic_energy')),
                     ('cyl16x8', lambda: cases.cylinder(16, 8))]:
        case = mk()
        with tempfile.TemporaryDirectory() as d:
            refrun.build_mesh(case.meshData, d)     # sets the builder's current mesh
        rho, rhoU, rhoE = cases.conservative(case)
        rng = np.random.default_rng(11)
        n = len(rho)
        rhoa, rhoUa, rhoEa = rng.normal(size=(n, 1)), rng.normal(size=(n, 3)), rng.normal(size=(n, 1)) * 1e-5

        class Solver:
            gamma = 1.4
        e = rmesh.cmesh.computeEnergy(Solver(), rhoa, rhoUa, rhoEa, rho, rhoU, rhoE)
        out[name + '/energy'] = np.array(e)
        for k, v in dict(rhoa=rhoa, rhoUa=rhoUa, rhoEa=rhoEa, rho=rho, rhoU=rhoU, rhoE=rhoE).items():
            out[name + '/' + k] = v
    path = os.path.join(HERE, 'energy.npz')
    np.savez_compressed(path, **out)
    print('energy ->', path, {k: float(v) for k, v in out.items() if k.endswith('/energy')})


VISCOSITY_CASES = {'cyl16x8': lambda: cases.cylinder(16, 8), 'box6': lambda: cases.box(6),
                   'vane16x8': lambda: cases.vane_channel(16, 8)}


def make_viscosity():
    """The adjoint stabilisation of the reference itself: postpro.computeAdjointViscosity
    (adFVM/postpro.py:491-697) for the 'turkel', 'abarbanel' and 'uniform' symmetrisers and
    postpro.viscositySolver (postpro.py:699-718), on seeded states. Their two compiled helpers
    are restated for the stand-in: get_max_eigenvalue (scaling.cpp:84-104, the largest
    eigenvalue of each symmetric 5x5) and apply_adjoint_viscosity (scaling.cpp:135-159: the
    implicit heat equation of matop_petsc.cpp:230-372, here solved exactly by sparse LU)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    ns = refrun.load()
    import adpy.tensor as AT
    from adpy.tensor import Variable, Function
    from adFVM import postpro
    out = {}
    AT.EXTERNAL['get_max_eigenvalue'] = lambda MS: [np.linalg.eigvalsh(MS.reshape(-1, 5, 5))[:, -1].reshape(-1, 1)]
    for name, mk in VISCOSITY_CASES.items():
        case = mk()
        cfg, hook = reference_config(case)
        with tempfile.TemporaryDirectory() as d:
            rcf, cons = refrun.make_rcf(case.meshData, d, case.bc, case.U, case.T, case.p, before_compile=hook, **cfg)
        m = rcf.mesh
        n = m.nInternalCells
        V = np.asarray(m.volumes).reshape(-1)
        cf = np.asarray(m.cellFaces).reshape(-1, 6)
        cn = np.asarray(m.cellNeighboursMatOp).reshape(-1, 6)

        def heat(u0, u1, u2, u3, u4, rho, rhoU, rhoE, DTF, dt):
            dtv = float(np.asarray(dt).reshape(-1)[0])
            DTF = np.asarray(DTF).reshape(-1)
            rows, cols, vals = [], [], []
            diag = np.ones(n)
            for k in range(6):
                ok = cn[:, k] > -1
                coef = -DTF[cf[:, k]] / V * dtv
                diag -= np.where(ok, coef, 0.0)
                rows.append(np.arange(n)[ok]); cols.append(cn[ok, k]); vals.append(coef[ok])
            A = sp.csr_matrix((np.concatenate(vals + [diag]), (np.concatenate(rows + [np.arange(n)]),
                                                              np.concatenate(cols + [np.arange(n)]))), shape=(n, n))
            lu = spla.splu(A.tocsc())
            return [lu.solve(np.asarray(u).reshape(-1)).reshape(-1, 1) for u in (u0, u1, u2, u3, u4)]
        AT.EXTERNAL['apply_adjoint_viscosity'] = heat
        rng = np.random.default_rng(21)
        x = [a * (1 + 0.01 * rng.standard_normal(a.shape)) for a in cases.conservative(case)]
        sm = m.symMesh
        meshIn = sm.getTensor() + sm.getScalar() + rcf.getBoundaryTensor(0) + [v[0] for v in rcf.extraArgs]
        meshVal = m.getTensor() + m.getScalar() + rcf.getBoundaryTensor(1) + [v[1] for v in rcf.extraArgs]
        for k, nm in enumerate(['rho', 'rhoU', 'rhoE']):
            out['%s/%s' % (name, nm)] = x[k]
        for kind, scale in (('turkel', 1e-3), ('abarbanel', 0.5), ('uniform', 2.0)):
            rho, rhoU, rhoE = Variable((n, 1)), Variable((n, 3)), Variable((n, 1))
            scaling = Variable((1, 1))
            M2, DT = postpro.computeAdjointViscosity(rcf, kind, rho, rhoU, rhoE, scaling)
            F = Function('viscosity', [rho, rhoU, rhoE, scaling] + meshIn, [M2, DT])
            M2v, DTv = F(x[0], x[1], x[2], np.array([[scale]]), *meshVal)
            out['%s/%s/scaling' % (name, kind)] = np.array(scale)
            out['%s/%s/M' % (name, kind)] = M2v.reshape(-1)
            out['%s/%s/DT' % (name, kind)] = DTv.reshape(-1)
        # the smoother on seeded adjoint fields with the 'abarbanel' DT and a large dt
        a = [rng.standard_normal((n, 1)), rng.standard_normal((n, 3)), rng.standard_normal((n, 1))]
        rho, rhoU, rhoE = Variable((n, 1)), Variable((n, 3)), Variable((n, 1))
        ra, rUa, rEa = Variable((n, 1)), Variable((n, 3)), Variable((n, 1))
        DT = Variable((m.nFaces, 1))
        outs = postpro.viscositySolver(rcf, rho, rhoU, rhoE, ra, rUa, rEa, DT)
        dt = 1e-2 if name != 'vane16x8' else 1e-6
        F = Function('smooth', [rho, rhoU, rhoE, ra, rUa, rEa, DT, rcf.dt] + meshIn, list(outs))
        res = F(x[0], x[1], x[2], a[0], a[1], a[2], out['%s/abarbanel/DT' % name].reshape(-1, 1),
                np.array([[dt]]), *meshVal)
        out['%s/smooth/dt' % name] = np.array(dt)
        for k, nm in enumerate(['rhoa', 'rhoUa', 'rhoEa']):
            out['%s/smooth/in_%s' % (name, nm)] = a[k]
            out['%s/smooth/out_%s' % (name, nm)] = res[k]
    path = os.path.join(HERE, 'viscosity.npz')
    np.savez_compressed(path, **out)
    print('viscosity ->', path, os.path.getsize(path), 'bytes')


def make_sod_sharp():
    """The Sod tube with the one-cell jump of the reference's own shock-tube case
    (cases/shockTube/system/setFieldsDict: p 1e5 | 1e4, T 348.4 | 278.7 K): the reference's first
    step map call returns a non-finite CFL sum and a state that is non-finite in the cells around
    the jump, after which its Solver.run stops (Field.info -> MPI Abort, adFVM/field.py:36-53).
    Records that call's outputs."""
    refrun.load()
    case = cases.sod(1000, smooth_cells=None)
    with tempfile.TemporaryDirectory() as d:
        cfg, hook = reference_config(case)
        rcf, cons = refrun.make_rcf(case.meshData, d, case.bc, case.U, case.T, case.p, before_compile=hook, **cfg)
        inputs = ([c.field for c in cons] + [np.array([[case.dt]])] + rcf.mesh.getTensor() + rcf.mesh.getScalar() +
                  [x[1] for x in rcf.sourceTerms] + rcf.getBoundaryTensor(1) + [x[1] for x in rcf.extraArgs])
        out = rcf.map(*inputs, return_reusable=True, replace_reusable=True)
    res = {'mesh_digest': np.array(mesh_digest(case.meshData)), 'dt0': np.array(case.dt),
           'dtc': np.array(float(out[3][0, 0])), 'obj': np.array(float(out[4][0, 0]))}
    for k, name in enumerate(['rho', 'rhoU', 'rhoE']):
        res[name + '_init'] = np.asarray(cons[k].field)
        res[name + '_1'] = np.asarray(out[k])
    path = os.path.join(HERE, 'sod1000_sharp.npz')
    np.savez_compressed(path, **res)
    bad = np.where(~np.isfinite(res['rho_1']).all(axis=1))[0]
    print('sod1000_sharp: dtc %r, non-finite cells %s -> %s' % (float(res['dtc']), bad.tolist(), path))


def main(names):
    for name in names:
        if name == 'sod1000_sharp':
            make_sod_sharp()
            continue
        if name == 'geometry':
            make_geometry()
            continue
        if name == 'energy':
            make_energy()
            continue
        if name == 'viscosity':
            make_viscosity()
            continue
        case, nSteps, keep, src = CASES[name]()
        out = run_case(case, nSteps, keep, src)
        path = os.path.join(HERE, name + '.npz')
        np.savez_compressed(path, **out)
        rec = out['record']
        print('%s: %d steps, final dt %.6e dtc %.6e obj %.6e -> %s (%d bytes)' % (
            name, nSteps, rec[-1, 0], rec[-1, 1], rec[-1, 2], path, os.path.getsize(path)))


if __name__ == '__main__':
    main(sys.argv[1:] or (['geometry', 'energy', 'viscosity', 'sod1000_sharp'] + list(CASES)))
