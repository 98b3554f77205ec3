"""Run the reference's own solver code on CPU (test infrastructure, this container only).

Imports the reference package from its checkout with three stand-ins in front of it:
``oracle/refshim/adpy`` (NumPy evaluator of the adpy DSL), ``oracle/refshim/mpi4py``
(one rank) and the reference's own adFVM/cpp/cmesh.cpp compiled by ``oracle/build.py``
into ``oracle/_ref``. The case set-up replaces the file readers only: meshes come from
``adfvm_gb300.meshgen`` through the reference's ``Mesh.build`` (adFVM/mesh.py:84-127), fields
are handed to the reference ``IOField``/``CellField`` objects exactly as
``RCF.readFields`` builds them (adFVM/density.py:113-137), and time stepping is the
reference's ``Solver.run`` (adFVM/solver.py:210-411) in ``mode='forward'``.
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
from .build import REFERENCE  # noqa: E402  (the one place the checkout's location is set)

_loaded = {}


def load():
    """Import the reference modules; returns a namespace with density, mesh, field, BCs."""
    if _loaded:
        return _loaded['ns']
    from . import build as obuild
    so = obuild.build_ref()
    if so is None:
        raise RuntimeError('reference checkout not available at %s' % REFERENCE)
    sys.path.insert(0, os.path.join(HERE, 'refshim'))
    sys.path.insert(1, REFERENCE)
    saved_argv = sys.argv
    sys.argv = [sys.argv[0]]
    spec = importlib.util.spec_from_file_location('cmesh', so)
    cmesh = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cmesh)
    cpp = types.ModuleType('adFVM.cpp')
    cpp.cmesh = cmesh
    cpp.cmesh_gpu = cmesh
    sys.modules['adFVM.cpp'] = cpp
    sys.modules['adFVM.cpp.cmesh'] = cmesh
    compat = types.ModuleType('adFVM.compat')
    for name in ['intersectPlane', 'reduceAbsMin', 'selectMultipleRange', 'reduceSum']:
        setattr(compat, name, None)
    sys.modules['adFVM.compat'] = compat
    import adFVM  # noqa: F401
    adFVM.cpp = cpp
    adFVM.compat = compat
    from adFVM import config, density, mesh, field, BCs, timestep, solver  # noqa: F401
    sys.argv = saved_argv
    ns = types.SimpleNamespace(config=config, density=density, mesh=mesh, field=field, BCs=BCs,
                               timestep=timestep, solver=solver)
    _loaded['ns'] = ns
    return ns


class LegacyArray(np.ndarray):
    """ndarray with NumPy 1's ``tostring`` (removed in NumPy 2), which the reference's file
    writers call (field.py writeField, mesh.py writeFoamFile)."""

    def tostring(self):
        return self.tobytes()


class _LegacyNumpy(types.ModuleType):
    """numpy with NumPy 1's binary ``fromstring`` (a copying ``frombuffer``), which the
    reference's file readers call (mesh.py readFoamFile, extractField)."""

    def __init__(self):
        super().__init__('numpy')

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def fromstring(data, dtype=float, count=-1, sep=''):
        if sep:
            return np.fromstring(data, dtype, count, sep)
        return np.frombuffer(data, dtype, count).copy()


def legacy_numpy():
    """Let the reference's mesh/field file IO run on this NumPy (idempotent)."""
    ns = load()
    shim = _LegacyNumpy()
    for mod in (ns.mesh, ns.field):
        mod.np = shim
    return ns


def build_mesh(meshData, case_dir):
    ns = load()
    points, faces, owner, neighbour, boundary = meshData
    m = ns.mesh.Mesh()
    m.case = case_dir.rstrip('/') + '/'
    m.caseDir = m.case
    bnd = {k: dict(v) for k, v in boundary.items()}
    m.build((points.copy(), faces.copy(), owner.copy(), neighbour.copy(), [], bnd))
    return m


def make_rcf(meshData, case_dir, fields_bc, U, T, p, before_compile=None, **rcf_config):
    """Construct the reference RCF solver on a generated mesh.

    fields_bc: {'U': {patch: bcdict}, 'T': ..., 'p': ...} in the reference's boundary-dict
    form ({'type': ..., 'value'/'U0'/'T0'/'p0': ndarray}). U, T, p: internal-cell values.
    Returns (rcf, conservative_fields) where the latter is what readFields returns.
    before_compile(rcf), if given, runs before the step function is compiled (where a case file
    calls helpers that append solver.extraArgs, e.g. objectives/vane.py getPlane/getWeights).
    """
    ns = load()
    density = ns.density
    mesh = build_mesh(meshData, case_dir)
    Mesh = ns.mesh.Mesh
    orig_create = Mesh.__dict__['create']
    Mesh.create = classmethod(lambda cls, caseDir=None, currTime='constant': mesh)
    # Solver.__init__ mutates the class-level defaults; start from a clean copy
    saved_defaults = density.RCF.defaultConfig.copy()
    try:
        rcf = density.RCF(case_dir, **rcf_config)
    finally:
        Mesh.create = orig_create
        density.RCF.defaultConfig = saved_defaults
    IOField = ns.field.IOField
    fields = []
    for name, val, dims in [('U', U, (3,)), ('T', T, (1,)), ('p', p, (1,))]:
        phi = IOField(name, np.ascontiguousarray(val, np.float64).reshape((-1,) + dims), dims,
                      {k: dict(v) for k, v in fields_bc[name].items()})
        fields.append(phi)
    # RCF.readFields, first-run branch (adFVM/density.py:128-137)
    rcf.U, rcf.T, rcf.p = fields
    rcf.fields = fields
    for phi in rcf.fields:
        phi.completeField()
    rcf.gradFields = [ns.field.CellField(phi.name, None, phi.dimensions + (3,)) for phi in rcf.fields]
    rcf.firstRun = False
    cons = list(rcf.conservative(*rcf.fields))
    rcf.readFields = lambda t, suffix='': cons
    if before_compile is not None:
        before_compile(rcf)
    rcf.compileInit()
    rcf.compileSolver()
    return rcf, cons


def run_forward(rcf, nSteps, dt, source=None, startTime=0.0):
    """Reference Solver.run in forward mode; records (dt, dtc, obj) of every map call."""
    record = []
    orig_map = rcf.map

    def recording_map(*inputs, **options):
        out = orig_map(*inputs, **options)
        record.append((float(np.asarray(inputs[3]).reshape(-1)[0]), float(out[3][0, 0]), float(out[4][0, 0])))
        return out

    rcf.map = recording_map
    kwargs = {}
    if source is not None:
        kwargs['source'] = source
    sols = rcf.run(startTime=startTime, dt=dt, nSteps=nSteps, mode='forward', **kwargs)
    rcf.map = orig_map
    return sols, record
