"""Host-side mirror of the reference solver's call surface, backed by libafvm on one GPU.

``RCF`` takes the reference's options (adFVM/density.py:22-39, adFVM/solver.py:21-42) and
exposes:

* ``map(*inputs)`` - the compiled step function the reference's time loop calls
  (adFVM/solver.py:312-323): the same positional inputs ``[rho, rhoU, rhoE, dt] +
  mesh.getTensor() + mesh.getScalar() + sources + getBoundaryTensor(1)`` and the same outputs
  ``[rhoN, rhoUN, rhoEN, dtc (1,1), obj (1,1)]`` as numpy arrays;
* ``step(...)`` - the same step on device tensors (torch CUDA), no host copies;
* ``run(...)`` - the reference's ``Solver.run`` loop (time-step rule, ``round(t0+dt, 12)``,
  objective sum; adFVM/solver.py:210-411) in ``simulation``/``orig``/``perturb``/``forward``
  modes; on a case directory it writes the fields every ``writeInterval`` steps together with
  ``status.pkl``, and resumes from ``startIndex``/``result`` as apps/problem.py:76-80 does;
* ``fromCase(caseDir)``, ``readFields(t)``, ``writeFields(fields, t)`` - OpenFOAM case files
  (density.py:113-158): U, T, p are read with their boundary dicts; rho, rhoU, rhoE, U, T, p
  are written with the ghost-cell values of the boundary map as the patch values;
* ``run_device(...)`` - n steps resident on the GPU (``afvm_primal_run``).

``objective`` is one of the built-in kinds ('none', 'kinetic_energy', 'sum_T', 'drag:<patch>',
'vane') or, like a reference case file's ``objective(fields, solver)`` (adFVM/density.py:354-357),
a function ``objective([U, T, p], solver)`` returning a scalar torch tensor. It is called on
float64 CUDA tensors of the primitives of the step's second RK stage - every cell, ghosts
included - and ``solver`` gives ``mesh`` (the Mesh), ``meshTensor(name)`` (a mesh array as a
CUDA tensor), ``mu(T)``, ``gamma``, ``Cp``, ``Cv``, ``Pr``. Its adjoint seed is torch autograd
of the same function (afvm_set_objective_sink / afvm_set_objective_seed).
The GPU library is mandatory: there is no CPU path.
"""
import collections
import ctypes as C
import os
import sys

import numpy as np

from . import _lib as L
from . import foam
from .mesh import Mesh, CYCLIC_PATCHES

_BC = {'zeroGradient': L.AFVM_BC_ZERO_GRADIENT, 'empty': L.AFVM_BC_ZERO_GRADIENT,
       'inletOutlet': L.AFVM_BC_ZERO_GRADIENT, 'calculated': L.AFVM_BC_ZERO_GRADIENT,
       'fixedValue': L.AFVM_BC_FIXED_VALUE, 'symmetryPlane': L.AFVM_BC_SYMMETRY_PLANE,
       'slip': L.AFVM_BC_SYMMETRY_PLANE, 'cyclic': L.AFVM_BC_CYCLIC, 'CBC_UPT': L.AFVM_BC_CBC_UPT,
       'CBC_TOTAL_PT': L.AFVM_BC_CBC_TOTAL_PT}
_RIEMANN = {'eulerRoe': L.AFVM_RIEMANN_ROE, 'eulerLaxFriedrichs': L.AFVM_RIEMANN_LF}
DEFAULTS = {'Cp': 1004.5, 'gamma': 1.4, 'Pr': 0.7, 'CFL': 1.2, 'stepFactor': 1.2,
            'riemannSolver': 'eulerRoe', 'boundaryRiemannSolver': 'eulerRoe', 'mu': None,
            'fixedTimeStep': False, 'timeIntegrator': 'SSPRK', 'nStages': 3,
            'faceReconstructor': 'secondOrder'}
SUTHERLAND = (1.4792e-06, 116.)            # adFVM/density.py:27


def _torch():
    import torch
    return torch


class ObjectiveSolver(object):
    """What an objective written as a torch function sees as its ``solver`` argument: the gas
    constants, ``mu(T)`` (adFVM/density.py:27 for Sutherland), the Mesh, and its arrays as CUDA
    tensors (``meshTensor``); ``tensors`` replaces some of them (autograd leaves for the mesh
    gradient)."""

    def __init__(self, rcf, tensors=None):
        self._rcf = rcf
        self._tensors = tensors or {}
        self.mesh = rcf.mesh
        self.gamma, self.Cp, self.Cv, self.Pr = rcf.gamma, rcf.Cp, rcf.Cv, rcf.Pr

    def meshTensor(self, name):
        return self._tensors[name] if name in self._tensors else self._rcf.meshTensor(name)

    def mu(self, T):
        if self._rcf.mu is None:
            return SUTHERLAND[0] * T ** 1.5 / (T + SUTHERLAND[1])
        return T * 0 + float(self._rcf.mu)


class RCF(object):
    """GB300 drop-in for the reference RCF solver's residual/step evaluation."""

    names = ['rho', 'rhoU', 'rhoE']
    dimensions = [(1,), (3,), (1,)]

    def __init__(self, mesh, bc, objective='none', precision='fp64', device=0, gauge=None, **config):
        for k in config:
            if k not in DEFAULTS:
                raise ValueError('unknown RCF option %r' % k)
        cfg = dict(DEFAULTS)
        cfg.update(config)
        if cfg['timeIntegrator'] != 'SSPRK' or cfg['faceReconstructor'] != 'secondOrder':
            raise NotImplementedError('SSPRK with secondOrder reconstruction is the implemented path')
        self.config = cfg
        for k, v in cfg.items():
            setattr(self, k, v)
        self.Cv = self.Cp / self.gamma
        self.mesh = mesh if isinstance(mesh, Mesh) else Mesh.create(mesh)
        self.bc = bc
        # the turbine-vane objective: 'vane' (adFVM/objectives/vane.py's own plane and weights)
        # or a description from adfvm_gb300.vane.options(...)
        self.vane = None
        self.objectiveFn = objective if callable(objective) else None
        if isinstance(objective, dict) or objective == 'vane':
            from . import vane as _vane
            self.vane = dict(objective) if isinstance(objective, dict) else _vane.options(self.mesh)
            objective = 'vane'
        self.objective = objective
        # 'fp64'; 'fp32'; 'mixed': FP32 mesh tables, records, face fluxes and face arithmetic
        # with the conservative state, RK stages, sources and adjoints in FP64
        self.precision = {'fp64': L.AFVM_FP64, 'fp32': L.AFVM_FP32, 'mixed': L.AFVM_FP32_STATE64}[precision]
        self.dtype = np.float32 if self.precision == L.AFVM_FP32 else np.float64                # state
        self.record_dtype = np.float64 if self.precision == L.AFVM_FP64 else np.float32         # records
        self.device = device
        self._ctx = None
        self._create()
        # the gauge state (p, T, H) of the FP32 records ('fp32', 'mixed'): by default the
        # boundary conditions' (afvm_set_gauge); give one for a case whose boundaries fix no p or T
        if gauge is not None:
            L.check(L.lib().afvm_set_gauge(self._ctx, *[float(v) for v in gauge]), self._ctx, 'afvm_set_gauge')

    # ------------------------------------------------------------------ set-up
    def _physics(self):
        mu = self.mu
        if mu is None:
            model, mu0 = L.AFVM_MU_SUTHERLAND, 0.0
        elif callable(mu):
            raise NotImplementedError('mu must be None (Sutherland) or a constant')
        else:
            model, mu0 = L.AFVM_MU_CONSTANT, float(mu)
        obj, objPatch = L.AFVM_OBJ_NONE, -1
        if self.objectiveFn is not None:
            pass                          # evaluated on the host side of the sink (objective_value)
        elif self.vane is not None:
            obj = L.AFVM_OBJ_VANE
        elif self.objective == 'kinetic_energy':
            obj = L.AFVM_OBJ_KINETIC_ENERGY
        elif self.objective == 'sum_T':
            obj = L.AFVM_OBJ_SUM_T
        elif self.objective.startswith('drag:'):
            obj = L.AFVM_OBJ_DRAG
            objPatch = self.mesh.sortedPatches.index(self.objective.split(':', 1)[1])
        elif self.objective != 'none':
            raise ValueError('unknown objective %r' % self.objective)
        return L.Physics(self.gamma, self.Cp, self.Pr, model, mu0, SUTHERLAND[0], SUTHERLAND[1],
                         _RIEMANN[self.riemannSolver], _RIEMANN[self.boundaryRiemannSolver], obj, objPatch)

    def _bc_struct(self):
        m = self.mesh
        arr = (L.PatchBC * max(1, len(m.sortedPatches)))()
        keep = []
        for i, name in enumerate(m.sortedPatches):
            kinds = {f: self.bc[f][name]['type'] for f in ('U', 'T', 'p')}
            vals = {}
            for f, dims in (('U', 3), ('T', 1), ('p', 1)):
                b = self.bc[f][name]
                if b['type'] == 'fixedValue':
                    vals[f] = np.ascontiguousarray(b['value'], np.float64).reshape(-1, dims)
                elif b['type'] == 'CBC_UPT':
                    cb = self.bc['p'][name]       # characteristicBoundary uses p's BC (density.py:333-337)
                    vals[f] = np.ascontiguousarray(cb[f + '0'], np.float64).reshape(-1, dims)
                elif b['type'] == 'CBC_TOTAL_PT':
                    cb = self.bc['p'][name]
                    key = {'U': 'direction', 'T': 'Tt', 'p': 'pt'}[f]
                    if key in cb:
                        vals[f] = np.ascontiguousarray(cb[key], np.float64).reshape(-1, dims)
            keep.append(vals)
            ptr = lambda f: L.dptr(vals[f]) if f in vals else None
            arr[i] = L.PatchBC(_BC[kinds['U']], _BC[kinds['T']], _BC[kinds['p']], ptr('U'), ptr('T'), ptr('p'))
        return arr, keep

    def _create(self):
        mt, keep = self.mesh.tensorsStruct()
        bcs, keep2 = self._bc_struct()
        phys = self._physics()
        ctx = C.c_void_p()
        st = L.lib().afvm_ctx_create(C.byref(mt), bcs, C.byref(phys), self.precision, self.device, C.byref(ctx))
        L.check(st, None, 'afvm_ctx_create')
        self._ctx = ctx
        self._bcvals = self.getBoundaryTensor(1)
        if self.vane is not None:
            self._set_vane(self.vane)
        if self.objectiveFn is not None:
            torch = _torch()
            rd = torch.float64 if self.record_dtype == np.float64 else torch.float32
            self._objPrims = torch.empty((self.mesh.nCells, 5), dtype=rd, device='cuda:%d' % self.device)
            L.check(L.lib().afvm_set_objective_sink(self._ctx, C.c_void_p(self._objPrims.data_ptr())), self._ctx)

    def _set_vane(self, v):
        m = self.mesh
        cells = np.ascontiguousarray(v['planeCells'], np.int32).reshape(-1)
        areas = np.ascontiguousarray(v['planeAreas'], np.float64).reshape(-1)
        names = [p for p in m.sortedPatches if p in v['heat']]
        idx = np.array([m.sortedPatches.index(p) for p in names], np.int32)
        ws = [np.ascontiguousarray(v['heat'][p], np.float64).reshape(-1) for p in names]
        wp = (L._d * max(1, len(ws)))(*[L.dptr(w) for w in ws])
        d = L.ObjectiveVane(len(cells), L.iptr(cells), L.dptr(areas), (C.c_double * 3)(*[float(x) for x in v['normal']]),
                            float(v['ptin']), len(names), L.iptr(idx) if len(idx) else None, wp, float(v['Tw']),
                            float(v['a']), float(v['b']))
        L.check(L.lib().afvm_set_objective_vane(self._ctx, C.byref(d)), self._ctx, 'afvm_set_objective_vane')
        self._bcVersion = getattr(self, '_bcVersion', 0) + 1
        self.vane = dict(v, planeCells=cells, planeAreas=areas.reshape(-1, 1))

    def extraArgs(self):
        """The objective's extra step inputs, as the reference's getPlane/getWeights append them
        to solver.extraArgs (vane.py:33-37, 79-80): [nPlaneCells, cells, areas] + a weight array
        per heat patch (in the order of objectives/vane.py's ``patches``)."""
        if self.vane is None:
            return []
        v = self.vane
        from .vane import HEAT_PATCHES
        order = [p for p in HEAT_PATCHES if p in v['heat']] + [p for p in v['heat'] if p not in HEAT_PATCHES]
        return ([np.int32(len(v['planeCells'])), np.asarray(v['planeCells'], np.int32).reshape(-1, 1),
                 np.asarray(v['planeAreas'], np.float64).reshape(-1, 1)] +
                [np.asarray(v['heat'][p], np.float64).reshape(-1, 1) for p in order])

    def _apply_extra(self, extra):
        """Re-upload the vane inputs when the extra step inputs differ from the current ones."""
        if self.vane is None:
            if len(extra):
                raise ValueError('map: %d inputs past the boundary tensors, the objective takes none' % len(extra))
            return
        cur = self.extraArgs()
        if len(extra) != len(cur):
            raise ValueError('map: expected %d objective inputs, got %d' % (len(cur), len(extra)))
        if all(np.array_equal(np.asarray(a), np.asarray(b)) for a, b in zip(extra, cur)):
            return
        from .vane import HEAT_PATCHES
        order = [p for p in HEAT_PATCHES if p in self.vane['heat']] + \
            [p for p in self.vane['heat'] if p not in HEAT_PATCHES]
        v = dict(self.vane, planeCells=np.asarray(extra[1]).reshape(-1), planeAreas=np.asarray(extra[2]),
                 heat={p: np.asarray(w) for p, w in zip(order, extra[3:])})
        self._set_vane(v)

    def close(self):
        if self._ctx is not None:
            L.lib().afvm_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self):
        return int(L.lib().afvm_ctx_device_bytes(self._ctx))

    # ------------------------------------------------------------------ reference call surface
    def getBoundaryTensor(self, index=1):
        """BC input values in the reference order (Solver.getBoundaryTensor, solver.py:91-92;
        CellField.getTensor, field.py:141-146): per field U, T, p, per sorted patch, the
        fixedValue 'value' or the CBC_UPT U0, T0, p0 arrays."""
        out = []
        for f, dims in (('U', 3), ('T', 1), ('p', 1)):
            for name in self.mesh.sortedPatches:
                b = self.bc[f][name]
                if b['type'] == 'fixedValue':
                    out.append(np.asarray(b['value']).reshape(-1, dims))
                elif b['type'] == 'CBC_UPT':
                    out.extend([np.asarray(b['U0']).reshape(-1, 3), np.asarray(b['T0']).reshape(-1, 1),
                                np.asarray(b['p0']).reshape(-1, 1)])
                elif b['type'] == 'CBC_TOTAL_PT':
                    # createInput order of BCs.py:168-175: Tt, pt, then direction when given
                    out.extend([np.asarray(b['Tt']).reshape(-1, 1), np.asarray(b['pt']).reshape(-1, 1)])
                    if 'direction' in b:
                        out.append(np.asarray(b['direction']).reshape(-1, 3))
        return out

    def _apply_bc_tensors(self, vals):
        """Upload changed BC values (per-call inputs of the reference's map)."""
        pos = 0
        for fi, (f, dims) in enumerate((('U', 3), ('T', 1), ('p', 1))):
            for pi, name in enumerate(self.mesh.sortedPatches):
                b = self.bc[f][name]
                if b['type'] == 'fixedValue':
                    v = np.ascontiguousarray(vals[pos], np.float64)
                    if not np.array_equal(v, self._bcvals[pos]):
                        self._bcVersion = getattr(self, '_bcVersion', 0) + 1
                        L.check(L.lib().afvm_set_bc_value(self._ctx, pi, fi, L.dptr(v)), self._ctx)
                        self._bcvals[pos] = v.copy()
                    pos += 1
                elif b['type'] == 'CBC_UPT':
                    if f == 'p':
                        for k, (ff, d) in enumerate((('U', 3), ('T', 1), ('p', 1))):
                            v = np.ascontiguousarray(vals[pos + k], np.float64)
                            if not np.array_equal(v, self._bcvals[pos + k]):
                                self._bcVersion = getattr(self, '_bcVersion', 0) + 1
                                L.check(L.lib().afvm_set_bc_value(self._ctx, pi, k, L.dptr(v)), self._ctx)
                                self._bcvals[pos + k] = v.copy()
                    pos += 3
                elif b['type'] == 'CBC_TOTAL_PT':
                    nv = 3 if 'direction' in b else 2
                    if f == 'p':
                        for k, field in zip(range(nv), (1, 2, 0)):      # Tt -> T, pt -> p, direction -> U
                            v = np.ascontiguousarray(vals[pos + k], np.float64)
                            if not np.array_equal(v, self._bcvals[pos + k]):
                                self._bcVersion = getattr(self, '_bcVersion', 0) + 1
                                L.check(L.lib().afvm_set_bc_value(self._ctx, pi, field, L.dptr(v)), self._ctx)
                                self._bcvals[pos + k] = v.copy()
                    pos += nv
        if pos != len(vals):
            raise ValueError('expected %d boundary tensors, got %d' % (pos, len(vals)))

    def map(self, *inputs, **options):
        """The reference's primal step function (RCF.compileSolver, density.py:80-105):
        inputs [rho, rhoU, rhoE, dt] + mesh.getTensor() + mesh.getScalar() + sources +
        BC tensors; returns [rhoN, rhoUN, rhoEN, dtc, obj] (numpy)."""
        m = self.mesh
        nT, nS = len(Mesh.gradFields) + len(Mesh.intFields), len(m.getScalar())
        base = 4 + nT + nS
        if len(inputs) < base + 3:
            raise ValueError('map: expected at least %d inputs, got %d' % (base + 3, len(inputs)))
        rho, rhoU, rhoE, dt = inputs[:4]
        scal = list(inputs[4 + nT:base])
        if scal[:len(Mesh.constants)] != [getattr(m, a) for a in Mesh.constants]:
            raise ValueError('map: mesh constants differ from the mesh this solver was built on')
        S = inputs[base:base + 3]
        nBC = len(self._bcvals)
        self._apply_bc_tensors(list(inputs[base + 3:base + 3 + nBC]))
        self._apply_extra(list(inputs[base + 3 + nBC:]))
        n = m.nInternalCells
        dt = float(np.asarray(dt).reshape(-1)[0])
        ins = self._host_fields((rho, rhoU, rhoE))
        Ss = self._host_fields(S)
        if all(s is not None and not s.any() for s in Ss):
            Ss = [None, None, None]
        if self.keep_stages:
            return self._map_keeping_stages((rho, rhoU, rhoE), ins, Ss, dt)
        ins = [np.ascontiguousarray(a, self.dtype) for a in ins]
        Ss = [None if a is None else np.ascontiguousarray(a, self.dtype) for a in Ss]
        outs = [np.empty((n, d), self.dtype) for d in (1, 3, 1)]
        dtc = C.c_double()
        obj = C.c_double()
        vp = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
        st = L.lib().afvm_primal_step_host(self._ctx, vp(ins[0]), vp(ins[1]), vp(ins[2]), dt,
                                           vp(Ss[0]), vp(Ss[1]), vp(Ss[2]), vp(outs[0]), vp(outs[1]), vp(outs[2]),
                                           C.byref(dtc), C.byref(obj), None)
        L.check(st, self._ctx, 'afvm_primal_step_host')
        return outs + [np.array([[dtc.value]]), np.array([[self._objective_after(obj.value)]])]

    # ---- the stages of recent map calls, for Adjoint.map on the same states -------------
    # The reference's adjoint loop re-runs the primal over a checkpoint interval through map
    # and then calls the adjoint map on exactly those states (apps/adjoint.py:227, 255-291).
    # map keeps each call's RK stage states on the device, keyed by its input arrays (their
    # identity, dt and a sample of their values), for the last keep_stages calls; Adjoint.map
    # then skips the forward recompute. keep_stages = 0 turns this off.
    keep_stages = 32

    def _host_fields(self, arrays):
        """(rho, rhoU, rhoE)-shaped host arrays as (n,1), (n,3), (n,1) views, float64 or float32
        as given (other types become float64); None stays None."""
        n = self.mesh.nInternalCells
        out = []
        for a, d in zip(arrays, (1, 3, 1)):
            if a is None:
                out.append(None)
                continue
            a = np.asarray(a)
            if a.dtype not in (np.float64, np.float32):
                a = a.astype(np.float64)
            out.append(np.ascontiguousarray(a.reshape(n, d)))
        return out

    def upload(self, arrays):
        """Device tensors of the state type from (rho, rhoU, rhoE)-shaped host arrays of any
        float type in any host memory, through the library's pipelined host copy."""
        torch = _torch()
        td = torch.float64 if self.dtype == np.float64 else torch.float32
        dev = 'cuda:%d' % self.device
        return [L.to_device(a, torch.empty(a.shape, dtype=td, device=dev)) for a in self._host_fields(arrays)]

    def download(self, tensors, dtype=np.float64):
        """Host arrays of `dtype` holding the device tensors (pipelined host copy). An array this
        context returned before is written again only when nothing else refers to it any more
        (its reference count shows only this context's pool): a caller that keeps a result, or
        a view of it, keeps its values. The reused arrays' pages are already mapped, so the copy
        runs at the link's rate instead of the first-touch page-fault rate of a new array."""
        return [L.to_host(t, self._host_array(tuple(t.shape), dtype)) for t in tensors]

    def _host_array(self, shape, dtype):
        pool = self.__dict__.setdefault('_hostPool', [])
        dtype = np.dtype(dtype)
        for i in range(len(pool)):
            # 2: the pool's own reference and getrefcount's argument
            if pool[i].shape == shape and pool[i].dtype == dtype and sys.getrefcount(pool[i]) == 2:
                return pool[i]
        a = np.empty(shape, dtype)
        if len(pool) < 12:
            pool.append(a)
        return a

    def _fingerprint(self, arrays, dt):
        parts = [repr(float(dt)).encode(), str(getattr(self, '_bcVersion', 0)).encode()]
        for a in arrays:
            if a is None:
                parts.append(b'-')
                continue
            v = np.asarray(a).reshape(-1)
            idx = np.linspace(0, len(v) - 1, num=min(len(v), 97)).astype(np.int64)
            parts.append(np.ascontiguousarray(v[idx]).tobytes())
            parts.append(str(v.shape).encode())
        return b'|'.join(parts)

    def _map_keeping_stages(self, originals, ins, Ss, dt):
        torch = _torch()
        dev = 'cuda:%d' % self.device
        if not hasattr(self, '_stageCache'):
            self._stageCache = collections.OrderedDict()
        key = tuple(id(a) for a in originals)
        fp = self._fingerprint(list(ins) + list(Ss), dt)
        if key in self._stageCache:
            buf = self._stageCache.pop(key)[1]
        elif len(self._stageCache) >= self.keep_stages:
            buf = self._stageCache.popitem(last=False)[1][1]
        else:
            buf = self.stage_buffer()
        x = self.upload(ins)
        Sd = None if Ss[0] is None else self.upload(Ss)
        r = self.step(x[0], x[1], x[2], dt, S=Sd, out=x, stages=buf)
        self._stageCache[key] = (fp, buf)
        outs = self.download(r[:3], self.dtype)
        return outs + [np.array([[r[3]]]), np.array([[r[4]]])]

    def kept_stages(self, rho, rhoU, rhoE, dt, S=None):
        """The stage buffer a map call on these host arrays kept, or None."""
        cache = getattr(self, '_stageCache', None)
        if not cache:
            return None
        hit = cache.get((id(rho), id(rhoU), id(rhoE)))
        if hit is None:
            return None
        ins = self._host_fields((rho, rhoU, rhoE))
        Ss = [None, None, None] if S is None else self._host_fields(S)
        if all(s is not None and not s.any() for s in Ss):
            Ss = [None, None, None]
        return hit[1] if hit[0] == self._fingerprint(list(ins) + list(Ss), dt) else None

    def mapInputs(self, rho, rhoU, rhoE, dt, sources=None):
        """The positional input list the reference's time loop builds (solver.py:312-317)."""
        m = self.mesh
        n = m.nInternalCells
        if sources is None:
            sources = [np.zeros((n, 1)), np.zeros((n, 3)), np.zeros((n, 1))]
        return ([rho, rhoU, rhoE, np.array([[dt]])] + m.getTensor() + m.getScalar() + list(sources) +
                self.getBoundaryTensor(1) + self.extraArgs())

    def step_host(self, rho, rhoU, rhoE, dt, S=None, out=None):
        """One step through the host-buffer entry point (afvm_primal_step_host): host arrays in
        (pinned or pageable), host arrays out, copies inside. Returns (rhoN, rhoUN, rhoEN, dtc, obj)."""
        n = self.mesh.nInternalCells
        ins = [np.ascontiguousarray(a, self.dtype) for a in (rho, rhoU, rhoE)]
        if out is None:
            out = [np.empty((n, d), self.dtype) for d in (1, 3, 1)]
        Ss = [None, None, None] if S is None else [np.ascontiguousarray(a, self.dtype) for a in S]
        vp = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
        dtc = C.c_double()
        obj = C.c_double()
        st = L.lib().afvm_primal_step_host(self._ctx, vp(ins[0]), vp(ins[1]), vp(ins[2]), float(dt),
                                           vp(Ss[0]), vp(Ss[1]), vp(Ss[2]), vp(out[0]), vp(out[1]), vp(out[2]),
                                           C.byref(dtc), C.byref(obj), None)
        L.check(st, self._ctx, 'afvm_primal_step_host')
        return out[0], out[1], out[2], dtc.value, self._objective_after(obj.value)

    # ------------------------------------------------------------------ per-kernel timing
    def profile(self, on=True):
        L.check(L.lib().afvm_profile(self._ctx, 1 if on else 0), self._ctx)

    def profile_read(self):
        """{kernel name: (milliseconds, launches)} since profile(True)."""
        names = L.kernel_names()
        ms = (C.c_double * len(names))()
        cnt = (C.c_int64 * len(names))()
        L.check(L.lib().afvm_profile_read(self._ctx, len(names), ms, cnt), self._ctx)
        return {n: (ms[i], cnt[i]) for i, n in enumerate(names) if cnt[i]}

    # ------------------------------------------------------------------ device path
    def stage_buffer(self):
        """A device buffer for the two RK stage states of one step (afvm_primal_step_stages)."""
        torch = _torch()
        td = torch.float64 if self.dtype == np.float64 else torch.float32
        return torch.empty(10 * self.mesh.nInternalCells, dtype=td, device='cuda:%d' % self.device)

    @property
    def tape_bytes(self):
        """Bytes of one step's face tape (afvm_tape_elements values of the record type)."""
        return int(L.lib().afvm_tape_elements(self._ctx)) * np.dtype(self.record_dtype).itemsize

    def tape_buffer(self):
        """A device buffer for the face tape of one step (afvm_primal_step_tape): the forward
        values the adjoint step would otherwise re-evaluate; kept together with a stage_buffer."""
        torch = _torch()
        td = torch.float64 if self.record_dtype == np.float64 else torch.float32
        return torch.empty(int(L.lib().afvm_tape_elements(self._ctx)), dtype=td, device='cuda:%d' % self.device)

    def _check_tape(self, tape, stages):
        torch = _torch()
        td = torch.float64 if self.record_dtype == np.float64 else torch.float32
        if stages is None:
            raise ValueError('tape: kept together with stages')
        if tape.dtype != td or tape.numel() < int(L.lib().afvm_tape_elements(self._ctx)) or \
                not tape.is_contiguous() or not tape.is_cuda:
            raise ValueError('tape: a contiguous device buffer of afvm_tape_elements %s values' % td)
        return tape

    def step(self, rho, rhoU, rhoE, dt, S=None, out=None, want_scalars=True, stages=None, tape=None):
        """One step on CUDA tensors (reference layouts). Returns (rhoN, rhoUN, rhoEN, dtc, obj).
        stages: optional stage_buffer() that receives the step's RK stage states, for
        adjoint_step(..., stages=) on the same state; tape: optional tape_buffer() (with stages)
        that receives the step's face tape, for adjoint_step(..., tape=)."""
        torch = _torch()
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        if out is None:
            out = (torch.empty_like(rho), torch.empty_like(rhoU), torch.empty_like(rhoE))
        Sp = [None, None, None] if S is None else [C.c_void_p(s.data_ptr()) for s in S]
        dtc = C.c_double()
        obj = C.c_double()
        sp = None if stages is None else C.c_void_p(self._check_stages(stages).data_ptr())
        tp = None if tape is None else C.c_void_p(self._check_tape(tape, stages).data_ptr())
        st = L.lib().afvm_primal_step_tape(self._ctx, C.c_void_p(rho.data_ptr()), C.c_void_p(rhoU.data_ptr()),
                                           C.c_void_p(rhoE.data_ptr()), float(dt), Sp[0], Sp[1], Sp[2],
                                           C.c_void_p(out[0].data_ptr()), C.c_void_p(out[1].data_ptr()),
                                           C.c_void_p(out[2].data_ptr()), sp, tp,
                                           C.byref(dtc) if want_scalars else None,
                                           C.byref(obj) if want_scalars else None, C.c_void_p(stream))
        L.check(st, self._ctx, 'afvm_primal_step_tape')
        return out[0], out[1], out[2], dtc.value, self._objective_after(obj.value) if want_scalars else obj.value

    def _check_stages(self, stages):
        torch = _torch()
        td = torch.float64 if self.dtype == np.float64 else torch.float32
        if stages.dtype != td or stages.numel() < 10 * self.mesh.nInternalCells or not stages.is_contiguous() \
                or not stages.is_cuda:
            raise ValueError('stages: a contiguous device buffer of 10 x nInternalCells %s values' % td)
        return stages

    # the mesh tensors the reference differentiates for parameters = 'mesh' (Mesh.gradFields,
    # adFVM/mesh.py:28-31), in the order of its map's outputs
    MESH_GRAD_FIELDS = ('areas', 'volumesL', 'volumesR', 'weights', 'deltas', 'normals', 'deltasUnit',
                        'linearWeights', 'quadraticWeights', 'volumes')

    def param_shapes(self, parameters):
        """Shapes of the gradients that adjoint_step(params=parameters) returns: for 'mesh' those
        of the ten Mesh.gradFields tensors; for ('BCs', field, patch, key) that of the one
        boundary input (apps/adjoint.py:104-121)."""
        m = self.mesh
        if parameters == 'mesh':
            return [tuple(np.shape(getattr(m, k))) for k in self.MESH_GRAD_FIELDS]
        field = self._bc_param(parameters)[1]
        return [(int(m.boundary[parameters[2]]['nFaces']), 3 if field == 0 else 1)]

    def _bc_param(self, parameters):
        """('BCs', field, patch, key) -> (sorted patch index, ghost field 0/1/2, active). The
        input sets the ghost values of the patch: fixedValue 'value' its own field; CBC_UPT U0,
        T0, p0 and CBC_TOTAL_PT direction, Tt, pt (read from the p field's BC, as the reference's
        characteristic boundary does, density.py:333-337) U, T, p. The copies held by the U and
        T fields of a characteristic patch are inputs the step never reads (active False)."""
        if not (isinstance(parameters, tuple) and len(parameters) == 4 and parameters[0] == 'BCs'):
            raise ValueError('parameters: source, mesh or (BCs, field, patch, key)')
        _, phi, patch, key = parameters
        if phi not in ('U', 'T', 'p') or patch not in self.mesh.sortedPatches:
            raise ValueError('parameters: unknown field or patch %r' % (parameters,))
        kind = self.bc[phi][patch]['type']
        keys = {'fixedValue': {'value': 'UTp'.index(phi)}, 'CBC_UPT': {'U0': 0, 'T0': 1, 'p0': 2},
                'CBC_TOTAL_PT': {'direction': 0, 'Tt': 1, 'pt': 2}}.get(kind, {})
        if key not in keys:
            raise ValueError('parameters: %s on patch %s (%s) has no input %r' % (phi, patch, kind, key))
        if kind == 'CBC_TOTAL_PT' and key == 'direction' and 'direction' not in self.bc['p'][patch]:
            raise ValueError('parameters: that CBC_TOTAL_PT direction is the face normals (a mesh input)')
        active = kind == 'fixedValue' or phi == 'p'
        return self.mesh.sortedPatches.index(patch), keys[key], active

    # ------------------------------------------------------------------ objectives as torch functions
    def meshTensor(self, name):
        """A mesh array as a CUDA tensor: float64, or int64 for the connectivity (cached)."""
        torch = _torch()
        cache = self.__dict__.setdefault('_meshT', {})
        if name not in cache:
            a = np.ascontiguousarray(getattr(self.mesh, name))
            dt = torch.int64 if a.dtype.kind in 'iu' else torch.float64
            cache[name] = torch.as_tensor(a, device='cuda:%d' % self.device).to(dt)
        return cache[name]

    @property
    def gauge(self):
        """(p, T, H) of the gauge state of the FP32 records (afvm_get_gauge)."""
        out = np.zeros(3)
        L.check(L.lib().afvm_get_gauge(self._ctx, out.ctypes.data_as(C.POINTER(C.c_double))), self._ctx)
        return tuple(float(v) for v in out)

    def _call_objective(self, prims, view=None):
        P = prims.double()
        return self.objectiveFn([P[:, 0:3], P[:, 3:4], P[:, 4:5]], view or ObjectiveSolver(self))

    def _objective_after(self, kernel_obj):
        """The step's objective: the built-in one from the kernels, or the caller's function on
        the primitives the step copied into the sink."""
        if self.objectiveFn is None:
            return kernel_obj
        torch = _torch()
        with torch.no_grad():
            return float(self._call_objective(self._objPrims))

    def _objective_prims(self, rho, rhoU, rhoE, dt, S, tape):
        """The objective-stage primitives (nCells x 5) of the step from this state: from its
        tape's second-stage cell records, or by running the step again into the sink."""
        torch = _torch()
        m = self.mesh
        if tape is not None:
            off = int(L.lib().afvm_tape_elements(self._ctx)) - 3 * 20 * m.nCells + 20 * m.nCells
            prims = tape[off:off + 20 * m.nCells].view(m.nCells, 20)[:, :5]
            if self.record_dtype == np.float64:
                return prims
            # FP32 records hold T and p as offsets from the gauge state
            g = self.gauge
            return prims.double() + torch.tensor([0.0, 0.0, 0.0, g[1], g[0]], dtype=torch.float64,
                                                 device=prims.device)
        tmp = (torch.empty_like(rho), torch.empty_like(rhoU), torch.empty_like(rhoE))
        self.step(rho, rhoU, rhoE, dt, S=S, out=tmp, want_scalars=False)
        return self._objPrims.clone()

    def adjoint_step(self, rho, rhoU, rhoE, dt, seeds, obja=1.0, S=None, out=None, source_grad=True, stages=None,
                     tape=None, params=None, source_out=None):
        """VJP of one step on CUDA tensors (see _adjoint_step); with an objective given as a
        torch function, its gradient with respect to the objective-stage primitives - torch
        autograd of the function - is the adjoint seed the kernels add (afvm_set_objective_seed),
        and for params='mesh' the function's own dependence on the mesh tensors (through
        solver.meshTensor) is added to the mesh gradients."""
        if self.objectiveFn is None or obja == 0.0:
            return self._adjoint_step(rho, rhoU, rhoE, dt, seeds, obja, S, out, source_grad, stages, tape, params,
                                      source_out)
        torch = _torch()
        prims = self._objective_prims(rho, rhoU, rhoE, dt, S, tape).double().detach().requires_grad_(True)
        leaves = {}
        if params == 'mesh':
            leaves = {k: self.meshTensor(k).detach().clone().requires_grad_(True) for k in self.MESH_GRAD_FIELDS}
        with torch.enable_grad():
            J = self._call_objective(prims, ObjectiveSolver(self, leaves))
            ins = [prims] + list(leaves.values())
            g = torch.autograd.grad(J, ins, allow_unused=True)
        g = [torch.zeros_like(v) if gi is None else gi for gi, v in zip(g, ins)]
        seed = g[0].contiguous()
        L.check(L.lib().afvm_set_objective_seed(self._ctx, C.c_void_p(seed.data_ptr())), self._ctx)
        try:
            r = self._adjoint_step(rho, rhoU, rhoE, dt, seeds, obja, S, out, source_grad, stages, tape, params,
                                   source_out)
        finally:
            L.lib().afvm_set_objective_seed(self._ctx, None)
        if params == 'mesh':
            for dst, gm in zip(r[4], g[1:]):
                dst += float(obja) * gm.reshape(dst.shape)
        return r

    def _adjoint_step(self, rho, rhoU, rhoE, dt, seeds, obja=1.0, S=None, out=None, source_grad=True, stages=None,
                      tape=None, params=None, source_out=None):
        """VJP of one step on CUDA tensors (afvm_adjoint_step): the adjoint of the input state
        (and of the sources) given the adjoint seeds of the output state and of the objective.
        dt is held fixed, the CFL-sum output gets no seed (dtca = 0, apps/adjoint.py:268).
        stages: the stage_buffer() a step(..., stages=) of this state filled; skips the
        forward recompute. tape: the tape_buffer() the same step filled; skips the face
        flux's re-evaluation inside the VJP. params: 'mesh' or ('BCs', field, patch, key) -
        also the gradients with respect to those parameters (afvm_adjoint_step_params, FP64
        contexts), returned as a fifth item: a list of float64 CUDA tensors of param_shapes()."""
        torch = _torch()
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        if out is None:
            out = (torch.empty_like(rho), torch.empty_like(rhoU), torch.empty_like(rhoE))
        Sg = None
        if source_grad:
            Sg = tuple(source_out) if source_out is not None else \
                (torch.empty_like(rho), torch.empty_like(rhoU), torch.empty_like(rhoE))
        Sp = [None, None, None] if S is None else [C.c_void_p(s.data_ptr()) for s in S]
        vp = lambda t: C.c_void_p(t.data_ptr())
        gp = [None, None, None] if Sg is None else [vp(t) for t in Sg]
        sp = None if stages is None else vp(self._check_stages(stages))
        tp = None if tape is None else vp(self._check_tape(tape, stages))
        if params is None:
            st = L.lib().afvm_adjoint_step_tape(self._ctx, vp(rho), vp(rhoU), vp(rhoE), float(dt), Sp[0], Sp[1],
                                                Sp[2], sp, tp, vp(seeds[0]), vp(seeds[1]), vp(seeds[2]), 0.0,
                                                float(obja), vp(out[0]), vp(out[1]), vp(out[2]), gp[0], gp[1], gp[2],
                                                C.c_void_p(stream))
            L.check(st, self._ctx, 'afvm_adjoint_step_tape')
            return out[0], out[1], out[2], Sg
        grads = [torch.empty(sh, dtype=torch.float64, device=rho.device) for sh in self.param_shapes(params)]
        dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), L._d)
        pg = L.ParamGrad()
        pg.bcPatch = -1
        active = True
        if params == 'mesh':
            for k, t in zip(self.MESH_GRAD_FIELDS, grads):
                if t.numel():
                    setattr(pg, k, dp(t))
        else:
            pi, field, active = self._bc_param(params)
            pg.bcPatch, pg.bcField, pg.bc = pi, field, dp(grads[0])
        if not active:
            # an input the step never reads: its gradient is zero
            r = self._adjoint_step(rho, rhoU, rhoE, dt, seeds, obja, S, out, source_grad, stages, tape)
            grads[0].zero_()
            return r + (grads,)
        st = L.lib().afvm_adjoint_step_params(self._ctx, vp(rho), vp(rhoU), vp(rhoE), float(dt), Sp[0], Sp[1], Sp[2],
                                              sp, tp, vp(seeds[0]), vp(seeds[1]), vp(seeds[2]), 0.0, float(obja),
                                              vp(out[0]), vp(out[1]), vp(out[2]), gp[0], gp[1], gp[2], C.byref(pg),
                                              C.c_void_p(stream))
        L.check(st, self._ctx, 'afvm_adjoint_step_params')
        return out[0], out[1], out[2], Sg, grads

    def adjoint_viscosity(self, rho, rhoU, rhoE, adj, dt, kind='turkel', scaling=1e-3, want_fields=False):
        """Artificial-viscosity stabilisation of the adjoint fields ``adj`` (three CUDA tensors,
        smoothed in place) for the primal state (rho, rhoU, rhoE) and time step dt
        (afvm_adjoint_viscosity; postpro.computeAdjointViscosity + viscositySolver). kind:
        'turkel', 'abarbanel' or 'uniform'. Returns the CG iterations, and with want_fields
        also the viscosity (nCells) and its face values (nFaces) as FP64 CUDA tensors."""
        torch = _torch()
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        vp = lambda t: C.c_void_p(t.data_ptr())
        Mt = DTt = None
        if want_fields:
            Mt = torch.empty(self.mesh.nCells, dtype=torch.float64, device=rho.device)
            DTt = torch.empty(self.mesh.nFaces, dtype=torch.float64, device=rho.device)
        it = C.c_int32()
        st = L.lib().afvm_adjoint_viscosity(self._ctx, vp(rho), vp(rhoU), vp(rhoE), L.AFVM_VISC[kind], float(scaling),
                                            float(dt), vp(adj[0]), vp(adj[1]), vp(adj[2]),
                                            None if Mt is None else C.cast(vp(Mt), L._d),
                                            None if DTt is None else C.cast(vp(DTt), L._d), C.byref(it),
                                            C.c_void_p(stream))
        L.check(st, self._ctx, 'afvm_adjoint_viscosity')
        if want_fields:
            return it.value, Mt, DTt
        return it.value

    def sensitivity(self, grads, perts):
        """sum_k <grads[k], perts[k]> in FP64 on the device (cmesh.computeSensitivity,
        cmesh.cpp:309-340); CUDA float64 tensors."""
        torch = _torch()
        k = len(grads)
        gs = [g.contiguous() for g in grads]
        ps = [p.contiguous() for p in perts]
        for g, p in zip(gs, ps):
            if g.dtype != torch.float64 or p.dtype != torch.float64 or g.numel() != p.numel():
                raise ValueError('sensitivity: float64 arrays of equal size required')
        ga = (L._d * k)(*[C.cast(C.c_void_p(g.data_ptr()), L._d) for g in gs])
        pa = (L._d * k)(*[C.cast(C.c_void_p(p.data_ptr()), L._d) for p in ps])
        na = (C.c_int64 * k)(*[g.numel() for g in gs])
        out = C.c_double()
        stream = torch.cuda.current_stream(gs[0].device).cuda_stream
        L.check(L.lib().afvm_sensitivity(self._ctx, k, ga, pa, na, C.byref(out), C.c_void_p(stream)), self._ctx)
        return out.value

    def adjoint_energy(self, adj, state):
        """sum_c w^T A(u) w V on the device (cmesh.computeEnergy, cmesh.cpp:342-425); adj and
        state are (rho, rhoU, rhoE) CUDA tensors. The reference's driver reports sqrt of it."""
        torch = _torch()
        vp = lambda t: C.c_void_p(t.data_ptr())
        out = C.c_double()
        stream = torch.cuda.current_stream(state[0].device).cuda_stream
        L.check(L.lib().afvm_adjoint_energy(self._ctx, vp(adj[0]), vp(adj[1]), vp(adj[2]), vp(state[0]),
                                            vp(state[1]), vp(state[2]), C.byref(out), C.c_void_p(stream)), self._ctx)
        return out.value

    def run_device(self, rho, rhoU, rhoE, nSteps, dt, S=None, record=True):
        """nSteps steps in place on CUDA tensors, dt control on the device
        (dt <- min(2*CFL/dtc, stepFactor*dt) unless fixedTimeStep). Returns device histories
        (dt, dtc, obj) or None."""
        torch = _torch()
        if self.objectiveFn is not None:
            raise NotImplementedError('run_device with an objective given as a function: use run() or step()')
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        hist = torch.zeros((3, max(1, nSteps)), dtype=torch.float64, device=rho.device) if record else None
        hp = [None, None, None] if hist is None else [C.cast(C.c_void_p(hist[k].data_ptr()), L._d) for k in range(3)]
        Sp = [None, None, None] if S is None else [C.c_void_p(s.data_ptr()) for s in S]
        st = L.lib().afvm_primal_run(self._ctx, C.c_void_p(rho.data_ptr()), C.c_void_p(rhoU.data_ptr()),
                                     C.c_void_p(rhoE.data_ptr()), int(nSteps), float(dt), float(self.CFL),
                                     float(self.stepFactor), 1 if self.fixedTimeStep else 0, Sp[0], Sp[1], Sp[2],
                                     hp[0], hp[1], hp[2], C.c_void_p(stream))
        L.check(st, self._ctx, 'afvm_primal_run')
        return hist

    # ------------------------------------------------------------------ case files
    @classmethod
    def fromCase(cls, caseDir, time=0.0, objective='none', precision='fp64', device=0, **config):
        """The solver on an OpenFOAM case directory: the reference's ``RCF(caseDir)`` (mesh from
        constant/polyMesh, Solver.__init__ solver.py:44-49) with the U, T, p boundary conditions
        of time ``time``."""
        meshData = foam.read_mesh(caseDir, time)
        mesh = Mesh.create(meshData)
        td = os.path.join(caseDir, foam.time_name(time))
        bc = {name: foam.read_field(td, name, mesh.boundary, mesh.nInternalCells)[1] for name in ('U', 'T', 'p')}
        rcf = cls(mesh, bc, objective=objective, precision=precision, device=device, **config)
        rcf.case = caseDir
        return rcf

    @property
    def statusFile(self):
        return os.path.join(self.case, 'status.pkl')

    def readStatusFile(self):
        """[timeIndex, t, dt, result] (Solver.readStatusFile, solver.py:185-192); None if absent."""
        return foam.read_status(self.statusFile)

    def writeStatusFile(self, data):
        foam.write_status(self.statusFile, data)

    def removeStatusFile(self):
        try:
            os.remove(self.statusFile)
        except OSError:
            pass

    def readFields(self, t, suffix=''):
        """U, T, p of time t -> conservative (rho, rhoU, rhoE) host arrays (RCF.readFields,
        density.py:113-137). The boundary values found there replace the current ones."""
        m = self.mesh
        td = os.path.join(self.case, foam.time_name(t))
        prim = {}
        for name in ('U', 'T', 'p'):
            prim[name], b = foam.read_field(td, name + suffix, m.boundary, m.nInternalCells)
            for patch, entry in b.items():
                cur = self.bc[name].get(patch)
                if cur is None or cur.get('type') != entry.get('type'):
                    raise ValueError('%s: boundary type of patch %s changed between times' % (name, patch))
                for k, v in entry.items():
                    if isinstance(v, np.ndarray):
                        cur[k] = v
        self._apply_bc_tensors(self.getBoundaryTensor(1))
        return self.conservative(prim['U'], prim['T'], prim['p'])

    def boundary_values(self, rho, rhoU, rhoE):
        """Ghost-cell U, T, p (nGhostCells x 5 CUDA tensor of the record type: FP64 for 'fp64',
        FP32 otherwise) of a device state: the boundary map (afvm_boundary_values)."""
        torch = _torch()
        rd = torch.float64 if self.record_dtype == np.float64 else torch.float32
        out = torch.empty((self.mesh.nGhostCells, 5), dtype=rd, device=rho.device)
        stream = torch.cuda.current_stream(rho.device).cuda_stream
        st = L.lib().afvm_boundary_values(self._ctx, C.c_void_p(rho.data_ptr()), C.c_void_p(rhoU.data_ptr()),
                                          C.c_void_p(rhoE.data_ptr()), C.c_void_p(out.data_ptr()),
                                          C.c_void_p(stream))
        L.check(st, self._ctx, 'afvm_boundary_values')
        return out

    def primitive(self, rho, rhoU, rhoE):
        """RCF.primitive (density.py:161-170) on host arrays."""
        U = rhoU / rho
        E = rhoE / rho
        e = E - 0.5 * np.sum(U * U, axis=1, keepdims=True)
        p = (self.gamma - 1) * rho * e
        T = e * (1. / self.Cv)
        return U, T, p

    def writeFields(self, fields, t):
        """Write rho, rhoU, rhoE, U, T, p of time t (RCF.writeFields, density.py:146-158): internal
        values, and on every patch of a value type (BCs.py:18-23) the ghost-cell values of the
        boundary map; the conservative fields carry the mesh's default boundary types
        (IOField without a boundary, field.py:161-168), which hold no values."""
        torch = _torch()
        m = self.mesh
        n = m.nInternalCells
        dev = 'cuda:%d' % self.device
        x = [np.asarray(a, np.float64).reshape(n, d) for a, d in zip(fields[:3], (1, 3, 1))]
        xd = [torch.as_tensor(np.ascontiguousarray(a, self.dtype), device=dev) for a in x]
        ghost = self.boundary_values(*xd).cpu().numpy().astype(np.float64, copy=False)
        gU, gT, gp = ghost[:, 0:3], ghost[:, 3:4], ghost[:, 4:5]
        U, T, p = self.primitive(*x)
        td = os.path.join(self.case, foam.time_name(t))
        nIF = m.nInternalFaces

        def boundary(base, ghost_values):
            out = {}
            for patch, entry in base.items():
                e = dict(entry)
                if e.get('type') in foam.VALUE_PATCHES:
                    s = int(m.boundary[patch]['startFace']) - nIF
                    e['value'] = ghost_values[s:s + int(m.boundary[patch]['nFaces'])]
                out[patch] = e
            return out
        for name, internal in (('rho', x[0]), ('rhoU', x[1]), ('rhoE', x[2])):
            foam.write_field(td, name, internal, {k: dict(v) for k, v in m.defaultBoundary.items()})
        for name, internal, g in (('U', U, gU), ('T', T, gT), ('p', p, gp)):
            foam.write_field(td, name, internal, boundary(self.bc[name], g))

    # ------------------------------------------------------------------ time loop
    def run(self, fields, nSteps, dt, endTime=np.inf, startTime=0.0, mode='simulation', source=None, avgStart=0,
            writeInterval=None, startIndex=0, result=0.0):
        """Solver.run (adFVM/solver.py:210-411). fields: conservative (rho, rhoU, rhoE) numpy
        arrays. mode 'forward' returns every step's fields (and the record); otherwise returns
        the time-summed objective (and the record). On a case directory (``fromCase``) the
        fields and status.pkl are written every writeInterval steps and after the last one in
        'simulation'/'orig' modes, and 'orig'/'perturb' append the objective series to
        timeSeries.txt (solver.py:381-396)."""
        t = startTime
        timeIndex = startIndex
        sols = [list(fields)]
        record = []
        series = []
        case = getattr(self, 'case', None)
        every = writeInterval or np.inf
        sources = None if source is None else [np.asarray(s) for s in source]
        while t < endTime and timeIndex < nSteps:
            inputs = self.mapInputs(*fields, dt, sources)
            outputs = self.map(*inputs)
            fields = outputs[:3]
            dtc, objective = float(outputs[3][0, 0]), float(outputs[4][0, 0])
            record.append((dt, dtc, objective))
            series.append(objective)
            timeIndex += 1
            t = round(t + dt, 12)
            if not self.fixedTimeStep:
                dt = min(2 * self.CFL / dtc, dt * self.stepFactor, endTime - t)
            if timeIndex > avgStart:
                result += objective
            if mode == 'forward':
                sols.append(list(fields))
            elif case is not None and (timeIndex % every == 0 or not (t < endTime and timeIndex < nSteps)):
                if mode in ('orig', 'simulation'):
                    self.writeFields(fields, t)
                if mode in ('orig', 'perturb'):
                    with open(os.path.join(case, 'timeSeries.txt'), 'ab') as f:
                        np.savetxt(f, np.array(series))
                series = []
                self.writeStatusFile([timeIndex, t, dt, result])
        if mode == 'forward':
            return sols, record
        return result, record

    def conservative(self, U, T, p):
        """RCF.conservative (density.py:173-181) on host arrays, for initial conditions."""
        e = self.Cv * T
        rho = p / (e * (self.gamma - 1))
        rhoE = rho * (e + 0.5 * np.sum(U * U, axis=1, keepdims=True))
        rhoU = U * rho
        return rho, rhoU, rhoE
