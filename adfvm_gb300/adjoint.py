"""Adjoint driver: the reference's ``Adjoint`` (apps/adjoint.py:31-404) on the GPU.

* ``Adjoint.map(*inputs)`` is the per-step adjoint function the reference builds with
  ``primal.map.grad()`` (apps/adjoint.py:94-151): inputs are the primal step's inputs followed
  by the adjoint seeds ``[rhoNa, rhoUNa, rhoENa, dtca, obja]`` and ``[scaling]``; outputs are
  ``[rhoa, rhoUa, rhoEa]`` and the gradients of the parameters: the three source terms
  (``parameters = 'source'``), the ten Mesh.gradFields tensors (``'mesh'``), or one boundary
  input (``('BCs', field, patch, key)``), apps/adjoint.py:104-121.
* ``Adjoint.run(...)`` is the checkpointed backward sweep (apps/adjoint.py:176-404): the
  primal is re-run forward one checkpoint interval at a time (keeping every state of the
  interval on the device), then the adjoint steps run backwards through it with seeds
  dtca = 0, obja = 1; after every step the sensitivity to each perturbation is the FP64 dot
  product of the parameter gradients with it (cmesh.computeSensitivity), summed over steps past
  ``avgStart`` and divided by ``nSteps - avgStart`` as writeResult does (apps/problem.py:47-49).
  Adjoint fields are the plain gradients of the state (the reference keeps them multiplied
  by the cell volume, apps/adjoint.py:188; divide by the volumes to compare with its files).
"""
import numpy as np

from .mesh import Mesh


def _torch():
    import torch
    return torch


class Adjoint(object):
    def __init__(self, primal, parameters='source', adjParams=None, viscousInterval=1):
        """adjParams = [scaling, viscosityType, scaler] as in a case file (templates/vane.py:68):
        with a viscosityType ('turkel', 'abarbanel', 'uniform') every viscousInterval-th step of
        the sweep is followed by the artificial-viscosity smoothing (apps/adjoint.py:127-139,
        250, 288-289)."""
        self.parameters = parameters
        if parameters == 'source':
            self.nParams = 3
        elif parameters == 'mesh':
            self.nParams = len(primal.MESH_GRAD_FIELDS)
        else:
            primal._bc_param(parameters)          # raises for anything else
            self.nParams = 1
        self.primal = primal
        self.scaling = adjParams[0] if adjParams else None
        self.viscosityType = adjParams[1] if adjParams else None
        self.viscousInterval = viscousInterval
        self.mesh = primal.mesh
        self.names = [n + 'a' for n in primal.names]
        self._fwd = None   # map's forward buffers: None (not sized yet), False (do not fit)

    def _step(self, y, dt, a, S, out=None, stages=None, tape=None, obja=1.0):
        """One adjoint step; returns (state adjoints, parameter gradients as device tensors)."""
        p = self.primal
        if self.parameters == 'source':
            r = p.adjoint_step(y[0], y[1], y[2], dt, a, obja=obja, S=S, out=out, stages=stages, tape=tape)
            return r[:3], list(r[3])
        r = p.adjoint_step(y[0], y[1], y[2], dt, a, obja=obja, S=S, out=out, source_grad=False, stages=stages,
                           tape=tape, params=self.parameters)
        return r[:3], r[4]

    # ------------------------------------------------------------ per-step map
    def map(self, *inputs, **options):
        """The reference's adjoint step function (apps/adjoint.py:124-126, called at 291)."""
        p = self.primal
        m = self.mesh
        nT, nS = len(Mesh.gradFields) + len(Mesh.intFields), len(m.getScalar())
        base = 4 + nT + nS
        nBC = len(p.getBoundaryTensor(1)) + len(p.extraArgs())
        primal_in = inputs[:base + 3 + nBC]
        rest = inputs[base + 3 + nBC:]
        if len(rest) != 6:
            raise ValueError('adjoint map: expected 3 adjoint fields, dtca, obja and scaling after the primal inputs')
        nB = len(p.getBoundaryTensor(1))
        p._apply_bc_tensors(list(primal_in[base + 3:base + 3 + nB]))
        p._apply_extra(list(primal_in[base + 3 + nB:]))
        x = p.upload(primal_in[:3])
        dt = float(np.asarray(primal_in[3]).reshape(-1)[0])
        S = p.upload(primal_in[base:base + 3])
        seeds = p.upload(rest[:3])
        dtca = float(np.asarray(rest[3]).reshape(-1)[0])
        obja = float(np.asarray(rest[4]).reshape(-1)[0])
        if dtca != 0.0:
            raise NotImplementedError('dtca != 0: the CFL-sum output has no adjoint')
        # the stages the primal map kept for this very state, if any
        Sh = [primal_in[base + k] for k in range(3)]
        stages = p.kept_stages(primal_in[0], primal_in[1], primal_in[2], dt, Sh)
        tape = None
        if stages is None:
            stages, tape = self._forward_with_tape(x, dt, S)
        adj, grads = self._step(x, dt, seeds, S, stages=stages, tape=tape, obja=obja)
        # float64 host arrays (FP32 results widened on the way)
        return p.download(list(adj) + list(grads))

    def _forward_with_tape(self, x, dt, S):
        """The primal step of the map's state run once more with its stage states and tape kept
        (buffers reused across calls), so that the adjoint step reads the forward's cell records
        (and, in FP64, its face values) instead of re-evaluating them: the re-evaluation inside
        the FP64 face VJP costs more FP64 instructions than the forward flux that writes the
        tape. (None, None) - the adjoint step then recomputes its forward itself - when the
        buffers would take more than a quarter of the device's free memory."""
        p = self.primal
        if self._fwd is None:
            torch = _torch()
            free = torch.cuda.mem_get_info(p.device)[0]
            need = p.tape_bytes + 10 * self.mesh.nInternalCells * np.dtype(p.dtype).itemsize
            self._fwd = (p.stage_buffer(), p.tape_buffer()) if need <= free // 4 else False
        if not self._fwd:
            return None, None
        st, tp = self._fwd
        p.step(x[0], x[1], x[2], dt, S=S, want_scalars=False, stages=st, tape=tp)
        return st, tp

    def computeEnergy(self, adj, state):
        """sqrt of the adjoint energy (apps/adjoint.py:55 over cmesh.computeEnergy); device tensors."""
        return self.primal.adjoint_energy(adj, state) ** 0.5

    # ------------------------------------------------------------ the sweep
    def run(self, fields, nSteps, dt, writeInterval, perturbations=(), avgStart=0, source=None, keep_stages=True,
            keep_tapes=None):
        """Checkpointed adjoint sweep on the device.

        fields: initial conservative state (host arrays). dt: a float (fixed step) or the
        per-step dt series of the primal run. perturbations: list of perturbations of the
        parameters, each a tuple of host arrays shaped like the parameter gradients ((dS_rho,
        dS_rhoU, dS_rhoE) for 'source', the ten mesh tensors for 'mesh', the one boundary
        input otherwise). keep_stages: the interval's forward re-run also keeps every
        step's RK stage states (10 nInternalCells values a step) so that the adjoint steps
        do not recompute them. keep_tapes: with keep_stages, also keep every step's tape (its
        stages' cell records and, in FP64, the face tape); None: when the interval's tapes fit
        in 32 GB. Returns (sensitivities, adjoint fields at t0 (host), record)."""
        torch = _torch()
        p = self.primal
        if nSteps % writeInterval:
            raise ValueError('nSteps must be a multiple of writeInterval (apps/problem.py:30-31)')
        n = self.mesh.nInternalCells
        dev = 'cuda:%d' % p.device
        td = torch.float64 if p.dtype == np.float64 else torch.float32
        T = lambda a, d: torch.as_tensor(np.ascontiguousarray(np.asarray(a).reshape(n, d)), dtype=td, device=dev)
        x0 = [T(a, d) for a, d in zip(fields, (1, 3, 1))]
        S = None if source is None else [T(a, d) for a, d in zip(source, (1, 3, 1))]
        dts = list(dt) if np.ndim(dt) else [float(dt)] * nSteps
        # primal forward: keep the interval-start states (checkpoints) on the device
        checkpoints = []
        x = x0
        objs = []
        for k in range(nSteps):
            if k % writeInterval == 0:
                checkpoints.append([t.clone() for t in x])
            r = p.step(x[0], x[1], x[2], dts[k], S=S)
            objs.append(r[4])
            x = list(r[:3])
        perts = [[torch.as_tensor(np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1)), device=dev)
                  for a in pert] for pert in perturbations]
        result = [0.0] * len(perts)
        a = [torch.zeros_like(t) for t in x0]
        sens_series = []
        nCk = nSteps // writeInterval
        stages = [p.stage_buffer() for _ in range(writeInterval)] if keep_stages else None
        if keep_tapes is None:
            keep_tapes = writeInterval * p.tape_bytes <= 32e9
        tapes = [p.tape_buffer() for _ in range(writeInterval)] if keep_stages and keep_tapes else None
        for checkpoint in range(nCk):
            primalIndex = nSteps - (checkpoint + 1) * writeInterval
            states = [checkpoints[primalIndex // writeInterval]]
            last = primalIndex + writeInterval - (0 if keep_stages else 1)
            for k in range(primalIndex, last):
                y = states[-1]
                sb = stages[k - primalIndex] if keep_stages else None
                tb = tapes[k - primalIndex] if tapes else None
                states.append(list(p.step(y[0], y[1], y[2], dts[k], S=S, want_scalars=False, stages=sb,
                                          tape=tb)[:3]))
            for step in range(writeInterval):
                adjointIndex = writeInterval - 1 - step
                y = states[adjointIndex]
                sb = stages[adjointIndex] if keep_stages else None
                tb = tapes[adjointIndex] if tapes else None
                _, pgrads = self._step(y, dts[primalIndex + adjointIndex], a, S, out=a, stages=sb, tape=tb)
                if self.viscosityType and (step + 1) % self.viscousInterval == 0:
                    p.adjoint_viscosity(y[0], y[1], y[2], a, dts[primalIndex + adjointIndex], self.viscosityType,
                                        self.scaling)
                grads = [g.reshape(-1).double() for g in pgrads]
                sens = [p.sensitivity(grads, pert) for pert in perts]
                sens_series.append(sens)
                if (nSteps - (primalIndex + adjointIndex)) > avgStart:
                    for i, s in enumerate(sens):
                        result[i] += s
        out = [r / (nSteps - avgStart) for r in result]
        return out, [t.cpu().numpy() for t in a], {'objective': objs, 'sensitivity': sens_series}
