"""Continuous-batching server for sensitivity requests (primal run + adjoint sweep per request).

A request names a mesh (a jittered periodic box ``box<n>`` or a cylinder O-grid
``cyl<nt>x<nr>``), carries a seeded initial state and a source perturbation, and asks for the
sensitivity of the time-summed objective to that perturbation after ``nPrimal`` primal steps
and the adjoint sweep back to t0 - the work of apps/problem.py + apps/adjoint.py for one case.

Design:
* A *slot* owns one solver context (mesh tables and work buffers on the device), one CUDA
  stream, its state/checkpoint/adjoint buffers and three CUDA graphs captured once: ``k``
  primal steps in place; the recompute of a checkpoint segment; the ``k`` adjoint steps of a
  segment with the FP64 sensitivity accumulation. A slot is tied to a mesh and is reused by the
  next request on that mesh (new state and perturbation copied into the same buffers, so the
  graphs stay valid).
* Requests arriving while others run are admitted as soon as a slot for their mesh is free, or
  a new slot fits in the HBM budget (footprint measured on the first slot of each mesh,
  estimated before that). Slots of finished requests stay resident until memory is needed.
* Every engine pass launches the next graph of every active request, each on its own stream,
  so the work of all requests overlaps on the GPU; the host only polls events.
* Kernels are per request and reductions have fixed orders (no atomics across requests), so a
  request's result is bitwise the same alone and in any mix.
* Batched slots (``batch={key: K}``): one slot runs up to K requests on the same mesh in the
  same launches - its context is built on K disjoint copies of the mesh (cases.copies), each
  request's state and perturbation in its copy's cells, its sensitivity the sum over its own
  cells. Small meshes (thousands of cells) leave the GPU idle between their short kernels;
  packed K to a launch they fill it. Every cell of a copy computes exactly what it computes on
  the single mesh, so a request's result does not depend on which copy it runs in or on the
  other requests of the batch.
"""
import collections
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import cases
from .solver import RCF


def _torch():
    import torch
    return torch


def make_case(key):
    if key.startswith('box'):
        return cases.box(int(key[3:]), objective='kinetic_energy')
    if key.startswith('cyl'):
        a, b = key[3:].split('x')
        return cases.cylinder(int(a), int(b))
    raise ValueError(key)


class MeshLibrary(object):
    """Host cache of built cases (mesh geometry, BCs, initial state recipe) by key."""

    def __init__(self):
        self.cases = {}

    def get(self, key, copies=1):
        ck = key if copies == 1 else (key, copies)
        if ck not in self.cases:
            c = make_case(key) if copies == 1 else cases.copies(self.get(key), copies)
            c.build_mesh()
            self.cases[ck] = c
        return self.cases[ck]


@dataclass
class Request:
    rid: int
    key: str
    seed: int = 0
    nPrimal: int = 100
    arrival: float = 0.0
    # the request's payload: (state, source perturbation) as pinned host tensors, made by the
    # client (``prepare``); the server makes them itself when absent
    inputs: tuple = None
    # results
    sensitivity: float = None
    objective: float = None
    t_admit: float = None
    t_done: float = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def prepare(requests, library):
    """Client side: the payload of each request (seeded initial state and source perturbation,
    ``request_inputs``) as FP64 tensors in pinned host memory, so the server's copies to the
    device are asynchronous."""
    torch = _torch()
    for r in requests:
        if r.inputs is None:
            state, dS = request_inputs(library.get(r.key), r.seed)
            pin = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64)).pin_memory()
            r.inputs = ([pin(a) for a in state], [pin(a) for a in dS])
    return requests


def request_inputs(case, seed):
    """Seeded initial conservative state (the case recipe plus a 0.1 % seeded density
    perturbation) and source perturbation of a request."""
    rho, rhoU, rhoE = cases.conservative(case)
    rng = np.random.default_rng(1000 + seed)
    rho = rho * (1.0 + 1e-3 * rng.standard_normal(rho.shape))
    dS = cases.source_field(case.mesh, scale=1e-3, seed=seed)
    return (rho, rhoU, rhoE), dS


class Slot(object):
    def __init__(self, case, key, precision, device, k, nPrimal, copies=1):
        torch = _torch()
        self.key = key
        self.case = case
        self.copies = copies                  # requests a launch serves (disjoint mesh copies)
        self.k = k
        self.nPrimal = nPrimal
        self.nck = nPrimal // k
        self.dev = torch.device('cuda', device)
        # FP32 records: the gauge of the case's initial field (the far field's on a cylinder, the
        # mean state of a periodic box, which fixes no boundary value)
        self.rcf = RCF(case.mesh, case.bc, objective=case.objective, precision=precision, device=device,
                       gauge=None if precision == 'fp64' else cases.gauge(case), **case.config)
        self.td = torch.float32 if precision == 'fp32' else torch.float64      # state type
        n = case.mesh.nInternalCells
        shapes = [(n, 1), (n, 3), (n, 1)]
        z = lambda: [torch.zeros(s, dtype=self.td, device=self.dev) for s in shapes]
        self.x = z()
        self.ckpt = [z() for _ in range(self.nck)]
        self.states = [z() for _ in range(k)]
        self.last = z()                                        # output of the interval's last step
        self.stages = [self.rcf.stage_buffer() for _ in range(k)]
        self.tapes = [self.rcf.tape_buffer() for _ in range(k)]        # the stages' cell records
        self.a = z()
        self.S = z()
        self.dS = [torch.zeros(s, dtype=torch.float64, device=self.dev) for s in shapes]
        self.acc = torch.zeros(copies, dtype=torch.float64, device=self.dev)
        self.objacc = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self.dt = case.dt
        self.stream = torch.cuda.Stream(device=self.dev)
        self.busy = False
        self.req = None
        self.reqs = []
        self.graphs = None
        self.ev = torch.cuda.Event()

    # ---- the three step sequences (captured into graphs)
    def _primal_k(self):
        for _ in range(self.k):
            r = self.rcf.step(self.x[0], self.x[1], self.x[2], self.dt, S=self.S, out=self.x, want_scalars=False)

    def _recompute(self):
        # the interval's states and each step's RK stage states, for the adjoint steps
        for j in range(self.k):
            y = self.states[j]
            out = self.states[j + 1] if j + 1 < self.k else self.last
            self.rcf.step(y[0], y[1], y[2], self.dt, S=self.S, out=out, want_scalars=False, stages=self.stages[j],
                          tape=self.tapes[j])

    def _adjoint_k(self):
        torch = _torch()
        for j in range(self.k - 1, -1, -1):
            y = self.states[j]
            r = self.rcf.adjoint_step(y[0], y[1], y[2], self.dt, self.a, obja=1.0, S=self.S, out=self.a,
                                      stages=self.stages[j], tape=self.tapes[j])
            # FP64 sensitivity accumulation (cmesh.computeSensitivity summed over time), one sum a
            # request over its own cells
            K = self.copies
            s = (r[3][0].double() * self.dS[0]).view(K, -1).sum(1) + \
                (r[3][1].double() * self.dS[1]).view(K, -1).sum(1) + \
                (r[3][2].double() * self.dS[2]).view(K, -1).sum(1)
            self.acc.add_(s)

    def capture(self):
        torch = _torch()
        with torch.cuda.stream(self.stream):
            # warm-up (allocates the adjoint buffers outside capture)
            self._primal_k()
            self.states[0][0].copy_(self.x[0])
            self._recompute()
            self._adjoint_k()
        self.stream.synchronize()
        self.graphs = []
        for fn in (self._primal_k, self._recompute, self._adjoint_k):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream):
                fn()
            self.graphs.append(g)
        self.stream.synchronize()

    # ---- a request's work as a list of small host closures, run one per engine pass
    def start(self, reqs, payloads):
        """reqs: up to ``copies`` requests; payloads: their (state, dS), host arrays or pinned
        host tensors (copied asynchronously), each into its copy's cells. Copies without a
        request run the first request's state with a zero perturbation (their results unused)."""
        torch = _torch()
        self.reqs = list(reqs)
        self.req = self.reqs[0]
        self.busy = True
        host = lambda v: v if isinstance(v, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(v, np.float64))
        K = self.copies
        with torch.cuda.stream(self.stream):
            for j in range(K):
                state, dS = payloads[j] if j < len(payloads) else payloads[0]
                for t, v in zip(self.x, state):
                    v = host(v)
                    t.view(K, -1)[j].copy_(v.reshape(-1), non_blocking=v.is_pinned())
                for t, v in zip(self.dS, dS):
                    if j < len(payloads):
                        v = host(v)
                        t.view(K, -1)[j].copy_(v.reshape(-1), non_blocking=v.is_pinned())
                    else:
                        t.view(K, -1)[j].zero_()
            for t in self.a:
                t.zero_()
            self.acc.zero_()
        plan = []
        for c in range(self.nck):
            plan.append(('save', c))
            plan.append(('primal', c))
        for c in range(self.nck - 1, -1, -1):
            plan.append(('restore', c))
            plan.append(('recompute', c))
            plan.append(('adjoint', c))
        self.plan = collections.deque(plan)

    def advance(self):
        """Launch the next item of the plan on this slot's stream (no host sync)."""
        torch = _torch()
        if not self.plan:
            return False
        op, c = self.plan.popleft()
        with torch.cuda.stream(self.stream):
            if op == 'save':
                for d, s in zip(self.ckpt[c], self.x):
                    d.copy_(s)
            elif op == 'primal':
                self.graphs[0].replay()
            elif op == 'restore':
                for d, s in zip(self.states[0], self.ckpt[c]):
                    d.copy_(s)
            elif op == 'recompute':
                self.graphs[1].replay()
            elif op == 'adjoint':
                self.graphs[2].replay()
            if not self.plan:
                self.ev.record(self.stream)
        return True

    def finished(self):
        return self.busy and not self.plan and self.ev.query()

    def bytes(self):
        torch = _torch()
        es = 8 if self.td == torch.float64 else 4
        n = self.case.mesh.nInternalCells
        # checkpoints, interval states, last output, x, a, S; the k stage buffers and tapes; FP64 dS
        return int(self.rcf.device_bytes + (self.nck + self.k + 4) * 5 * n * es + self.k * 10 * n * es +
                   self.k * self.rcf.tape_bytes + 3 * 5 * n * 8)


class SensitivityServer(object):
    def __init__(self, precision='fp32', device=0, hbm_budget=40e9, k=10, nPrimal=100, max_slots=48,
                 library=None, batch=None):
        self.precision = precision
        self.device = device
        self.budget = hbm_budget
        self.k = k
        self.nPrimal = nPrimal
        self.max_slots = max_slots
        self.lib = library or MeshLibrary()
        self.slots = []
        self.bytes_of = {}
        self.used = 0
        self.batch = dict(batch or {})   # mesh key -> requests per launch (batched slots)
        self.evictions = 0          # idle slots released to make room for another mesh's slot
        self.queued = 0             # requests that waited for a slot after they arrived

    def close(self):
        """Release every slot's device context."""
        for s in self.slots:
            s.rcf.close()
        self.slots = []
        self.used = 0

    def warm(self, keys):
        """Create (and capture) slots ahead of traffic: as many slots of each mesh key as the
        key appears in ``keys`` (one per distinct key for a list of distinct keys), within
        the HBM budget and the slot limit; no slot is evicted for this. Returns the number of
        slots created."""
        made = 0
        for key, count in collections.Counter(keys).items():
            while sum(s.key == key for s in self.slots) < count:
                if self._new_slot(key, evict=False) is None:
                    if not any(s.key == key for s in self.slots):
                        raise RuntimeError('HBM budget too small for a slot of %s' % key)
                    break
                made += 1
        return made

    def _estimate(self, key):
        if key in self.bytes_of:
            return self.bytes_of[key]
        m = self.lib.get(key, self.batch.get(key, 1)).mesh
        er = 8 if self.precision == 'fp64' else 4      # mesh tables, records, face fluxes
        es = 4 if self.precision == 'fp32' else 8      # states, stages, checkpoints, adjoints
        # per face: tables, flux records, adjoint face records (and FP64 face tapes); per cell:
        # tables and cell records, RK and adjoint work states, checkpoints, interval states,
        # stage buffers and the tapes' cell records
        face_tape = 3 * 61 * 8 * self.k if self.precision == 'fp64' else 0
        return int(m.nFaces * (60 + 28 * er + 40 * er + face_tape) + m.nInternalCells * (150 + 40 * er + 40 * es
                   + (self.nPrimal // self.k + 3 * self.k + 8) * 5 * es) + m.nCells * 3 * 20 * er * self.k)

    def _slot_for(self, key):
        for s in self.slots:
            if s.key == key and not s.busy:
                return s
        return self._new_slot(key)

    def _new_slot(self, key, evict=True):
        need = self._estimate(key)
        while self.used + need > self.budget or len(self.slots) >= self.max_slots:
            idle = [s for s in self.slots if not s.busy]
            if not idle or not evict:
                return None
            victim = idle[0]
            self.slots.remove(victim)
            self.used -= victim.bytes()
            victim.rcf.close()
            self.evictions += 1
        K = self.batch.get(key, 1)
        s = Slot(self.lib.get(key, K), key, self.precision, self.device, self.k, self.nPrimal, copies=K)
        s.capture()
        self.bytes_of[key] = s.bytes()
        self.used += s.bytes()
        self.slots.append(s)
        return s

    def serve(self, requests, realtime=True):
        """Serve requests (sorted by arrival time, seconds from start). Returns stats."""
        torch = _torch()
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = collections.deque()
        active = []
        t0 = time.perf_counter()
        done = []
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and (pending[0].arrival <= now or not realtime):
                waiting.append(pending.popleft())
            # admission, FIFO
            while waiting:
                r = waiting[0]
                s = self._slot_for(r.key)
                if s is None:
                    if not getattr(r, '_queued', False):
                        r._queued = True
                        self.queued += 1
                    break
                # a batched slot takes the next waiting requests on the same mesh too, up to its
                # number of copies
                group = [waiting.popleft()]
                for q in list(waiting):
                    if len(group) >= s.copies:
                        break
                    if q.key == r.key:
                        waiting.remove(q)
                        group.append(q)
                base = self.lib.get(r.key)
                payloads = [q.inputs if q.inputs is not None else request_inputs(base, q.seed) for q in group]
                s.start(group, payloads)
                for q in group:
                    q.t_admit = time.perf_counter() - t0
                active.append(s)
            progressed = False
            for s in active:
                progressed |= s.advance()
            for s in list(active):
                if s.finished():
                    acc = s.acc.cpu().tolist()
                    for j, r in enumerate(s.reqs):
                        r.sensitivity = acc[j] / r.nPrimal
                        r.t_done = time.perf_counter() - t0
                        done.append(r)
                    s.busy = False
                    s.req = None
                    s.reqs = []
                    active.remove(s)
            if not progressed and not active and pending and realtime:
                time.sleep(max(0.0, min(0.002, pending[0].arrival - (time.perf_counter() - t0))))
        elapsed = time.perf_counter() - t0
        lat = sorted(r.latency for r in done)
        pct = lambda q: lat[min(len(lat) - 1, int(math.ceil(q * len(lat))) - 1)] if lat else None
        return {'requests': len(done), 'elapsed_s': elapsed, 'req_per_s': len(done) / elapsed if elapsed else None,
                'p50_s': pct(0.50), 'p99_s': pct(0.99), 'slots': len(self.slots),
                'device_bytes': self.used}


def plain_one_at_a_time(requests, library, device=0, nPrimal=100):
    """The plain form: FP64, one request at a time, step calls without graphs or overlap,
    the adjoint sweep storing every state (no checkpointing). Returns stats and results."""
    torch = _torch()
    ctxs = {}
    for r in requests:              # solver contexts are set up before the clock starts
        case = library.get(r.key)
        if r.key not in ctxs:
            ctxs[r.key] = RCF(case.mesh, case.bc, objective=case.objective, precision='fp64', device=device,
                              **case.config)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = []
    times = []
    for r in requests:
        tr = time.perf_counter()
        case = library.get(r.key)
        rcf = ctxs[r.key]
        state, dS = r.inputs if r.inputs is not None else request_inputs(case, r.seed)
        x = [torch.as_tensor(a).cuda(device) for a in state]
        d = [torch.as_tensor(a).cuda(device) for a in dS]
        states = [x]
        for n in range(nPrimal):
            y = rcf.step(x[0], x[1], x[2], case.dt, S=None, want_scalars=False)
            x = list(y[:3])
            states.append(x)
        a = [torch.zeros_like(t) for t in x]
        acc = torch.zeros((), dtype=torch.float64, device=x[0].device)
        for n in range(nPrimal - 1, -1, -1):
            y = states[n]
            rr = rcf.adjoint_step(y[0], y[1], y[2], case.dt, a, obja=1.0, out=a)
            acc += sum((g.double() * p).sum() for g, p in zip(rr[3], d))
        r.sensitivity = float(acc) / nPrimal
        out.append(r)
        times.append(time.perf_counter() - tr)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    return {'requests': len(out), 'elapsed_s': el, 'req_per_s': len(out) / el, 'seconds_per_request': times}
