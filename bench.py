"""Benchmark of the GB300 finite-volume step (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload box128|box64|...] [--precision fp64|fp32]

A step is one SSP-RK3 time step (three residual evaluations) of the periodic jittered box
(the throughput workload: 128^3 cells, Roe flux, Sutherland viscosity), state resident in
HBM. ``value`` is whole-job Mcell-steps/s; ``e2e`` is the same metric through the host-buffer
entry point (afvm_primal_step_host: pinned host state in, host state out, copies inside the
timed region). Multi-GPU runs are independent replicas (one per rank, weak scaling).
``--impl reference`` times the CPU oracle (the restated reference path) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'primal+adjoint Mcell-steps/s on 1 GB300 vs plain; sensitivity req/s, p99 @ tol'
UNIT = 'Mcell-steps/s'


def max_over_ranks(values, dist, device='cuda'):
    """Element-wise maximum of per-rank timings (the whole-job time of a replica run)."""
    import torch
    if dist is None:
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


# algorithmic (compulsory) bytes per launch of each primal kernel, FP64 / FP32 element size
# es and int32 indices (per-unit counts in the comments below)
def algorithmic_bytes(kernel, nIC, nIF, nF, nG, es, taped=False):
    REC, FREC, TAPE, GEO = 20, 6, 61, 15
    if kernel == 'k_flux':
        # per face: own+nbr (8), normals 3, deltas 1, deltasUnit 3, linearWeights 2,
        # quadraticWeights 6 -> 15 values, and in FP64 N - (N.D) D and N.D (4 more), flux record
        # write 6 (and the 61-value face tape when taped); cell records read once
        return nF * (8 + (GEO + 4 * (es == 8)) * es + FREC * es + (TAPE * es if taped else 0)) + (nIC + nG) * REC * es
    if kernel == 'k_grad':
        # per cell: 6 slots x (nbr 4 + w' + S*N' (3)) + 1/V, primitives of every cell once,
        # gradient write 15
        return nIC * (6 * (4 + 4 * es) + es + 15 * es) + (nIC + nG) * 5 * es
    if kernel == 'k_update':
        # per cell: 6 x (face id 4 + weight), 2 stage states + source (5 each), write 5;
        # face flux records read once
        return nIC * (6 * (4 + es) + 3 * 5 * es + 5 * es) + nF * FREC * es
    if kernel == 'k_prim':
        return nIC * 10 * es + nG * (8 + 5 * es + 5 * es)
    if kernel == 'k_adj_flux' and taped:
        # per face: own+nbr (8), A/V weights 2, geometry 15 (19 in FP64), the 61-value face tape,
        # 40-value adjoint record write; the 5 adjoint seeds of every cell once; the two cell
        # records of each boundary face (boundary faces are not taped)
        return nF * (8 + (2 + GEO + 4 * (es == 8) + TAPE + 40) * es) + nIC * 5 * es + (nF - nIF) * 2 * REC * es
    if kernel == 'k_adj_flux':
        # per face: own+nbr (8), A/V weights 2, geometry 15 (19 in FP64), 40-value adjoint record
        # write; cell records and the 5 adjoint seeds of every cell read once
        return nF * (8 + (2 + GEO + 4 * (es == 8)) * es + 40 * es) + (nIC + nG) * REC * es + nIC * 5 * es
    return 0


# the cell-step model of compulsory bytes (two passes per stage, every array once a pass): FP64
# primal 2,904 B, FP32 primal 1,524 B, FP64 adjoint 6,288 B (forward recompute + reverse); the
# FP32 adjoint scaled from the FP64 one by the primal ratio
STEP_BYTES = {('primal', 8): 2904, ('primal', 4): 1524, ('adjoint', 8): 6288, ('adjoint', 4): 3300}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch from an ncu capture of
# the 64^3 box (798,720 faces, 262,144 cells; profiles/), scaled to a launch of the benchmarked
# mesh by its number of faces (the kernel's traffic grows in proportion to the faces). The FP64
# kernels (taped: the benchmarked step with its 61-value face tape; untaped: --tape 0) are from
# captures of the current build, the FP32 ones from earlier captures of the same kernels.
MEASURED_TRAFFIC = {('k_flux', 8): (200.3e6, 798720), ('k_flux', 4): (81.56e6, 798720),
                    ('k_adj_flux', 8): (455.5e6, 798720), ('k_adj_flux', 4): (170.37e6, 798720),
                    ('k_flux+tape', 8): (547.1e6, 798720), ('k_adj_flux+tape', 8): (763.2e6, 798720)}
# FP64 thread instructions per face (DADD, DMUL, DFMA) of a launch in the same captures
# (smsp__sass_thread_inst_executed_op_d{add,mul,fma}_pred_on), current build; the untaped
# forward flux issues a few FP64 instructions fewer than the taped one (the tape's values it
# need not form)
MEASURED_FP64_INST = {'k_flux': (50.0, 85.1, 157.2), 'k_adj_flux': (82.0, 188.5, 314.4),
                      'k_flux+tape': (52.0, 90.1, 156.2), 'k_adj_flux+tape': (40.0, 105.7, 177.4)}
# every warp instruction the FP64 pipe issued, per face (smsp__inst_executed_pipe_fp64 x 32 / faces,
# the same captures): the arithmetic above plus the issues of warps whose lanes were partly masked
# (branches that only some of a warp's faces take)
MEASURED_FP64_PIPE_INST = {'k_flux': 295.0, 'k_adj_flux': 589.8, 'k_flux+tape': 301.0, 'k_adj_flux+tape': 328.8}


def measured_traffic(kernel, es, nF):
    v = MEASURED_TRAFFIC.get((kernel, es))
    if v is None:
        return None
    return int(v[0] * nF / v[1])


class ClockSampler(object):
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(smax) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def make_case(workload, builder=None):
    from adfvm_gb300 import cases
    if workload.startswith('box'):
        return cases.box(int(workload[3:]), objective='kinetic_energy', builder=builder)
    if workload.startswith('cylinder'):
        a, b = workload[8:].split('x')
        return cases.cylinder(int(a), int(b))
    if workload.startswith('sod'):
        return cases.sod(int(workload[3:]))
    raise ValueError(workload)


def describe(case, precision):
    m = case.mesh
    return {'workload': '%s: %d cells, %d faces (%d internal), Roe, SSP-RK3, %s, %s' % (
        case.name, m.nInternalCells, m.nFaces, m.nInternalFaces,
        'inviscid' if case.config.get('mu') == 0.0 else 'Sutherland viscosity', precision),
        'cells': int(m.nInternalCells), 'faces': int(m.nFaces)}


def reference_python():
    """The reference's own primal path (its Solver.run through the NumPy adpy stand-in), timed by
    oracle/time_reference.py on a development host that has the reference checkout (the machines
    that run this benchmark have none) and read from the fixture that script writes; None
    without it."""
    path = os.path.join(ROOT, 'oracle', 'reference_timing.json')
    try:
        with open(path) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    c = max(d['cases'], key=lambda x: x['cells'])
    return {'value': c['primal_mcell_steps_per_s'], 'unit': 'primal ' + UNIT, 'workload': c['workload'],
            'threads': d['threads'], 'host': '%s, %s cores' % (d['host'], d['cores']),
            'measured': 'on a development host with the reference checkout, %s (oracle/time_reference.py; not '
                        'on the benchmark machine, which has no checkout); the reference adjoint (adpy reverse '
                        'mode) is absent from the checkout' % d['measured_utc'],
            'cases': {x['workload'].split(':')[0]: x['primal_mcell_steps_per_s'] for x in d['cases']}}


def cpu_baseline(args, threads, seconds=10.0):
    """The reference path restated for the CPU, timed on the host cores on a bounded sample of
    the workload itself - the same mesh, state and dt:
      * the mesh built by the oracle's NumPy restatement of the reference's cmesh
        (oracle/geometry.py, bit for bit the reference's), so the timed arm loads no library;
      * FP64 primal steps by the C/OpenMP restatement of the residual and SSP-RK3 step
        (oracle/c/afvm_oracle.c);
      * FP64 adjoint steps by the host adjoint (oracle/c/adjoint_host.cpp: the C oracle's
        forward, the face VJP compiled for the host, the reverse sweep in OpenMP) - the
        reference has no CPU adjoint that runs (adpy's reverse mode is absent).
    value = primal+adjoint Mcell-steps/s from the per-cell-step times of the two; primal and
    adjoint are reported alone too."""
    from adfvm_gb300 import cases
    from oracle import geometry
    from oracle.c_ref import COracle
    os.environ['OMP_NUM_THREADS'] = str(threads)
    case = make_case(args.workload, builder=geometry.build_mesh)
    m = case.build_mesh()
    co = COracle(m, case.bc, case.config, case.objective)
    x = cases.conservative(case)
    co.step(x[0], x[1], x[2], case.dt)
    t0 = time.perf_counter()
    steps = 0
    while time.perf_counter() - t0 < seconds and steps < 200:
        x = co.step(x[0], x[1], x[2], case.dt)[:3]
        steps += 1
    tp = (time.perf_counter() - t0) / (steps * m.nInternalCells)        # s per cell-step
    seeds = [np.full(np.shape(a), 1e-3) for a in x]
    co.adjoint_step(x[0], x[1], x[2], case.dt, seeds)
    t0 = time.perf_counter()
    na = 0
    while time.perf_counter() - t0 < seconds and na < 200:
        a = co.adjoint_step(x[0], x[1], x[2], case.dt, seeds)
        seeds = list(a[:3])
        na += 1
    ta = (time.perf_counter() - t0) / (na * m.nInternalCells)
    return {'value': 1.0 / (tp + ta) / 1e6, 'unit': UNIT, 'cores': threads, 'kind': 'port',
            'config': describe(case, args.precision),
            'primal': round(1.0 / tp / 1e6, 4), 'adjoint': round(1.0 / ta / 1e6, 4), 'same_mesh': True,
            'sample': '%d FP64 primal steps (C/OpenMP oracle) and %d FP64 adjoint steps (host adjoint, OpenMP) of '
                      '%s (%d cells, the workload mesh, built by the oracle\'s restatement of the reference\'s '
                      'cmesh), %d threads' % (steps, na, case.name, m.nInternalCells, threads)}


def measure(case, precision, args, local, dist, world, clocks):
    """Timed primal steps and adjoint steps of one precision on the resident workload."""
    import torch
    from adfvm_gb300 import cases
    from adfvm_gb300.solver import RCF
    mesh = case.mesh
    rcf = RCF(mesh, case.bc, objective=case.objective, precision=precision, device=local,
              gauge=None if precision == 'fp64' else cases.gauge(case), **case.config)
    # state type (FP64 for 'fp64' and 'mixed') and record type (es: FP32 unless 'fp64')
    dt_np = np.float32 if precision == 'fp32' else np.float64
    tdt = torch.float32 if precision == 'fp32' else torch.float64
    x = [torch.as_tensor(np.ascontiguousarray(a, dt_np)).cuda() for a in cases.conservative(case)]
    dt = case.dt
    nIC, nIF, nF, nG = mesh.nInternalCells, mesh.nInternalFaces, mesh.nFaces, mesh.nGhostCells
    es = 8 if precision == 'fp64' else 4
    ss = 4 if precision == 'fp32' else 8
    stream = torch.cuda.current_stream()

    def timed(fn, steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        return max_over_ranks([ms], dist)[0]

    # a sweep: the primal steps keep their states, RK stage states and face tapes in rings of
    # the last R steps; the adjoint steps walk those steps backwards (cycling when K > R), each
    # on the state, stages and tape of one primal step, carrying the adjoint field as a real
    # sweep does. The ring is capped at 100 GB of tapes.
    # (a tape holds each stage's cell records, and in FP64 the face tape as well)
    use_tape = bool(args.tape)
    face_taped = use_tape and precision == 'fp64'
    tape_bytes = int(rcf.tape_buffer().numel()) * es if use_tape else 0
    R = max(1, min(args.steps, 32, int(100e9 // tape_bytes) if tape_bytes else 32))
    ring = [x] + [[torch.empty_like(t) for t in x] for _ in range(R)]
    stg = [rcf.stage_buffer() for _ in range(R)]
    tps = [rcf.tape_buffer() for _ in range(R)] if use_tape else [None] * R
    cnt = {'p': 0, 'a': 0}

    def primal():
        j = cnt['p']
        xi, xo = ring[j % (R + 1)], ring[(j + 1) % (R + 1)]
        rcf.step(xi[0], xi[1], xi[2], dt, out=xo, want_scalars=False, stages=stg[j % R], tape=tps[j % R])
        cnt['p'] = j + 1

    abuf = [torch.ones_like(t) * 1e-3 for t in x]
    sbuf = [torch.empty_like(t) for t in x]          # the source gradient, as the reference returns it

    def adjoint():
        q = cnt['a']
        cnt['a'] = q + 1
        j = cnt['p'] - 1 - (q % min(R, cnt['p']))
        xi = ring[j % (R + 1)]
        rcf.adjoint_step(xi[0], xi[1], xi[2], dt, abuf, obja=1.0, out=abuf, stages=stg[j % R], tape=tps[j % R],
                         source_out=sbuf)

    for _ in range(args.warmup):
        primal()
        adjoint()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    rcf.profile(True)
    ms_p = timed(primal, args.steps)
    prof = rcf.profile_read()
    rcf.profile(True)
    ms_a = timed(adjoint, args.steps)
    prof_a = rcf.profile_read()
    rcf.profile(False)
    clk = clocks.stop() if clocks else None
    K = args.steps
    vp = nIC * K * world / (ms_p / 1e3) / 1e6
    va = nIC * K * world / (ms_a / 1e3) / 1e6
    value = nIC * K * world / ((ms_p + ms_a) / 1e3) / 1e6

    # end to end through the host-buffer entry point (pinned host buffers)
    pin = [torch.empty(tuple(t.shape), dtype=tdt, pin_memory=True).numpy() for t in x]
    pout = [torch.empty(tuple(t.shape), dtype=tdt, pin_memory=True).numpy() for t in x]
    for a, b in zip(pin, ring[cnt['p'] % (R + 1)]):
        a[...] = b.cpu().numpy()
    rcf.step_host(pin[0], pin[1], pin[2], dt, out=pout)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    ke = max(1, K // 2)
    for _ in range(ke):
        rcf.step_host(pin[0], pin[1], pin[2], dt, out=pout)
        pin, pout = pout, pin
    te = time.perf_counter() - t0
    # adjoint through the reference-facing Adjoint.map (host arrays in and out)
    from adfvm_gb300.adjoint import Adjoint
    adj = Adjoint(rcf)
    host_x = [np.ascontiguousarray(a, np.float64) for a in pin]
    host_seeds = [np.full(a.shape, 1e-3) for a in host_x]
    ainputs = rcf.mapInputs(*host_x, dt) + host_seeds + [np.zeros((1, 1)), np.ones((1, 1)), np.zeros((1, 1))]
    adj.map(*ainputs)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        aout = adj.map(*ainputs)
    ta = time.perf_counter() - t0
    te, ta = max_over_ranks([te, ta], dist)
    state_bytes = int(sum(a.nbytes for a in pin))
    e2e = {'value': round(nIC * ke * world / (te + ta) / 1e6, 3), 'unit': UNIT,
           'h2d_bytes_per_step': state_bytes + int(3 * sum(a.size for a in host_x) * ss),
           'd2h_bytes_per_step': state_bytes + 16 + int(2 * sum(a.size for a in host_x) * ss),
           'path': 'primal: afvm_primal_step_host (pinned host state in/out, dtc and objective read back); '
                   'adjoint: Adjoint.map (reference input list; state, sources, seeds in; state and source '
                   'adjoints out)',
           'primal_only': round(nIC * ke * world / te / 1e6, 3), 'adjoint_only': round(nIC * ke * world / ta / 1e6, 3)}
    kernels = {k: {'ms_total': round(v[0], 4), 'launches': v[1], 'ms_avg': round(v[0] / v[1], 5)}
               for k, v in prof.items()}
    # the dominant kernel of the primal+adjoint step
    both = {}
    for pr in (prof, prof_a):
        for k, v in pr.items():
            t = both.setdefault(k, [0.0, 0])
            t[0] += v[0]
            t[1] += v[1]
    top = max(both.items(), key=lambda kv: kv[1][0])[0]
    peak, peak_kind = peaks()
    alg = algorithmic_bytes(top, nIC, nIF, nF, nG, es, taped=face_taped)
    topkey = top + ('+tape' if face_taped and top in ('k_flux', 'k_adj_flux') else '')
    avg_s = both[top][0] / both[top][1] / 1e3
    achieved = alg / avg_s / 1e9
    roofline = {'bound': 'hbm', 'kernel': topkey, 'achieved': round(achieved, 1), 'peak': peak,
                'peak_source': peak_kind, 'unit': 'GB/s', 'frac': round(achieved / peak, 4),
                'algorithmic_bytes_per_launch': int(alg), 'traffic': measured_traffic(topkey, es, nF),
                'share_of_step': round(both[top][0] / (ms_p + ms_a), 3)}
    step_model = {'unit': 'GB/s', 'peak': peak,
                  'primal': round(vp * 1e6 * STEP_BYTES[('primal', es)] / 1e9, 1),
                  'adjoint': round(va * 1e6 * STEP_BYTES[('adjoint', es)] / 1e9, 1),
                  'bytes_per_cell_step': {'primal': STEP_BYTES[('primal', es)],
                                          'adjoint': STEP_BYTES[('adjoint', es)]}}
    step_model['primal_frac'] = round(step_model['primal'] / peak, 4)
    step_model['adjoint_frac'] = round(step_model['adjoint'] / peak, 4)
    return {'value': round(value, 3), 'ms_per_step': round((ms_p + ms_a) / K, 4),
            'primal': {'value': round(vp, 3), 'ms_per_step': round(ms_p / K, 4)},
            'adjoint': {'value': round(va, 3), 'ms_per_step': round(ms_a / K, 4)},
            'roofline': roofline, 'kernels': kernels, 'step_model': step_model,
            '_top': (topkey, avg_s, nF), 'tape': face_taped,
            'adjoint_kernels': {k: {'ms_total': round(v[0], 4), 'launches': v[1], 'ms_avg': round(v[0] / v[1], 5)}
                                for k, v in prof_a.items()},
            'gpu_launches': int(sum(v[1] for v in prof.values()) + sum(v[1] for v in prof_a.values())),
            'e2e': e2e, 'clocks': clk, 'device_bytes': rcf.device_bytes}


def mesh_build_timing(case, local, reps=3):
    """Geometry/connectivity build of the workload mesh on the host (afvm_mesh_build, all
    cores) and on the GPU (afvm_mesh_build_device, host arrays in and out), and the solver
    context set-up (tables + upload) - the admission cost of a new mesh."""
    import torch
    from adfvm_gb300.mesh import Mesh
    from adfvm_gb300.solver import RCF
    md = case.meshData
    Mesh.create(md, device=local)
    th, td = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        Mesh.create(md)
        th.append(time.perf_counter() - t0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Mesh.create(md, device=local)
        td.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    rcf = RCF(case.mesh, case.bc, objective=case.objective, device=local, **case.config)
    tc = time.perf_counter() - t0
    rcf.close()
    return {'host_ms': round(1e3 * min(th), 1), 'device_ms': round(1e3 * min(td), 1),
            'host_threads': os.cpu_count(), 'context_ms': round(1e3 * tc, 1),
            'note': 'device_ms includes the upload of points/faces/owner/neighbour and the download of '
                    'every result to host arrays'}


def reorder_timing(n, local, steps=5):
    """The shuffled n^3 box (cells in random order, seed 1): the device renumbering
    (afvm_mesh_reorder_device, host arrays in and out) and the FP32 and FP64 primal steps on
    the mesh before and after it (CUDA events over ``steps`` steps) - what a mesh admitted in
    an arbitrary cell order costs without and with the renumbering."""
    import torch
    from adfvm_gb300 import cases, meshgen
    from adfvm_gb300.mesh import Mesh, reorder
    from adfvm_gb300.solver import RCF
    md = meshgen.periodic_box(n, reorder=False)
    reorder(meshgen.periodic_box(8, reorder=False), device=local)      # load and warm the path
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    md2, cn, _, bw = reorder(md, device=local)
    t_re = time.perf_counter() - t0
    ref = cases.box(n)
    out = {'mesh': 'box%d shuffled' % n, 'cells': int(len(cn)), 'reorder_ms': round(1e3 * t_re, 1),
           'bandwidth_before': bw[0], 'bandwidth_after': bw[1]}
    for tag, data in (('shuffled', md), ('reordered', md2)):
        mesh = Mesh.create(data, device=local)
        for prec, td in (('fp32', torch.float32), ('fp64', torch.float64)):
            rcf = RCF(mesh, ref.bc, objective=ref.objective, precision=prec, device=local, **ref.config)
            x = [torch.as_tensor(a).to(td).cuda(local)
                 for a in rcf.conservative(np.zeros((mesh.nInternalCells, 3)), np.full((mesh.nInternalCells, 1), 300.0),
                                           np.full((mesh.nInternalCells, 1), 1.0332e5))]
            for _ in range(2):
                rcf.step(x[0], x[1], x[2], ref.dt, out=x, want_scalars=False)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(steps):
                rcf.step(x[0], x[1], x[2], ref.dt, out=x, want_scalars=False)
            e1.record()
            torch.cuda.synchronize()
            out['%s_%s_ms_per_step' % (tag, prec)] = round(e0.elapsed_time(e1) / steps, 3)
            rcf.close()
    return out


SERVING_KEYS = ['box16', 'box24', 'box32', 'box48', 'box64', 'box96', 'cyl64x32', 'cyl128x64', 'cyl256x128']
SERVING_LAMBDAS = (1.0, 2.0, 5.0, 10.0, 20.0, 50.0, 100.0, 200.0)


def serving_bench(local, lams=SERVING_LAMBDAS, seed=4, n_mix=48, window_s=6.0, precision='fp32', compare='mixed',
                  cell_ns=None):
    """Sensitivity requests, each a jittered periodic box of side 16-96 or a cylinder O-grid
    64x32-256x128 drawn uniformly (seed 4), 100 primal + 100 adjoint steps.

    * capacity on one mix of n_mix requests: served (``precision``; continuous batching, all
      admitted at once) against the plain FP64 one-at-a-time form, whose time on the mix is
      the sum of its measured time per request of each mesh (it runs requests back to back);
      the same mix served in the ``compare`` precision as well ('mixed' = FP32 face
      arithmetic with FP64 state, stages and adjoints);
    * latency: Poisson arrivals swept over lambda = 1-200 req/s, min(n_mix, max(8, 6 s x
      lambda)) requests per rate, p50/p99 from arrival to result;
    * accuracy: the served sensitivity of one request per mesh against its plain FP64 one, in
      both served precisions."""
    from adfvm_gb300 import serving
    keys = SERVING_KEYS
    rng = np.random.default_rng(seed)
    ks = [keys[i] for i in rng.integers(0, len(keys), size=n_mix)]
    gaps = rng.exponential(1.0, size=n_mix)
    lib = serving.MeshLibrary()
    for k in keys:
        lib.get(k)
    # a server that stays up keeps its slots: contexts and graphs of the mix's meshes are made
    # before the timed serving, as the plain form's contexts are made before its timing
    srv = serving.SensitivityServer(precision=precision, device=local, k=10, nPrimal=100, library=lib,
                                     hbm_budget=120e9, max_slots=64)
    srv.warm(ks)
    srv.warm(keys)
    # plain FP64: one request per mesh, timed one by one
    # request payloads (initial state, source perturbation) are the clients' work: made before
    # the clocks of both forms start
    probe = serving.prepare([serving.Request(rid=1000 + i, key=k, seed=1000 + i, nPrimal=100)
                             for i, k in enumerate(keys)], lib)
    sp = serving.plain_one_at_a_time(probe, lib, device=local, nPrimal=100)
    t_plain = dict(zip(keys, sp['seconds_per_request']))
    plain_mix_s = sum(t_plain[k] for k in ks)
    # served: the same mix all at once, then the same probe requests for accuracy
    mix = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100, arrival=0.0)
                           for i, k in enumerate(ks)], lib)
    sm = srv.serve(mix, realtime=False)
    same = serving.prepare([serving.Request(rid=1000 + i, key=k, seed=1000 + i, nPrimal=100, arrival=0.0)
                            for i, k in enumerate(keys)], lib)
    srv.serve(same, realtime=False)
    rel = lambda rs: {a.key: float('%.3g' % (abs(a.sensitivity - b.sensitivity) / abs(b.sensitivity)))
                      for a, b in zip(rs, probe)}
    errs = rel(same)
    sweep = []
    for lam in lams:
        nr = int(min(n_mix, max(8, round(window_s * lam))))
        t = np.cumsum(gaps[:nr] / lam)
        reqs = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100, arrival=float(a))
                                for i, (k, a) in enumerate(zip(ks[:nr], t))], lib)
        st = srv.serve(reqs, realtime=True)
        sweep.append({'lambda': lam, 'requests': nr, 'req_per_s': round(st['req_per_s'], 3),
                      'p50_s': round(st['p50_s'], 4), 'p99_s': round(st['p99_s'], 4)})
    nslots = len(srv.slots)
    srv.close()
    other = None
    if compare and compare != precision:
        # the same mix and probes served in the comparison precision
        s32 = serving.SensitivityServer(precision=compare, device=local, k=10, nPrimal=100, library=lib,
                                        hbm_budget=120e9, max_slots=64)
        s32.warm(ks)
        s32.warm(keys)
        mix32 = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100, arrival=0.0)
                                 for i, k in enumerate(ks)], lib)
        sm32 = s32.serve(mix32, realtime=False)
        same32 = serving.prepare([serving.Request(rid=1000 + i, key=k, seed=1000 + i, nPrimal=100, arrival=0.0)
                                  for i, k in enumerate(keys)], lib)
        s32.serve(same32, realtime=False)
        e32 = rel(same32)
        other = {'precision': compare, 'served_req_per_s': round(n_mix / sm32['elapsed_s'], 3),
                 'max_rel_err_vs_fp64': max(e32.values()), 'rel_err_by_mesh': e32}
        s32.close()
    # the batching engine alone: the same mix served in FP64 against the plain FP64 form
    s64 = serving.SensitivityServer(precision='fp64', device=local, k=10, nPrimal=100, library=lib,
                                    hbm_budget=160e9, max_slots=64)
    # one slot per mesh first (an FP64 box96 slot, with its ten face tapes, is 47 GB), then more
    # slots of the mix's meshes while the budget allows
    s64.warm(sorted(set(ks)))
    s64.warm(ks)
    mix64 = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100, arrival=0.0)
                             for i, k in enumerate(ks)], lib)
    sm64 = s64.serve(mix64, realtime=False)
    s64.close()
    served_rate = n_mix / sm['elapsed_s']
    plain_rate = n_mix / plain_mix_s
    fp64_rate = n_mix / sm64['elapsed_s']
    return {'precision': precision, 'mix_requests': n_mix, 'served_req_per_s': round(served_rate, 3),
            'plain_fp64_req_per_s': round(plain_rate, 3), 'speedup_vs_plain': round(served_rate / plain_rate, 2),
            'served_fp64_req_per_s': round(fp64_rate, 3),
            'batching_gain_fp64': round(fp64_rate / plain_rate, 2),
            'small_class': small_class_bench(local, lib, batch={k: 4 for k in SMALL_KEYS}, cell_ns=cell_ns),
            'plain_seconds_per_request': {k: round(v, 4) for k, v in t_plain.items()},
            'latency_sweep': sweep, 'max_rel_err_vs_fp64': max(errs.values()), 'rel_err_by_mesh': errs,
            'compare': other, 'slots': nslots, 'meshes': keys,
            'steps_per_request': '100 primal + 100 adjoint (checkpoints every 10)'}


SMALL_KEYS = ['box16', 'box24', 'box32', 'cyl64x32']


def small_class_bench(local, lib, n_req=48, seed=6, precision='fp32', batch=None, cell_ns=None):
    """The small meshes of the serving mix, where launch and latency costs weigh most: n_req
    requests drawn from box16/24/32 and cyl64x32 served together, against the GPU time the same
    requests' graphs take replayed one request after another on one stream (CUDA events, no
    server and no overlap). served / sequential < 1 is what the overlap of requests on the GPU
    buys; close to 1 would leave room for a single ragged launch over all requests."""
    import torch
    from adfvm_gb300 import serving
    rng = np.random.default_rng(seed)
    ks = [SMALL_KEYS[i] for i in rng.integers(0, len(SMALL_KEYS), size=n_req)]
    srv = serving.SensitivityServer(precision=precision, device=local, k=10, nPrimal=100, library=lib,
                                    hbm_budget=60e9, max_slots=64)
    srv.warm(ks)
    reqs = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100) for i, k in enumerate(ks)], lib)
    st = srv.serve(reqs, realtime=False)
    batched = None
    if batch:
        # the same requests through batched slots: up to K requests on one mesh a launch
        sb = serving.SensitivityServer(precision=precision, device=local, k=10, nPrimal=100, library=lib,
                                       hbm_budget=60e9, max_slots=64, batch=batch)
        sb.warm([k for k in SMALL_KEYS for _ in range(-(-ks.count(k) // batch.get(k, 1)))])
        rb = serving.prepare([serving.Request(rid=i, key=k, seed=i, nPrimal=100) for i, k in enumerate(ks)], lib)
        stb = sb.serve(rb, realtime=False)
        worst = max(abs(a.sensitivity - b.sensitivity) / abs(b.sensitivity) for a, b in zip(rb, reqs))
        batched = {'batch': batch, 'served_s': round(stb['elapsed_s'], 4),
                   'served_req_per_s': round(n_req / stb['elapsed_s'], 2), 'slots': len(sb.slots),
                   'max_rel_diff_vs_unbatched': float('%.3g' % worst)}
        sb.close()
    # one request's graph replays per mesh, alone on one slot's stream
    per_key = {}
    for key in SMALL_KEYS:
        slot = next(s for s in srv.slots if s.key == key)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(slot.stream):          # a graph replays on the current stream
            e0.record(slot.stream)
            for _ in range(slot.nck):
                slot.graphs[0].replay()
            for _ in range(slot.nck):
                slot.graphs[1].replay()
                slot.graphs[2].replay()
            e1.record(slot.stream)
        torch.cuda.synchronize()
        per_key[key] = e0.elapsed_time(e1) / 1e3
    srv.close()
    seq = sum(per_key[k] for k in ks)
    # the kernel-time bound: the requests' cells at the workload box's cost per cell of two
    # primal steps (run and recompute) and one adjoint step, times the 100 steps
    bound = None
    if cell_ns:
        bound = sum(lib.get(k).mesh.nInternalCells for k in ks) * 100 * cell_ns * 1e-9
    return {'requests': n_req, 'meshes': SMALL_KEYS, 'precision': precision,
            'kernel_time_bound_s': None if bound is None else round(bound, 4),
            'bound_over_served': None if bound is None else round(bound / st['elapsed_s'], 3),
            'served_s': round(st['elapsed_s'], 4), 'served_req_per_s': round(n_req / st['elapsed_s'], 2),
            'sequential_graph_s': round(seq, 4), 'served_over_sequential': round(st['elapsed_s'] / seq, 3),
            'graph_s_per_request': {k: round(v, 5) for k, v in per_key.items()}, 'batched': batched}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    base = cpu_baseline(args, threads, seconds=max(2.0, min(10.0, 0.5 * (args.steps + args.warmup))))
    line = {'impl': 'reference', 'metric': METRIC, 'value': base['value'], 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            # the workload described as the GPU arm describes it (same mesh, same counts); the
            # sample the CPU timed is in cpu_baseline.sample
            'config': dict(base.pop('config'), parallelism='host cores (%d threads)' % threads),
            'cpu_baseline': base,
            'reference_python': reference_python(),
            'e2e': {'value': base['value'], 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours')
    ap.add_argument('--workload', default='box128')
    ap.add_argument('--precision', default='fp64')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--serving', type=int, default=1, help='1: add the serving measurement to the line')
    ap.add_argument('--tape', type=int, default=1,
                    help='1: the primal steps keep their face tapes for the adjoint steps (afvm_primal_step_tape)')
    ap.add_argument('--study', default='', help="'precision': the FP32-vs-FP64 cylinder study (own JSON line)")
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)
    if args.study == 'precision':
        from adfvm_gb300.studies import precision_study
        print(json.dumps({'study': 'precision', **precision_study()}))
        return 0

    import torch
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    torch.cuda.set_device(local)

    case = make_case(args.workload)
    mesh = case.build_mesh()
    clocks = ClockSampler(local)
    m64 = measure(case, args.precision, args, local, dist, world, clocks)
    m32 = measure(case, 'fp32', args, local, dist, world, None) if args.precision == 'fp64' else None
    mmx = measure(case, 'mixed', args, local, dist, world, None) if args.precision == 'fp64' else None
    clk = m64.pop('clocks')
    nIC = mesh.nInternalCells
    line = {'metric': METRIC, 'value': m64['value'], 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': m64['ms_per_step'], 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64' if args.precision == 'fp64' else 'f32',
            'data': 'synthetic',
            'config': dict(describe(case, args.precision),
                           l2='inputs larger than L2: %.2f GB device working set' % (m64['device_bytes'] / 1e9),
                           parallelism='replicas' if world > 1 else 'single GPU',
                           step='one SSP-RK3 primal step plus its adjoint step (value = cells x steps / '
                                '(primal + adjoint time)); the primal steps keep their RK stage states and '
                                'tapes (each stage\'s cell records%s) and the adjoint steps walk them backwards '
                                'as a sweep does; primal and adjoint also reported alone'
                                % (', FP64 face tapes' if m64['tape'] else ''),
                           tape=bool(m64['tape'])),
            'primal': m64['primal'], 'adjoint': m64['adjoint'],
            'roofline': m64['roofline'], 'step_model': m64['step_model'], 'kernels': m64['kernels'],
            'adjoint_kernels': m64['adjoint_kernels'], 'gpu_launches': m64['gpu_launches'],
            'e2e': m64['e2e'], 'clocks': clk}
    if mmx is not None:
        line['mixed'] = {k: mmx[k] for k in ('value', 'ms_per_step', 'primal', 'adjoint', 'kernels', 'adjoint_kernels')}
    if m32 is not None:
        m32.pop('clocks', None)
        line['fp32'] = {k: m32[k] for k in ('value', 'ms_per_step', 'primal', 'adjoint', 'roofline', 'step_model',
                                            'kernels', 'adjoint_kernels', 'e2e')}
    if args.serving and rank == 0:
        cell_ns = None
        if m32 is not None:
            cell_ns = (2 * m32['primal']['ms_per_step'] + m32['adjoint']['ms_per_step']) * 1e6 / nIC
        line['serving'] = serving_bench(local, cell_ns=cell_ns)
    if rank == 0 and args.serving:
        # FP32 / mixed against FP64 on the cylinder over 2000 steps (adfvm_gb300/studies.py)
        from adfvm_gb300.studies import precision_study
        line['precision_study'] = precision_study(device=local)
    if rank == 0:
        line['mesh_build'] = mesh_build_timing(case, local)
        if case.name.startswith('box'):
            line['mesh_reorder'] = reorder_timing(int(case.name[3:]), local)
    from adfvm_gb300 import _lib
    line['fma_peak_tflops'] = {'fp64': round(_lib.fma_peak(local, True), 2), 'fp32': round(_lib.fma_peak(local, False), 2)}
    top, avg_s, nF = m64.pop('_top')
    if args.precision == 'fp64' and top in MEASURED_FP64_INST:
        # the FP64 kernels are bound by the FP64 pipe, not HBM: counted FP64 instructions per
        # face (ncu) x faces / the launch's CUDA-event time, against the measured FMA peak
        da, dm, df = MEASURED_FP64_INST[top]
        flops = (da + dm + 2 * df) * nF
        fpk = line['fma_peak_tflops']['fp64']
        ach = flops / avg_s / 1e12
        line['compute_roofline'] = {
            'bound': 'fp64', 'kernel': top, 'achieved': round(ach, 3), 'peak': fpk, 'unit': 'TFLOP/s',
            'frac': round(ach / fpk, 4), 'flops_per_face': round(da + dm + 2 * df, 1),
            'issue_frac': round((da + dm + df) * nF / avg_s / (fpk * 1e12 / 2), 4),
            'pipe_issue_frac': round(MEASURED_FP64_PIPE_INST[top] * nF / avg_s / (fpk * 1e12 / 2), 4),
            'peak_source': 'afvm_fma_peak (a DFMA loop on this GPU, FMA = 2 flops)',
            'note': 'issue_frac counts DADD/DMUL/DFMA as one FP64 pipe issue each; pipe_issue_frac '
                    'every instruction the FP64 pipe issued (ncu), against the same issue rate'}
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(args, os.cpu_count() or 1)
        cb.pop('config', None)
        line['cpu_baseline'] = cb
        # the GPU's speed-up on the same mesh, FP64 both: primal and adjoint alone and together
        line['vs_cpu_baseline'] = {'primal': round(m64['primal']['value'] / cb['primal'], 2),
                                   'adjoint': round(m64['adjoint']['value'] / cb['adjoint'], 2),
                                   'primal_adjoint': round(m64['value'] / cb['value'], 2),
                                   'e2e': round(m64['e2e']['value'] / cb['value'], 2)}
        rp = reference_python()
        if rp is not None:
            line['reference_python'] = rp
            line['vs_reference_python'] = {'primal': round(m64['primal']['value'] / rp['value'], 1)}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == '__main__':
    sys.exit(main())
