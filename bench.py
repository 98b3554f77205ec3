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
# es and int32 indices; see DESIGN.md "Algorithmic bytes"
def algorithmic_bytes(kernel, nIC, nIF, nF, nG, es):
    REC, FREC = 20, 6
    if kernel == 'k_flux':
        # per face: own+nbr (8), normals 3, deltas 1, deltasUnit 3, linearWeights 2,
        # quadraticWeights 6 -> 15 values, flux record write 6; cell records read once
        return nF * (8 + 15 * es + FREC * es) + (nIC + nG) * REC * es
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
    return 0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch from an ncu capture of
# the 64^3 box (798,720 faces, 262,144 cells; profiles/), scaled to a launch of the benchmarked
# mesh by its number of faces (the kernel's traffic grows in proportion to the faces)
MEASURED_TRAFFIC = {('k_flux', 8): (174.24e6, 798720)}


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


def make_case(workload):
    from adfvm_gb300 import cases
    if workload.startswith('box'):
        return cases.box(int(workload[3:]), objective='kinetic_energy')
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


def cpu_baseline(args, threads, case=None, seconds=10.0):
    """The oracle on the host cores, on a bounded sample of the workload: primal steps of the
    C/OpenMP FP64 restatement (oracle/c) on the workload's own mesh for ~`seconds`, and the
    adjoint step as torch autograd of the float64 oracle (the only CPU adjoint: the reference's
    adpy reverse mode is absent) on a 32^3 box of the same recipe. value = primal+adjoint
    Mcell-steps/s from the two per-cell-step times."""
    import torch
    from adfvm_gb300 import cases
    from oracle import torch_ref
    from oracle.c_ref import COracle
    os.environ.setdefault('OMP_NUM_THREADS', str(threads))
    torch.set_num_threads(threads)
    if case is None:
        case = make_case(args.workload)
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
    small = cases.box(32, objective='kinetic_energy')
    sm = small.build_mesh()
    prob = torch_ref.Problem(sm, small.bc, small.config, small.objective)
    xs = [torch.as_tensor(a) for a in cases.conservative(small)]
    seeds = [torch.ones_like(t) * 1e-3 for t in xs]
    torch_ref.vjp_step(prob, xs[0], xs[1], xs[2], small.dt, None, seeds)
    t0 = time.perf_counter()
    na = 0
    while time.perf_counter() - t0 < seconds and na < 50:
        torch_ref.vjp_step(prob, xs[0], xs[1], xs[2], small.dt, None, seeds)
        na += 1
    ta = (time.perf_counter() - t0) / (na * sm.nInternalCells)
    return {'value': 1.0 / (tp + ta) / 1e6, 'unit': UNIT, 'cores': threads, 'kind': 'port',
            'primal': round(1.0 / tp / 1e6, 4), 'adjoint': round(1.0 / ta / 1e6, 4),
            'sample': '%d FP64 primal steps of %s (%d cells) by the C/OpenMP oracle; %d adjoint steps of the '
                      '32^3 box (%d cells) by torch autograd of the float64 oracle' % (
                          steps, case.name, m.nInternalCells, na, sm.nInternalCells)}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    base = cpu_baseline(args, threads, seconds=max(2.0, min(10.0, 0.5 * (args.steps + args.warmup))))
    line = {'impl': 'reference', 'metric': METRIC, 'value': base['value'], 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': args.workload + ' (CPU sample, see cpu_baseline.sample), Roe, SSP-RK3, '
                                   'Sutherland viscosity, FP64'},
            'cpu_baseline': base,
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
                                '(primal + adjoint time)); primal and adjoint also reported alone'),
            'primal': m64['primal'], 'adjoint': m64['adjoint'],
            'roofline': m64['roofline'], 'kernels': m64['kernels'], 'adjoint_kernels': m64['adjoint_kernels'],
            'gpu_launches': m64['gpu_launches'],
            'e2e': m64['e2e'], 'clocks': clk}
    if m32 is not None:
        m32.pop('clocks', None)
        line['fp32'] = {k: m32[k] for k in ('value', 'ms_per_step', 'primal', 'adjoint', 'roofline', 'kernels',
                                            'adjoint_kernels', 'e2e')}
    if args.serving and rank == 0:
        line['serving'] = serving_bench(local)
    from adfvm_gb300 import _lib
    line['fma_peak_tflops'] = {'fp64': round(_lib.fma_peak(local, True), 2), 'fp32': round(_lib.fma_peak(local, False), 2)}
    if rank == 0 and not args.no_cpu_baseline:
        line['cpu_baseline'] = cpu_baseline(args, os.cpu_count() or 1, case=case)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == '__main__':
    sys.exit(main())
