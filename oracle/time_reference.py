"""Time the reference's own primal path on CPU (test infrastructure; runs where the reference
checkout is).

The reference's ``Solver.run`` (adFVM/solver.py:210-411) in forward mode, its RCF step
(adFVM/density.py:339-414) evaluated through the NumPy adpy stand-in of ``oracle/refshim`` and
its own cmesh (``oracle/refrun.py``), on the periodic jittered boxes 16^3 and 32^3 of the
throughput recipe. The machines that run the benchmark have no reference checkout, so the
numbers are measured here and written to ``oracle/reference_timing.json``, which ``bench.py``
reports as ``reference_python`` beside its CPU baseline (the C/OpenMP restatement, timed where
the benchmark runs). The reference's
adjoint runs through adpy's reverse mode, which the checkout does not contain: only the primal
is timed.

    python -m oracle.time_reference
"""
import datetime
import json
import os
import platform
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

OUT = os.path.join(HERE, 'reference_timing.json')


def cpu_model():
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                if line.lower().startswith('model name'):
                    return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def time_box(n, steps=5, warmup=1):
    from adfvm_gb300 import cases
    from oracle import refrun
    from tests.golden.make_golden import reference_config
    case = cases.box(n, objective='kinetic_energy')
    with tempfile.TemporaryDirectory() as d:
        cfg, hook = reference_config(case)
        rcf, cons = refrun.make_rcf(case.meshData, d, case.bc, case.U, case.T, case.p, before_compile=hook, **cfg)
        refrun.run_forward(rcf, warmup, case.dt)
        t0 = time.perf_counter()
        refrun.run_forward(rcf, steps, case.dt)
        el = time.perf_counter() - t0
    cells = case.build_mesh().nInternalCells
    return {'workload': 'box%d: %d cells, Roe, SSP-RK3, Sutherland viscosity, FP64' % (n, cells),
            'cells': cells, 'steps': steps, 'seconds': round(el, 3),
            'primal_mcell_steps_per_s': round(cells * steps / el / 1e6, 5)}


def main():
    from oracle import refrun
    refrun.load()
    out = {'path': "the reference's Solver.run (forward mode) through the NumPy adpy stand-in and its own "
                   "cmesh", 'metric': 'primal Mcell-steps/s', 'host': cpu_model(), 'cores': os.cpu_count(),
           'threads': 'NumPy evaluates the adpy graph, mostly on one thread',
           'measured_utc': datetime.datetime.now(datetime.timezone.utc).strftime('%Y-%m-%d'),
           'cases': [time_box(16), time_box(32, steps=3)]}
    with open(OUT, 'w') as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == '__main__':
    main()
