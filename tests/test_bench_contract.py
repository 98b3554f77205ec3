"""bench.py structure, checked on the host: every module-level name that a bench function calls
is defined (a missing one only shows on the GPU machine otherwise), and the reference arm prints
its JSON line with the keys the contract asks for."""
import ast
import builtins
import json
import os
import subprocess
import sys

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_called_names_are_defined():
    tree = ast.parse(open(os.path.join(ROOT, 'bench.py')).read())
    missing = []
    for fn in [n for n in tree.body if isinstance(n, ast.FunctionDef)]:
        local = {a.arg for a in fn.args.args} | {a.arg for a in fn.args.kwonlyargs}
        for node in ast.walk(fn):
            if isinstance(node, (ast.Name,)) and isinstance(node.ctx, ast.Store):
                local.add(node.id)
            elif isinstance(node, (ast.FunctionDef, ast.Import, ast.ImportFrom)):
                if isinstance(node, ast.FunctionDef):
                    local.add(node.name)
                else:
                    local |= {(a.asname or a.name).split('.')[0] for a in node.names}
            elif isinstance(node, ast.arg):
                local.add(node.arg)
        for node in ast.walk(fn):
            if isinstance(node, ast.Call) and isinstance(node.func, ast.Name):
                name = node.func.id
                if name not in local and not hasattr(bench, name) and not hasattr(builtins, name):
                    missing.append((fn.name, name))
    assert not missing, missing


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS='2')
    out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--workload', 'box16',
                          '--steps', '1', '--warmup', '0'], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ('impl', 'metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'higher_is_better', 'cpu_baseline',
              'e2e', 'config'):
        assert k in line, k
    assert line['impl'] == 'reference' and line['value'] > 0
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['cpu_baseline']['kind'] in ('port', 'reference')


def test_reference_python_fixture():
    """The reference's own primal timing (oracle/time_reference.py, measured where the reference
    checkout is) is read into the bench line's reference_python with where it was measured."""
    import bench
    rp = bench.reference_python()
    assert rp is not None
    assert rp['value'] > 0 and rp['unit'].startswith('primal')
    assert 'not on the benchmark machine' in rp['measured']
    assert set(rp['cases']) >= {'box16', 'box32'}
