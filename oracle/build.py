"""Build recipes for the oracle (test infrastructure only).

* ``build_ref()`` compiles the reference's own mesh-builder sources, UNMODIFIED and where they
  lie (adFVM/cpp/cmesh.cpp and adFVM/cpp/mesh.cpp under the reference checkout), against the
  stand-in headers in oracle/refshim, into the Python extension ``oracle/_ref/cmesh``. It
  runs only where the reference checkout exists (``AFVM_REFERENCE`` or /root/reference).
* ``build_c()`` compiles the C restatements of the residual (oracle/c/afvm_oracle.c, also the
  timed CPU baseline) and of the cell renumbering (oracle/c/reorder_oracle.c) into
  ``oracle/_ref/liboracle.so``.
Both use -ffp-contract=off so that x86 and Arm give identical results.
"""
import os
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
REFERENCE = os.environ.get('AFVM_REFERENCE', '/root/reference')


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('oracle build failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))


def reference_available():
    return os.path.exists(os.path.join(REFERENCE, 'adFVM', 'cpp', 'cmesh.cpp'))


def build_ref():
    """Compile the reference mesh builder into oracle/_ref/cmesh<EXT_SUFFIX>."""
    if not reference_available():
        return None
    import numpy as np
    os.makedirs(OUT, exist_ok=True)
    cpp = os.path.join(REFERENCE, 'adFVM', 'cpp')
    target = os.path.join(OUT, 'cmesh' + sysconfig.get_config_var('EXT_SUFFIX'))
    srcs = [os.path.join(cpp, 'cmesh.cpp'), os.path.join(cpp, 'mesh.cpp')]
    shim = [os.path.join(HERE, 'refshim', f) for f in os.listdir(os.path.join(HERE, 'refshim'))]
    if os.path.exists(target) and all(os.path.getmtime(target) > os.path.getmtime(s) for s in srcs + shim):
        return target
    cmd = ['g++', '-O2', '-std=c++11', '-shared', '-fPIC', '-fopenmp', '-ffp-contract=off',
           '-UNDEBUG', '-w',
           '-I' + os.path.join(HERE, 'refshim'), '-I' + os.path.join(cpp, 'include'),
           '-I' + sysconfig.get_paths()['include'], '-I' + np.get_include()] + srcs + ['-o', target, '-lgomp']
    _run(cmd)
    return target


def build_c():
    """Compile the C restatements (the residual, oracle/c/afvm_oracle.c; the cell renumbering,
    oracle/c/reorder_oracle.c) into oracle/_ref/liboracle.so."""
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, 'c', f) for f in ('afvm_oracle.c', 'reorder_oracle.c')]
    if not all(os.path.exists(s) for s in srcs):
        return None
    target = os.path.join(OUT, 'liboracle.so')
    if os.path.exists(target) and all(os.path.getmtime(target) > os.path.getmtime(s) for s in srcs):
        return target
    _run(['gcc', '-O3', '-std=c11', '-shared', '-fPIC', '-fopenmp', '-ffp-contract=off'] + srcs + ['-o', target, '-lm'])
    return target


def build():
    return build_ref(), build_c()


if __name__ == '__main__':
    print(build())
