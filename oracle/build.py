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
    oracle/c/reorder_oracle.c) and the host adjoint baseline (oracle/c/adjoint_host.cpp, which
    compiles the library's face VJP adfvm_gb300/csrc/face.cuh for the host) into
    oracle/_ref/liboracle.so."""
    os.makedirs(OUT, exist_ok=True)
    csrc = [os.path.join(HERE, 'c', f) for f in ('afvm_oracle.c', 'reorder_oracle.c')]
    cxx = os.path.join(HERE, 'c', 'adjoint_host.cpp')
    root = os.path.dirname(HERE)
    inc = ['-I' + os.path.join(HERE, 'c'), '-I' + os.path.join(root, 'adfvm_gb300', 'csrc'),
           '-I' + os.path.join(root, 'include')]
    deps = csrc + [cxx, os.path.join(HERE, 'c', 'afvm_oracle.h')] + \
        [os.path.join(root, 'adfvm_gb300', 'csrc', f) for f in ('face.cuh', 'physics.cuh')]
    if not all(os.path.exists(s) for s in deps):
        return None
    target = os.path.join(OUT, 'liboracle.so')
    if os.path.exists(target) and all(os.path.getmtime(target) > os.path.getmtime(s) for s in deps):
        return target
    objs = []
    for src in csrc:
        obj = os.path.join(OUT, os.path.basename(src) + '.o')
        _run(['gcc', '-O3', '-std=c11', '-fPIC', '-fopenmp', '-ffp-contract=off'] + inc + ['-c', src, '-o', obj])
        objs.append(obj)
    obj = os.path.join(OUT, 'adjoint_host.cpp.o')
    _run(['g++', '-O3', '-std=c++17', '-fPIC', '-fopenmp', '-ffp-contract=off'] + inc + ['-c', cxx, '-o', obj])
    objs.append(obj)
    _run(['g++', '-shared', '-fopenmp'] + objs + ['-o', target, '-lm'])
    return target


def build():
    return build_ref(), build_c()


if __name__ == '__main__':
    print(build())
