"""Build recipe for the native library ``adfvm_gb300/libafvm.so``.

Host C++ (mesh geometry) is compiled by g++ without floating-point contraction; the CUDA
translation units are compiled by nvcc for sm_103a only. Objects are built in parallel and
linked into one shared library that the package loads with ctypes.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, 'include')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libafvm.so')

NVCC = os.environ.get('NVCC', 'nvcc')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
HOST_FLAGS = ['-O3', '-fPIC', '-fopenmp', '-ffp-contract=off', '-std=c++17']
NVCC_FLAGS = ARCH + ['-O3', '-lineinfo', '-std=c++17', '--expt-relaxed-constexpr',
                     '-Xcompiler', '-fPIC,-ffp-contract=off,-fopenmp', '-I' + INCLUDE, '-I' + CSRC]
# the device mesh builder rounds every product and sum as the host builder does
PER_FILE_FLAGS = {'geometry_dev.cu': ['-fmad=false']}


def _sources():
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith('.cpp'))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith('.cu'))
    return cpp, cu


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh', '.hpp'))]
    return hs


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cpp, cu = _sources()
    headers = _headers()
    jobs = []
    objs = []
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + '.o')
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append(['g++'] + HOST_FLAGS + ['-I' + INCLUDE, '-I' + CSRC, '-c', src, '-o', obj])
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + '.o')
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + PER_FILE_FLAGS.get(f, []) + ['-c', src, '-o', obj])

    def run(cmd):
        if verbose:
            print(' '.join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('compile failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or force or _newer(LIB, objs):
        run([NVCC] + ARCH + ['-shared', '-o', LIB] + objs + ['-Xcompiler', '-fopenmp', '-lgomp', '-lcudart'])
    return LIB


if __name__ == '__main__':
    build(verbose='-v' in sys.argv, force='-f' in sys.argv)
    print(LIB)
