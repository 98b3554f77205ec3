"""The FP64 reciprocal and reciprocal square root of the GPU kernels (rcp_nr, rsqrt_nr,
adfvm_gb300/csrc/physics.cuh): an FP32 hardware seed refined by one third-order correction
(the series of 1/(1 - e) and (1 - e)^(-1/2) in the seed's residual e) in place of IEEE
division and square root on every FP64 path.

Checked on the GPU over arguments 2^[-130, 130] (random mantissas, both signs), at the
2^-120 / 2^121 switch-over exponents, and on 0, -0, subnormals, inf, -inf, NaN and the
largest and smallest normal numbers:
* inside 2^[-120, 121): within 0.51 units in the last place of the exactly rounded 1/x and
  1/sqrt(x) (references in numpy long double, which carries more bits than double);
* outside that range, for 0, subnormals, inf and NaN, and for negative arguments of
  rsqrt_nr: bitwise the IEEE operations 1.0/x and 1.0/sqrt(x).
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, 'tests', 'native', 'rcp_probe.cu')


@pytest.fixture(scope='module')
def probe():
    out = os.path.join(tempfile.mkdtemp(prefix='rcp_probe_'), 'rcp_probe.so')
    subprocess.check_call([os.environ.get('NVCC', 'nvcc'), '-gencode', 'arch=compute_103a,code=sm_103a', '-O3',
                           '-std=c++17', '-shared', '-Xcompiler', '-fPIC', '-I' + os.path.join(ROOT, 'include'),
                           '-I' + os.path.join(ROOT, 'adfvm_gb300', 'csrc'), SRC, '-o', out])
    lib = C.CDLL(out)
    dp = C.POINTER(C.c_double)
    lib.rcp_probe.argtypes = [dp, dp, dp, C.c_int]

    def run(x):
        x = np.ascontiguousarray(x, np.float64)
        r = np.empty_like(x)
        rs = np.empty_like(x)
        st = lib.rcp_probe(x.ctypes.data_as(dp), r.ctypes.data_as(dp), rs.ctypes.data_as(dp), len(x))
        assert st == 0, st
        return r, rs
    return run


def _inside(x):
    e = np.frexp(np.abs(x))[1] - 1          # unbiased exponent: |x| = m 2^e, m in [1, 2)
    return np.isfinite(x) & (x != 0) & (e >= -120) & (e <= 120)


def _ulps(got, exact):
    """|got - exact| in units of the last place of the double nearest to the exact value."""
    ref = exact.astype(np.float64)
    return (np.abs(got.astype(np.longdouble) - exact) / np.spacing(np.abs(ref)).astype(np.longdouble)).astype(np.float64)


def _arguments():
    rng = np.random.default_rng(11)
    e = rng.integers(-130, 131, size=200000)
    m = rng.uniform(1.0, 2.0, size=e.size)
    x = np.ldexp(m, e) * np.where(rng.random(e.size) < 0.5, -1.0, 1.0)
    edges = []
    for k in (-121, -120, -119, 119, 120, 121, 122):
        for mm in (1.0, np.nextafter(1.0, 2.0), 1.5, np.nextafter(2.0, 1.0)):
            edges += [np.ldexp(mm, k), -np.ldexp(mm, k)]
    tiny = np.finfo(np.float64).tiny
    special = [0.0, -0.0, np.inf, -np.inf, np.nan, tiny, -tiny, tiny / 3, 5e-324, -5e-324,
               np.finfo(np.float64).max, -np.finfo(np.float64).max, 1.0, -1.0, 2.0, 0.5, 3.0]
    return np.concatenate([x, np.array(edges), np.array(special)])


def test_rcp_within_one_ulp_and_ieee_outside(probe):
    x = _arguments()
    r, _ = probe(x)
    ins = _inside(x)
    exact = np.longdouble(1) / x[ins].astype(np.longdouble)
    u = _ulps(r[ins], exact)
    assert u.max() <= 0.51, 'rcp_nr: max error %.3f ulp at x = %r' % (u.max(), x[ins][np.argmax(u)])
    with np.errstate(divide='ignore', over='ignore', invalid='ignore'):
        ieee = 1.0 / x[~ins]
    same = (r[~ins].view(np.int64) == ieee.view(np.int64)) | (np.isnan(r[~ins]) & np.isnan(ieee))
    assert same.all(), 'rcp_nr differs from 1.0/x at %r' % (x[~ins][~same][:5],)
    print('rcp_nr: max %.3f ulp over %d arguments inside 2^[-120, 121)' % (u.max(), ins.sum()))


def test_rsqrt_within_one_ulp_and_ieee_outside(probe):
    x = _arguments()
    _, rs = probe(x)
    ins = _inside(x) & (x > 0)
    exact = np.longdouble(1) / np.sqrt(x[ins].astype(np.longdouble))
    u = _ulps(rs[ins], exact)
    assert u.max() <= 0.51, 'rsqrt_nr: max error %.3f ulp at x = %r' % (u.max(), x[ins][np.argmax(u)])
    with np.errstate(divide='ignore', over='ignore', invalid='ignore'):
        ieee = 1.0 / np.sqrt(x[~ins])
    same = (rs[~ins].view(np.int64) == ieee.view(np.int64)) | (np.isnan(rs[~ins]) & np.isnan(ieee))
    assert same.all(), 'rsqrt_nr differs from 1.0/sqrt(x) at %r' % (x[~ins][~same][:5],)
    assert np.isnan(rs[x < 0]).all()
    print('rsqrt_nr: max %.3f ulp over %d positive arguments inside 2^[-120, 121)' % (u.max(), ins.sum()))
