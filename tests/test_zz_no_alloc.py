"""The allocation-free sensitivity entry point (afvm_sensitivity_noalloc).

It exists for callers that may not allocate device memory: an application that gives this
library a fixed share of the GPU up front and makes every allocation itself, or a plug-in
loaded into a host program whose memory pool it must not touch. Its scratch is a static
device array of the library. This file is collected last on purpose: if it fails, a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from adfvm_gb300 import _lib as L
from adfvm_gb300 import cases
from adfvm_gb300.solver import RCF

pytestmark = pytest.mark.gpu

MAX_ARRAYS = 16   # AFVM_SENSITIVITY_NOALLOC_MAX_ARRAYS in include/afvm.h


def _arrays(k, seed):
    rng = np.random.default_rng(seed)
    sizes = [int(s) for s in rng.integers(1, 400000, size=k)]
    g = [torch.as_tensor(rng.normal(size=n)).cuda() for n in sizes]
    p = [torch.as_tensor(rng.normal(size=n)).cuda() for n in sizes]
    return g, p


def _noalloc(g, p, k=None, device=None):
    k = len(g) if k is None else k
    m = max(1, len(g))
    ga = (L._d * m)(*[C.cast(C.c_void_p(t.data_ptr()), L._d) for t in g])
    pa = (L._d * m)(*[C.cast(C.c_void_p(t.data_ptr()), L._d) for t in p])
    na = (C.c_int64 * m)(*[t.numel() for t in g])
    out = C.c_double(float('nan'))
    stream = torch.cuda.current_stream().cuda_stream
    dev = torch.cuda.current_device() if device is None else device
    st = L.lib().afvm_sensitivity_noalloc(dev, k, ga, pa, na, C.byref(out),
                                          C.c_void_p(stream))
    return st, out.value


def test_noalloc_matches_allocating_entry_point_twice():
    case = cases.box(6, objective='kinetic_energy')
    rcf = RCF(case.build_mesh(), case.bc, objective=case.objective, **case.config)
    g, p = _arrays(5, 3)
    ref = rcf.sensitivity(g, p)
    scale = sum(float((a * b).abs().sum()) for a, b in zip(g, p))
    st1, v1 = _noalloc(g, p)
    assert st1 == L.AFVM_OK
    free_before = torch.cuda.mem_get_info()[0]
    st2, v2 = _noalloc(g, p)
    free_after = torch.cuda.mem_get_info()[0]
    assert st2 == L.AFVM_OK
    # within the tolerance of the sensitivity test (1e-12 of the sum of |terms|)
    assert abs(v1 - ref) <= 1e-12 * scale
    assert abs(v2 - ref) <= 1e-12 * scale
    assert v1 == v2                       # same kernels, same fixed reduction order
    assert free_after == free_before      # the call allocated no device memory
    # a different call in between leaves nothing behind that changes the next result
    g2, p2 = _arrays(MAX_ARRAYS, 4)
    st3, v3 = _noalloc(g2, p2)
    assert st3 == L.AFVM_OK
    assert abs(v3 - rcf.sensitivity(g2, p2)) <= 1e-12 * sum(float((a * b).abs().sum()) for a, b in zip(g2, p2))
    st4, v4 = _noalloc(g, p)
    assert st4 == L.AFVM_OK and v4 == v1


def test_noalloc_rejects_more_arrays_than_its_scratch_holds():
    g, p = _arrays(MAX_ARRAYS + 1, 5)
    st, v = _noalloc(g, p)
    assert st == L.AFVM_ERR_BAD_ARG


def test_noalloc_rejects_no_arrays_and_unknown_devices():
    g, p = _arrays(2, 6)
    assert _noalloc(g, p, k=0)[0] == L.AFVM_ERR_BAD_ARG
    assert _noalloc(g, p, k=-1)[0] == L.AFVM_ERR_BAD_ARG
    assert _noalloc(g, p, device=-1)[0] == L.AFVM_ERR_BAD_ARG
    assert _noalloc(g, p, device=torch.cuda.device_count())[0] == L.AFVM_ERR_BAD_ARG
    # a rejected call leaves the next one unaffected
    st, v = _noalloc(g, p)
    assert st == L.AFVM_OK
    ref = sum(float((a * b).sum()) for a, b in zip(g, p))
    assert abs(v - ref) <= 1e-12 * sum(float((a * b).abs().sum()) for a, b in zip(g, p))


def test_noalloc_rejects_arrays_that_are_not_on_the_device():
    g, p = _arrays(2, 7)
    host = np.random.default_rng(8).normal(size=g[1].numel())
    k = 2
    ga = (L._d * k)(C.cast(C.c_void_p(g[0].data_ptr()), L._d), host.ctypes.data_as(L._d))
    pa = (L._d * k)(*[C.cast(C.c_void_p(t.data_ptr()), L._d) for t in p])
    na = (C.c_int64 * k)(*[t.numel() for t in g])
    out = C.c_double(float('nan'))
    st = L.lib().afvm_sensitivity_noalloc(torch.cuda.current_device(), k, ga, pa, na, C.byref(out),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == L.AFVM_ERR_BAD_ARG
    # the next valid call is unaffected
    st, v = _noalloc(g, p)
    assert st == L.AFVM_OK
    ref = sum(float((a * b).sum()) for a, b in zip(g, p))
    assert abs(v - ref) <= 1e-12 * sum(float((a * b).abs().sum()) for a, b in zip(g, p))
