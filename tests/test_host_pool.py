"""RCF.download's host arrays: an array the context returned before is reused only when
nothing else refers to it (its reference count shows only the context's pool) - results the
caller keeps, directly or through a view, are never overwritten."""
import numpy as np

from adfvm_gb300.solver import RCF


class _Ctx(object):
    pass


def test_only_unreferenced_arrays_are_reused():
    f = _Ctx()
    a = RCF._host_array(f, (5, 3), np.float64)
    b = RCF._host_array(f, (5, 3), np.float64)
    assert a is not b                                    # both still held here
    ida = id(a)
    del a
    c = RCF._host_array(f, (5, 3), np.float64)
    assert id(c) == ida                                  # the released one comes back
    view = c[:, 1]
    idc = id(c)
    del c
    d = RCF._host_array(f, (5, 3), np.float64)
    assert id(d) != idc and view.base is not None        # a view keeps its base out of reuse
    e = RCF._host_array(f, (5, 3), np.float32)
    assert e.dtype == np.float32 and e.shape == (5, 3)   # shape and type must match
    held = [RCF._host_array(f, (2,), np.float64) for _ in range(20)]
    assert len({id(x) for x in held}) == 20              # the pool is bounded, new arrays beyond it
    assert len(f._hostPool) <= 12
