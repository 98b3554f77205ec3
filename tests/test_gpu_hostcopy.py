"""Host <-> device field copies (afvm_copy_to_device / afvm_copy_to_host) and the reference-facing
maps that use them.

The copies are exact for equal types and round to nearest for FP64 -> FP32 (numpy's astype);
FP32 -> FP64 is exact. Adjoint.map must return the same values, bit for bit, as the device-side
adjoint step it wraps, in every precision.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from adfvm_gb300 import _lib as L
from adfvm_gb300.adjoint import Adjoint
from adfvm_gb300.solver import RCF
from tests import golden_cases as G

pytestmark = pytest.mark.gpu

# 8 MB staging chunks: sizes below, at and across chunk boundaries for both element sizes
SIZES = [0, 1, 7, 1 << 20, (1 << 20) + 3, (2 << 20) + 5, 5 * (1 << 20) + 11]


def _host(n, dtype, pinned, seed):
    v = np.random.default_rng(seed).standard_normal(n) * 1e3
    if pinned:
        a = torch.empty(n, dtype=torch.float64 if dtype == np.float64 else torch.float32, pin_memory=True).numpy()
        a[...] = v
        return a
    return v.astype(dtype)


@pytest.mark.parametrize('pinned', [False, True])
@pytest.mark.parametrize('host_t,dev_t', [(np.float64, torch.float64), (np.float32, torch.float32),
                                          (np.float64, torch.float32), (np.float32, torch.float64)])
def test_round_trip(host_t, dev_t, pinned):
    for i, n in enumerate(SIZES):
        a = _host(n, host_t, pinned, i)
        t = L.to_device(a, torch.empty(n, dtype=dev_t, device='cuda:0'))
        want = torch.from_numpy(a.astype(np.float64 if dev_t == torch.float64 else np.float32))
        assert torch.equal(t.cpu(), want), (n, host_t, dev_t)
        back = np.full(n, np.nan, host_t)
        L.to_host(t, back)
        assert np.array_equal(back, want.numpy().astype(host_t)), (n, host_t, dev_t)


def test_copies_are_stream_ordered():
    """A copy on a side stream sees the kernels queued before it on that stream."""
    n = (3 << 20) + 1
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        t = torch.zeros(n, dtype=torch.float64, device='cuda:0')
        for _ in range(20):
            t += 1.0
        out = np.empty(n, np.float32)
        L.to_host(t, out)
    assert (out == 20.0).all()


def test_bad_arguments():
    lib = L.lib()
    assert lib.afvm_copy_to_device(0, None, 8, None, 8, 0, None) == L.AFVM_OK
    assert lib.afvm_copy_to_device(0, None, 8, None, 8, 5, None) == L.AFVM_ERR_BAD_ARG
    t = torch.empty(4, dtype=torch.float64, device='cuda:0')
    a = np.zeros(4)
    dp, hp = C.c_void_p(t.data_ptr()), C.c_void_p(a.ctypes.data)
    assert lib.afvm_copy_to_device(0, dp, 2, hp, 8, 4, None) == L.AFVM_ERR_BAD_ARG
    assert lib.afvm_copy_to_host(0, hp, 8, dp, 8, -1, None) == L.AFVM_ERR_BAD_ARG
    assert lib.afvm_copy_to_host(-1, hp, 8, dp, 8, 4, None) == L.AFVM_ERR_BAD_ARG
    with pytest.raises(ValueError):
        L.to_device(np.zeros(3), t)


@pytest.mark.parametrize('precision', ['fp64', 'fp32', 'mixed'])
def test_adjoint_map_matches_adjoint_step(precision):
    """Adjoint.map runs the forward with its stages and tape kept and then the taped adjoint
    step: bit for bit that device path; without room for the tape (forced here), bit for bit
    the adjoint step that recomputes its forward. The two agree within the taped adjoint's
    tolerances (FMA contraction differs between the kernels)."""
    case, g = G.load('cyl32x16')
    rcf = RCF(case.build_mesh(), case.bc, objective=case.objective, precision=precision, **case.config)
    n = rcf.mesh.nInternalCells
    x = [np.asarray(g['rho_init']).reshape(-1, 1), np.asarray(g['rhoU_init']).reshape(-1, 3),
         np.asarray(g['rhoE_init']).reshape(-1, 1)]
    dt = float(g['dt0'])
    rng = np.random.default_rng(3)
    seeds = [rng.standard_normal((n, d)) * 1e-3 for d in (1, 3, 1)]
    inputs = rcf.mapInputs(*x, dt) + seeds + [np.zeros((1, 1)), np.ones((1, 1)), np.zeros((1, 1))]
    adj = Adjoint(rcf)
    got = adj.map(*inputs)
    assert adj._fwd
    adj._fwd = False
    got_untaped = adj.map(*inputs)
    td = torch.float64 if rcf.dtype == np.float64 else torch.float32
    xd = [torch.as_tensor(a.astype(rcf.dtype), device='cuda:0') for a in x]
    sd = [torch.as_tensor(a.astype(rcf.dtype), device='cuda:0') for a in seeds]
    zero = [torch.zeros((n, d), dtype=td, device='cuda:0') for d in (1, 3, 1)]
    st, tp = rcf.stage_buffer(), rcf.tape_buffer()
    rcf.step(xd[0], xd[1], xd[2], dt, S=zero, stages=st, tape=tp)
    r = rcf.adjoint_step(xd[0], xd[1], xd[2], dt, sd, obja=1.0, S=zero, stages=st, tape=tp)
    want = [t.double().cpu().numpy() for t in list(r[:3]) + list(r[3])]
    r0 = rcf.adjoint_step(xd[0], xd[1], xd[2], dt, sd, obja=1.0, S=zero)
    want_untaped = [t.double().cpu().numpy() for t in list(r0[:3]) + list(r0[3])]
    tol = 1e-5 if precision == 'fp32' else (1e-6 if precision == 'mixed' else 1e-13)
    assert len(got) == len(want) == len(got_untaped) == 6
    for a, b, c, d in zip(got, want, got_untaped, want_untaped):
        assert a.dtype == np.float64 and a.shape == b.shape
        assert np.array_equal(a, b)
        assert np.array_equal(c, d)
        assert G.rel_err(a, c) <= tol
    # the primal map (which keeps its stages for the adjoint map) returns the device step's state
    out = rcf.map(*rcf.mapInputs(*x, dt))
    y = rcf.step(xd[0], xd[1], xd[2], dt, S=zero)
    for a, b in zip(out[:3], y[:3]):
        assert a.dtype == rcf.dtype and np.array_equal(a, b.cpu().numpy())
