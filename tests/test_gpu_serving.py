"""Continuous-batching sensitivity server: a request's result is the same alone and in a
mix; the served FP64 result equals the plain one-at-a-time computation; FP32 and mixed
(FP32 records and fluxes, FP64 state) are within their stated bounds of FP64."""
import numpy as np
import pytest

from adfvm_gb300 import serving

pytestmark = pytest.mark.gpu

KEYS = ['box8', 'cyl16x8', 'box6']


def _reqs(keys, seeds, nPrimal):
    return [serving.Request(rid=i, key=k, seed=s, nPrimal=nPrimal) for i, (k, s) in enumerate(zip(keys, seeds))]


def test_same_result_alone_and_in_the_mix():
    lib = serving.MeshLibrary()
    alone = _reqs(['box8'], [3], 8)
    srv = serving.SensitivityServer(precision='fp64', k=4, nPrimal=8, library=lib)
    srv.serve(alone, realtime=False)
    mix = _reqs(['cyl16x8', 'box8', 'box6', 'box8', 'cyl16x8'], [1, 3, 2, 4, 5], 8)
    srv2 = serving.SensitivityServer(precision='fp64', k=4, nPrimal=8, library=lib)
    st = srv2.serve(mix, realtime=False)
    assert st['requests'] == 5
    assert mix[1].sensitivity == alone[0].sensitivity          # bitwise
    plain = _reqs(['cyl16x8', 'box8', 'box6'], [1, 3, 2], 8)
    serving.plain_one_at_a_time(plain, lib, nPrimal=8)
    for r, q in zip(plain, [mix[0], mix[1], mix[2]]):
        assert abs(r.sensitivity - q.sensitivity) <= 1e-12 * abs(r.sensitivity), (r.key, r.sensitivity, q.sensitivity)


def test_fp32_served_within_bound_of_fp64():
    lib = serving.MeshLibrary()
    r64 = _reqs(KEYS, [7, 8, 9], 8)
    serving.plain_one_at_a_time(r64, lib, nPrimal=8)
    r32 = _reqs(KEYS, [7, 8, 9], 8)
    srv = serving.SensitivityServer(precision='fp32', k=4, nPrimal=8, library=lib)
    srv.serve(r32, realtime=False)
    for a, b in zip(r32, r64):
        # FP32 storage and flux arithmetic, FP64 sensitivity accumulation: 1e-3 relative over
        # 8 primal + 8 adjoint steps
        assert abs(a.sensitivity - b.sensitivity) <= 1e-3 * abs(b.sensitivity), (a.key, a.sensitivity, b.sensitivity)


def test_mixed_served_within_bound_of_fp64():
    lib = serving.MeshLibrary()
    r64 = _reqs(KEYS, [7, 8, 9], 8)
    serving.plain_one_at_a_time(r64, lib, nPrimal=8)
    rm = _reqs(KEYS, [7, 8, 9], 8)
    srv = serving.SensitivityServer(precision='mixed', k=4, nPrimal=8, library=lib)
    srv.serve(rm, realtime=False)
    for a, b in zip(rm, r64):
        # FP32 face arithmetic, FP64 state, stages, adjoints and sums: 1e-5 relative
        assert abs(a.sensitivity - b.sensitivity) <= 1e-5 * abs(b.sensitivity), (a.key, a.sensitivity, b.sensitivity)
