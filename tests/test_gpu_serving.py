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


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_reduced_precision_served_within_1e5_of_fp64(precision):
    """The served request as the workload defines it - 100 primal + 100 adjoint steps,
    checkpoints every 10 - on the smallest box and the smallest cylinder of the serving mix:
    FP32 storage and flux arithmetic with FP64 sensitivity accumulation ('fp32'), and the same
    with FP64 state, stages and adjoints ('mixed'), within 1e-5 relative of plain FP64."""
    lib = serving.MeshLibrary()
    keys = ['box16', 'cyl64x32']
    r64 = _reqs(keys, [7, 8], 100)
    serving.plain_one_at_a_time(r64, lib, nPrimal=100)
    rr = _reqs(keys, [7, 8], 100)
    srv = serving.SensitivityServer(precision=precision, k=10, nPrimal=100, library=lib)
    srv.serve(rr, realtime=False)
    for a, b in zip(rr, r64):
        e = abs(a.sensitivity - b.sensitivity) / abs(b.sensitivity)
        assert e <= 1e-5, '%s %s: rel err %.3e' % (precision, a.key, e)
    srv.close()


def test_admission_under_memory_pressure():
    """An HBM budget that holds two slots, three meshes, requests arriving in real time while
    others run: requests queue, an idle slot of one mesh is evicted for another mesh, requests
    are admitted mid-flight - and every FP64 result is bitwise the one of the same request
    served alone."""
    lib = serving.MeshLibrary()
    keys = ['box8', 'cyl16x8', 'box6', 'box8', 'box6', 'cyl16x8', 'box8']
    seeds = [11, 12, 13, 14, 15, 16, 17]
    alone = []
    big = serving.SensitivityServer(precision='fp64', k=4, nPrimal=20, library=lib)
    for k, sd in zip(keys, seeds):
        r = serving.Request(rid=0, key=k, seed=sd, nPrimal=20)
        big.serve([r], realtime=False)
        alone.append(r.sensitivity)
    sizes = {k: big.bytes_of[k] for k in set(keys)}
    big.close()
    budget = sum(sorted(sizes.values())[-2:]) + 1       # the two largest slots, no third
    srv = serving.SensitivityServer(precision='fp64', k=4, nPrimal=20, library=lib, hbm_budget=budget)
    srv.bytes_of.update(sizes)
    reqs = [serving.Request(rid=i, key=k, seed=sd, nPrimal=20, arrival=0.002 * i)
            for i, (k, sd) in enumerate(zip(keys, seeds))]
    st = srv.serve(reqs, realtime=True)
    assert st['requests'] == len(reqs)
    assert srv.evictions >= 1 and srv.queued >= 1, (srv.evictions, srv.queued)
    assert len(srv.slots) <= 2 and srv.used <= budget
    assert any(r.t_admit > r.arrival + 1e-3 for r in reqs)          # waited for a slot
    for r, ref in zip(reqs, alone):
        assert r.sensitivity == ref, (r.rid, r.key, r.sensitivity, ref)
    srv.close()


def test_batched_slots_give_each_request_its_own_result():
    """A batched slot runs up to K requests on one mesh in the same launches (K disjoint copies
    of the mesh): each request's FP64 sensitivity is bitwise the same whichever copy it runs in,
    alone or with others, and equals the plain one-at-a-time result within 1e-12."""
    lib = serving.MeshLibrary()
    keys = ['box8', 'box8', 'cyl16x8', 'box8', 'cyl16x8']
    seeds = [21, 22, 23, 24, 25]
    srv = serving.SensitivityServer(precision='fp64', k=4, nPrimal=8, library=lib, batch={'box8': 3, 'cyl16x8': 2})
    mix = _reqs(keys, seeds, 8)
    srv.serve(mix, realtime=False)
    assert all(s.copies in (2, 3) for s in srv.slots)
    # the box8 requests ran as one batch (seeds 21, 22, 24 in copies 0, 1, 2): seed 24 alone in
    # copy 0 (the other copies idle), and in copy 1 of a batch in another order
    alone = _reqs(['box8'], [24], 8)
    srv.serve(alone, realtime=False)
    assert alone[0].sensitivity == mix[3].sensitivity
    other = _reqs(['box8', 'box8', 'box8'], [22, 24, 21], 8)
    srv.serve(other, realtime=False)
    assert other[1].sensitivity == mix[3].sensitivity
    assert other[2].sensitivity == mix[0].sensitivity
    assert other[0].sensitivity == mix[1].sensitivity
    plain = _reqs(keys, seeds, 8)
    serving.plain_one_at_a_time(plain, lib, nPrimal=8)
    for a, b in zip(mix, plain):
        assert abs(a.sensitivity - b.sensitivity) <= 1e-12 * abs(b.sensitivity), (a.key, a.sensitivity, b.sensitivity)
    srv.close()
