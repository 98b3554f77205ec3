"""The gauge form of the FP32 face flux (adfvm_gb300/csrc/face.cuh face_flux_gauge, compiled for
the host): in double it equals the reference's flux less gaugeP N (momentum) and gaugeH times the
mass flux (energy); in float it is far closer to the exact flux than the absolute form on a
low-Mach face set, which is what the FP32 records' gauge is for."""
import ctypes as C

import numpy as np
import pytest

from tests.test_face_adjoint import KINDS, host, native_in, phys, random_faces  # noqa: F401

CFGS = [dict(mu=None, riemann='eulerRoe', briemann='eulerRoe'),
        dict(mu=2.5e-5, riemann='eulerLaxFriedrichs', briemann='eulerLaxFriedrichs'),
        dict(mu=0.0, riemann='eulerRoe', briemann='eulerLaxFriedrichs')]
GAUGE = np.array([1.0e5, 300.0, 1004.5 * 300.0 + 0.5 * 100.0 ** 2])


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run(host, fn, kind, cfg, X, *extra):
    n = len(X)
    F = np.zeros((n, 6))
    inviscid = 1 if cfg['mu'] == 0.0 else 0
    ph = phys(cfg)
    args = [n, KINDS[kind], inviscid, dp(ph)] + list(extra) + [dp(np.ascontiguousarray(X)), dp(F)]
    getattr(host, fn)(*args)
    return F


def gauge_of(host, kind, cfg, X, f32):
    host.afvm_host_face_gauge.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    return run(host, 'afvm_host_face_gauge', kind, cfg, X, dp(GAUGE), 1 if f32 else 0)


def restore(Fg, X):
    """The reference's flux from the gauge form: + gaugeP N on the momentum, + gaugeH F[0] on
    the energy (what the closed-cell sums and the update's correction restore)."""
    F = Fg.copy()
    F[:, 1:4] += GAUGE[0] * X[:, 40:43]
    F[:, 4] += GAUGE[2] * Fg[:, 0]
    return F


@pytest.mark.parametrize('cfg', CFGS, ids=lambda c: '%s-%s-%s' % (c['riemann'], c['briemann'], c['mu']))
@pytest.mark.parametrize('kind', list(KINDS))
def test_gauge_form_is_the_flux_less_the_gauge_terms(host, kind, cfg):
    X = native_in(random_faces(400, 11 + KINDS[kind]))
    F = run(host, 'afvm_host_face', kind, cfg, X)
    Fg = restore(gauge_of(host, kind, cfg, X, False), X)
    scale = np.abs(F).max(axis=0)
    err = np.abs(Fg - F).max(axis=0) / scale
    assert err.max() <= 1e-12, err


def low_mach_faces(n, seed):
    """Faces of a Mach ~0.3 flow near the gauge state: p 1e5 +- 1e2 Pa, T 300 +- 0.3 K, U ~ 100 m/s
    varying by ~1 m/s between the two sides, gradients to match."""
    rng = np.random.default_rng(seed)
    X = random_faces(n, seed)
    U0 = np.array([100.0, 10.0, 0.0])
    X[:, 0:3] = U0 + rng.normal(0, 1.0, (n, 3))
    X[:, 5:8] = X[:, 0:3] + rng.normal(0, 0.5, (n, 3))
    X[:, 3] = 300 + rng.normal(0, 0.3, n)
    X[:, 8] = X[:, 3] + rng.normal(0, 0.03, n)
    X[:, 4] = 1e5 + rng.normal(0, 1e2, n)
    X[:, 9] = X[:, 4] + rng.normal(0, 10.0, n)
    X[:, 10:40] = rng.normal(0, 1, (n, 30)) * np.concatenate([np.full(9, 50.), np.full(3, 30.), np.full(3, 1e4),
                                                             np.full(9, 50.), np.full(3, 30.), np.full(3, 1e4)])
    return native_in(X)


@pytest.mark.parametrize('kind', ['internal', 'characteristic', 'boundary'])
def test_float_gauge_form_keeps_the_low_mach_digits(host, kind):
    cfg = CFGS[0]
    X = low_mach_faces(2000, 5 + KINDS[kind])
    host.afvm_host_face_f32.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
    F64 = run(host, 'afvm_host_face', kind, cfg, X)
    Fabs32 = run(host, 'afvm_host_face_f32', kind, cfg, X)
    G64 = gauge_of(host, kind, cfg, X, False)
    G32 = gauge_of(host, kind, cfg, X, True)
    # what the cell sums see: the absolute FP32 flux's error against the gauge FP32 flux's
    # (the gauge terms are restored exactly in the update and by the closed-cell sums)
    e_abs = np.abs(Fabs32 - F64)[:, :5].mean(axis=0)
    e_g = np.abs(G32 - G64)[:, :5].mean(axis=0)
    # momentum: the rounding of p N (p ~ 1e5) is gone, that of rho U Un (~1e4) stays - 6-20x
    # smaller errors; energy: rho h Un (~3.5e7) becomes rho (h - gaugeH) Un - ~140x smaller
    assert (e_g[1:4] * 4 < e_abs[1:4]).all(), (e_g, e_abs)
    assert e_g[4] * 50 < e_abs[4], (e_g, e_abs)
    assert e_g[0] <= 2 * e_abs[0] + 1e-12, (e_g, e_abs)
