"""The hand-derived face adjoint (adfvm_gb300/csrc/face.cuh, compiled for the host) against
torch autograd of the oracle's face physics, on random physically plausible face states."""
import ctypes as C
import os
import subprocess
import types

import numpy as np
import pytest
import torch

from oracle import torch_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, 'tests', 'native', 'face_host.cpp')
OUT = os.path.join(ROOT, 'tests', 'native', '_face_host.so')

KINDS = {'internal': 0, 'coupled': 1, 'characteristic': 2, 'boundary': 3}
NAMES_IN = (['UP%d' % k for k in range(3)] + ['TP', 'pP'] + ['UN%d' % k for k in range(3)] + ['TN', 'pN'] +
            ['gUP%d' % k for k in range(9)] + ['gTP%d' % k for k in range(3)] + ['gpP%d' % k for k in range(3)] +
            ['gUN%d' % k for k in range(9)] + ['gTN%d' % k for k in range(3)] + ['gpN%d' % k for k in range(3)])


@pytest.fixture(scope='module')
def host():
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(ROOT, 'adfvm_gb300', 'csrc', 'face.cuh')),
            os.path.getmtime(os.path.join(ROOT, 'adfvm_gb300', 'csrc', 'physics.cuh'))):
        subprocess.check_call(['g++', '-O2', '-std=c++17', '-fPIC', '-shared', '-ffp-contract=off',
                               '-I' + os.path.join(ROOT, 'include'), '-I' + os.path.join(ROOT, 'adfvm_gb300', 'csrc'),
                               SRC, '-o', OUT])
    lib = C.CDLL(OUT)
    d = C.POINTER(C.c_double)
    lib.afvm_host_face.argtypes = [C.c_int, C.c_int, C.c_int, d, d, d]
    lib.afvm_host_face_vjp.argtypes = [C.c_int, C.c_int, C.c_int, d, d, d, d]
    lib.afvm_host_face_vjp_f32.argtypes = [C.c_int, C.c_int, C.c_int, d, d, d, d]
    lib.afvm_host_face_vjp_geo.argtypes = [C.c_int, C.c_int, C.c_int, d, d, d, d]
    return lib


def random_faces(n, seed, char=False):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 55))
    U = rng.normal(0, 80, (n, 6))
    X[:, 0:3] = U[:, :3]
    X[:, 5:8] = U[:, 3:]
    X[:, 3] = rng.uniform(250, 350, n)
    X[:, 8] = X[:, 3] * rng.uniform(0.9, 1.1, n)
    X[:, 4] = rng.uniform(0.8e5, 1.2e5, n)
    X[:, 9] = X[:, 4] * rng.uniform(0.9, 1.1, n)
    X[:, 10:40] = rng.normal(0, 1, (n, 30)) * np.concatenate([np.full(9, 500.), np.full(3, 300.), np.full(3, 1e5),
                                                             np.full(9, 500.), np.full(3, 300.), np.full(3, 1e5)])
    N = rng.normal(size=(n, 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    D = N + 0.1 * rng.normal(size=(n, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    X[:, 40:43] = N
    X[:, 43:46] = D
    X[:, 46] = rng.uniform(0.1, 0.25, n)      # lw0
    X[:, 47] = rng.uniform(0.1, 0.25, n)      # lw1
    X[:, 48:51] = 1e-3 * rng.normal(size=(n, 3))
    X[:, 51:54] = 1e-3 * rng.normal(size=(n, 3))
    X[:, 54] = rng.uniform(0.005, 0.02, n)    # delta
    return X


def native_in(X):
    """The native face input: slot 54 holds 1/delta (a mesh table of the device path)."""
    Xn = np.array(X, np.float64)
    Xn[:, 54] = 1.0 / Xn[:, 54]
    return Xn


def torch_face(kind, X, cfg):
    """The oracle's face physics for a batch of faces (RCF.flux / RCF.boundaryFlux)."""
    obj = types.SimpleNamespace()
    obj.gamma, obj.Cp, obj.Pr = 1.4, 1004.5, 0.7
    obj.Cv = obj.Cp / obj.gamma
    if cfg['mu'] is None:
        obj.mu = lambda T: 1.4792e-06 * T ** 1.5 / (T + 116.)
    else:
        obj.mu = lambda T, v=cfg['mu']: v
    obj.riemann = cfg['riemann']
    obj.boundaryRiemann = cfg['briemann']
    n = X.shape[0]
    N, D = X[:, 40:43], X[:, 43:46]
    obj.normals, obj.deltasUnit, obj.deltas = N, D, X[:, 54:55]
    P = torch_ref.Problem
    UP, TP, pP = X[:, 0:3], X[:, 3:4], X[:, 4:5]
    UN, TN, pN = X[:, 5:8], X[:, 8:9], X[:, 9:10]
    gUP, gTP, gpP = X[:, 10:19].reshape(n, 3, 3), X[:, 19:22].reshape(n, 1, 3), X[:, 22:25].reshape(n, 1, 3)
    gUN, gTN, gpN = X[:, 25:34].reshape(n, 3, 3), X[:, 34:37].reshape(n, 1, 3), X[:, 37:40].reshape(n, 1, 3)
    lw0, lw1 = X[:, 46:47], X[:, 47:48]
    qw0, qw1 = X[:, 48:51], X[:, 51:54]
    sl = slice(0, n)
    if kind == 'boundary':
        rho, rhoU, rhoE = P.conservative(obj, UN, TN, pN)
        Un = torch_ref.dot3(UN, N).unsqueeze(-1)
        F0, Fu, FE = rho * Un, rhoU * Un + pN * N, (rhoE + pN) * Un
        TF, UF, gTF, gUF = TN, UN, gTN[:, 0], gUN
    else:
        ULF = P._recon(UP, UN, gUP, lw0, qw0)
        TLF = P._recon(TP, TN, gTP, lw0, qw0)
        pLF = P._recon(pP, pN, gpP, lw0, qw0)
        rhoL, rhoUL, rhoEL = P.conservative(obj, ULF, TLF, pLF)
        if kind == 'characteristic':
            URF, TRF, pRF = UN, TN, pN
            solver = obj.boundaryRiemann
        else:
            URF = P._recon(UN, UP, gUN, lw1, qw1)
            TRF = P._recon(TN, TP, gTN, lw1, qw1)
            pRF = P._recon(pN, pP, gpN, lw1, qw1)
            solver = obj.riemann
        rhoR, rhoUR, rhoER = P.conservative(obj, URF, TRF, pRF)
        fn = P._roe if solver == 'eulerRoe' else P._lf
        F0, Fu, FE = fn(obj, pLF, pRF, TLF, TRF, ULF, URF, rhoL, rhoR, rhoUL, rhoUR, rhoEL, rhoER, N)
        if kind == 'characteristic':
            TF, UF, gTF, gUF = TN, UN, gTN[:, 0], gUN
        else:
            TF, UF = 0.5 * (TLF + TRF), 0.5 * (ULF + URF)
            gTF, gUF = 0.5 * (gTP + gTN)[:, 0], 0.5 * (gUP + gUN)
    if cfg['mu'] != 0.0:
        vU, vE = P._viscous(obj, TP, TN, UP, UN, TF, UF, gTF, gUF, sl)
        Fu = Fu + vU
        FE = FE + vE
    aF = (obj.Cp * TF * (obj.gamma - 1)).sqrt()
    maxaF = torch_ref.dot3(UF, N).unsqueeze(-1).abs() + aF
    return torch.cat([F0, Fu, FE, maxaF], dim=1)


CONFIGS = [
    ('internal', {'mu': None, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
    ('internal', {'mu': 0.0, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
    ('internal', {'mu': 2.5e-5, 'riemann': 'eulerLaxFriedrichs', 'briemann': 'eulerRoe'}),
    ('coupled', {'mu': None, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
    ('characteristic', {'mu': None, 'riemann': 'eulerRoe', 'briemann': 'eulerLaxFriedrichs'}),
    ('characteristic', {'mu': None, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
    ('boundary', {'mu': None, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
    ('boundary', {'mu': 0.0, 'riemann': 'eulerRoe', 'briemann': 'eulerRoe'}),
]


def phys(cfg):
    mu_model = 1 if cfg['mu'] is None else 0
    mu0 = 0.0 if cfg['mu'] is None else cfg['mu']
    r = {'eulerRoe': 0, 'eulerLaxFriedrichs': 1}
    return np.array([1.4, 1004.5, 0.7, mu_model, mu0, 1.4792e-06, 116., r[cfg['riemann']], r[cfg['briemann']]])


def dp(a):
    return np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize('kind,cfg', CONFIGS)
def test_face_forward_matches_oracle(host, kind, cfg):
    X = random_faces(64, 11)
    F = np.zeros((64, 6))
    host.afvm_host_face(64, KINDS[kind], 1 if cfg['mu'] == 0.0 else 0, dp(phys(cfg)), dp(native_in(X)), dp(F))
    ref = torch_face(kind, torch.as_tensor(X), cfg).numpy()
    err = np.abs(F - ref) / (np.abs(ref).max(axis=0) + 1e-300)
    assert err.max() < 1e-12, err.max(axis=0)


@pytest.mark.parametrize('kind,cfg', CONFIGS)
def test_face_adjoint_matches_autograd(host, kind, cfg):
    n = 64
    X = random_faces(n, 12)
    Fb = np.random.default_rng(13).normal(size=(n, 5))
    out = np.zeros((n, 40))
    host.afvm_host_face_vjp(n, KINDS[kind], 1 if cfg['mu'] == 0.0 else 0, dp(phys(cfg)), dp(native_in(X)), dp(Fb), dp(out))
    Xt = torch.as_tensor(X).clone().requires_grad_(True)
    F = torch_face(kind, Xt, cfg)
    J = (F[:, :5] * torch.as_tensor(Fb)).sum()
    (g,) = torch.autograd.grad(J, Xt)
    ref = g.numpy()[:, :40]
    scale = np.abs(ref).max(axis=0) + 1e-300
    err = np.abs(out - ref) / scale
    bad = [(NAMES_IN[k], float(err[:, k].max())) for k in range(40) if err[:, k].max() > 1e-10]
    assert not bad, bad


@pytest.mark.parametrize('kind,cfg', CONFIGS)
def test_fp32_face_adjoint_matches_fp64(host, kind, cfg):
    """The FP32 VJP (a lean local tape: the Roe and viscous intermediates re-evaluated in the
    reverse sweep) against the FP64 one (the full tape) on the same faces: within FP32 rounding
    (1e-3 of each input's largest adjoint; a wrong term would be O(1))."""
    n = 64
    X = random_faces(n, 14)
    Fb = np.random.default_rng(15).normal(size=(n, 5))
    o64, o32 = np.zeros((n, 40)), np.zeros((n, 40))
    inv = 1 if cfg['mu'] == 0.0 else 0
    host.afvm_host_face_vjp(n, KINDS[kind], inv, dp(phys(cfg)), dp(native_in(X)), dp(Fb), dp(o64))
    host.afvm_host_face_vjp_f32(n, KINDS[kind], inv, dp(phys(cfg)), dp(native_in(X)), dp(Fb), dp(o32))
    scale = np.abs(o64).max(axis=0) + 1e-300
    err = np.abs(o32 - o64) / scale
    bad = [(NAMES_IN[k], float(err[:, k].max())) for k in range(40) if err[:, k].max() > 1e-3]
    assert not bad, bad


GEO_NAMES = ['N0', 'N1', 'N2', 'D0', 'D1', 'D2', 'lw0', 'lw1', 'qw0_0', 'qw0_1', 'qw0_2', 'qw1_0', 'qw1_1', 'qw1_2',
             'deltas']


@pytest.mark.parametrize('kind,cfg', CONFIGS)
def test_face_adjoint_with_geometry_matches_autograd(host, kind, cfg):
    """The VJP that also returns the adjoints of the face geometry (normals, deltasUnit,
    linearWeights, quadraticWeights, deltas: the face's share of the reference's mesh
    gradient, parameters = 'mesh', apps/adjoint.py:108-110) against autograd with respect to
    those inputs; the 40 state adjoints are the ones of the plain VJP, bit for bit."""
    n = 64
    X = random_faces(n, 16)
    Fb = np.random.default_rng(17).normal(size=(n, 5))
    out = np.zeros((n, 55))
    plain = np.zeros((n, 40))
    inv = 1 if cfg['mu'] == 0.0 else 0
    host.afvm_host_face_vjp_geo(n, KINDS[kind], inv, dp(phys(cfg)), dp(native_in(X)), dp(Fb), dp(out))
    host.afvm_host_face_vjp(n, KINDS[kind], inv, dp(phys(cfg)), dp(native_in(X)), dp(Fb), dp(plain))
    assert np.array_equal(out[:, :40], plain)
    # the native input is 1/deltas: d/d(deltas) = -(1/deltas)^2 d/d(1/deltas)
    geo = out[:, 40:].copy()
    geo[:, 14] = -geo[:, 14] / X[:, 54] ** 2
    Xt = torch.as_tensor(X).clone().requires_grad_(True)
    F = torch_face(kind, Xt, cfg)
    J = (F[:, :5] * torch.as_tensor(Fb)).sum()
    (g,) = torch.autograd.grad(J, Xt)
    ref = g.numpy()[:, 40:]
    scale = np.abs(ref).max(axis=0) + 1e-300
    err = np.abs(geo - ref) / scale
    bad = [(GEO_NAMES[k], float(err[:, k].max())) for k in range(15) if err[:, k].max() > 1e-12]
    assert not bad, bad
