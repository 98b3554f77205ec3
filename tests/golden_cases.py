"""Golden trajectories of the reference solver (tests/golden/*.npz) and the cases they came from."""
import os

import numpy as np

from adfvm_gb300 import cases

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

CASES = {
    'sod1000': lambda: cases.sod(1000),
    'sod200_sym_lf': lambda: cases.sod(200, side='symmetryPlane', riemann='eulerLaxFriedrichs'),
    'box8': lambda: cases.box(8, objective='kinetic_energy'),
    'box6_inviscid_sumT': lambda: cases.box(6, objective='sum_T', viscous=False),
    'cyl32x16': lambda: cases.cylinder(32, 16, objective='drag:cylinder'),
    'duct100_totalpt': lambda: cases.duct(100),
    'duct60_totalpt_normals': lambda: cases.duct(60, direction=False, U0=-20.0),
    'vane32x12': lambda: cases.vane_channel(32, 12, reference_constants=True),
}


def available():
    return [k for k in CASES if os.path.exists(os.path.join(HERE, k + '.npz'))]


def load(name):
    g = dict(np.load(os.path.join(HERE, name + '.npz')))
    case = CASES[name]()
    return case, g


def rel_err(x, ref):
    """max|x-ref| / max|ref| per field (the relative error of the reference's tests,
    tests/test_op.py:15-18)."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    assert x.shape == ref.shape, (x.shape, ref.shape)
    den = np.max(np.abs(ref))
    return float(np.max(np.abs(x - ref)) / (den if den > 0 else 1.0))


def load_sharp_sod():
    """The reference's first step on the one-cell-jump Sod tube (tests/golden/sod1000_sharp.npz):
    it returns a non-finite CFL sum and a state non-finite around the jump."""
    g = dict(np.load(os.path.join(HERE, 'sod1000_sharp.npz')))
    return cases.sod(1000, smooth_cells=None), g


def nonfinite_parity(x, ref):
    """(same non-finite entries, max|x-ref|/max|ref| over the entries finite in both)."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    assert x.shape == ref.shape, (x.shape, ref.shape)
    fx, fr = np.isfinite(x), np.isfinite(ref)
    ok = fx & fr
    den = np.max(np.abs(ref[ok])) if ok.any() else 1.0
    return bool(np.array_equal(fx, fr)), float(np.max(np.abs(x[ok] - ref[ok])) / den) if ok.any() else 0.0
