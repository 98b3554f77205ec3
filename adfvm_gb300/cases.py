"""The workloads of this path: meshes, boundary conditions, initial states and solver options.

Boundary conditions use the reference's boundary-dict form (what ``IOField`` reads from a
case's 0/ directory): ``{'U': {patch: {'type': ..., 'value'|'U0'|'T0'|'p0': array}}, 'T':
..., 'p': ...}``.

* ``sod``       - Sod shock tube on an n x 1 x 1 hex tube; p=1e5/1e4 Pa, T=348.4/278.7 K,
                  U=0; inviscid, Roe, SSP-RK3, CFL 0.5.
* ``box``       - periodic jittered n^3 box; rho=1.2, T=300 K, Mach-0.3 Taylor-Green velocity
                  plus 1% Gaussian noise; Sutherland viscosity, Roe.
* ``cylinder``  - 2-D cylinder O-grid; no-slip wall, characteristic (CBC_UPT) far field at
                  Mach 0.3, T=300 K, p=1e5 Pa; Sutherland viscosity, Roe inside and
                  Lax-Friedrichs on the far field.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import meshgen
from .mesh import Mesh

GAMMA = 1.4
CP = 1004.5
R_GAS = CP - CP / GAMMA


@dataclass
class Case:
    name: str
    meshData: tuple
    bc: dict
    U: np.ndarray
    T: np.ndarray
    p: np.ndarray
    config: dict = field(default_factory=dict)   # RCF options (reference names)
    objective: str = 'none'                      # none | kinetic_energy | drag:<patch> | sum_T
    dt: float = 1e-7
    source: tuple = None                         # (S_rho, S_rhoU, S_rhoE) or None
    mesh: Mesh = None
    builder: object = None                       # meshData -> mesh; None: Mesh.create (this library)

    def build_mesh(self):
        if self.mesh is None:
            self.mesh = (self.builder or Mesh.create)(self.meshData)
        return self.mesh


def _uniform_bc(mesh_boundary, kind_of):
    out = {'U': {}, 'T': {}, 'p': {}}
    for patch, b in mesh_boundary.items():
        for f in out:
            out[f][patch] = kind_of(patch, b, f)
    return out


def sod(n=1000, side='empty', riemann='eulerRoe', cfl=0.5, smooth_cells=2.0):
    md = meshgen.sod_tube(n, side_type=side)
    bnd = md[4]

    def kind(patch, b, f):
        if b['type'] in ('empty', 'symmetryPlane'):
            return {'type': b['type']}
        return {'type': 'zeroGradient'}
    case = Case('sod%d' % n, md, _uniform_bc(bnd, kind), None, None, None,
                config={'mu': 0.0, 'riemannSolver': riemann, 'CFL': cfl, 'stepFactor': 1.2},
                dt=1e-7)
    mesh = case.build_mesh()
    x = mesh.cellCentres[:mesh.nInternalCells, 0:1]
    # the jump is spread over ~2 cells (tanh): with a one-cell jump (smooth_cells=None) the
    # reference's unlimited second-order reconstruction (adFVM/interp.py:20-28) gives a
    # negative face pressure in the first stage and its solver stops with NaN
    if smooth_cells is None:
        s = (x < 0.5).astype(np.float64)
    else:
        s = 0.5 * (1.0 - np.tanh((x - 0.5) / (smooth_cells / n)))
    case.U = np.zeros((mesh.nInternalCells, 3))
    case.T = 278.7 + (348.4 - 278.7) * s
    case.p = 1e4 + (1e5 - 1e4) * s
    return case


def taylor_green(cc, L=1.0, T0=300.0, mach=0.3, noise=0.01, seed=2):
    c = math.sqrt(GAMMA * R_GAS * T0)
    uinf = mach * c
    xh = 2 * np.pi * cc[:, 0] / L
    yh = 2 * np.pi * cc[:, 1] / L
    zh = 2 * np.pi * cc[:, 2] / L
    U = np.zeros((len(cc), 3))
    U[:, 0] = uinf * np.sin(xh) * np.cos(yh) * np.cos(zh)
    U[:, 1] = -uinf * np.cos(xh) * np.sin(yh) * np.cos(zh)
    U += np.random.default_rng(seed).normal(0.0, noise * uinf, size=U.shape)
    return U


def box(n=128, objective='kinetic_energy', riemann='eulerRoe', viscous=True, seed=0, cfl=0.5,
        reorder=True, builder=None):
    md = meshgen.periodic_box(n, seed_jitter=seed, reorder=reorder)
    bc = _uniform_bc(md[4], lambda patch, b, f: {'type': 'cyclic'})
    cfg = {'riemannSolver': riemann, 'fixedTimeStep': True}
    if not viscous:
        cfg['mu'] = 0.0
    case = Case('box%d' % n, md, bc, None, None, None, config=cfg, objective=objective, builder=builder)
    mesh = case.build_mesh()
    cc = mesh.cellCentres[:mesh.nInternalCells]
    rho0, T0 = 1.2, 300.0
    case.U = taylor_green(cc)
    case.T = np.full((mesh.nInternalCells, 1), T0)
    case.p = np.full((mesh.nInternalCells, 1), rho0 * R_GAS * T0)
    # dt from CFL at t=0: dt = 2*CFL/max_c sum_f (|U.n|+a) A/V with cell-centred estimates
    a = math.sqrt(GAMMA * R_GAS * T0)
    h = 1.0 / n
    umax = np.abs(case.U).max()
    case.dt = float(cfl * h / (umax * math.sqrt(3.0) + a))
    return case


def cylinder(n_theta=256, n_r=128, mach=0.3, T0=300.0, p0=1e5, objective='drag:cylinder',
             boundary_riemann='eulerLaxFriedrichs', mu=None):
    md = meshgen.cylinder_ogrid(n_theta, n_r)
    bnd = md[4]
    c = math.sqrt(GAMMA * R_GAS * T0)
    uinf = mach * c

    def kind(patch, b, f):
        nf = b['nFaces']
        if patch == 'cylinder':
            if f == 'U':
                return {'type': 'fixedValue', 'value': np.zeros((nf, 3))}
            return {'type': 'zeroGradient'}
        if patch == 'farfield':
            U0 = np.zeros((nf, 3)); U0[:, 0] = uinf
            return {'type': 'CBC_UPT', 'U0': U0, 'T0': np.full((nf, 1), T0), 'p0': np.full((nf, 1), p0)}
        return {'type': 'empty'}
    cfg = {'boundaryRiemannSolver': boundary_riemann, 'fixedTimeStep': True}
    if mu is not None:
        cfg['mu'] = mu
    case = Case('cylinder%dx%d' % (n_theta, n_r), md, _uniform_bc(bnd, kind), None, None, None,
                config=cfg, objective=objective)
    mesh = case.build_mesh()
    nc = mesh.nInternalCells
    case.U = np.zeros((nc, 3)); case.U[:, 0] = uinf
    case.T = np.full((nc, 1), T0)
    case.p = np.full((nc, 1), p0)
    # wall-normal spacing sets the acoustic CFL
    r0 = 0.5
    growth = (20.0 / r0) ** (1.0 / n_r)
    dr = r0 * (growth - 1)
    case.dt = float(0.5 * dr / (uinf + c))
    return case


def duct(n=100, Tt=310.0, pt=1.05e5, U0=50.0, T0=300.0, p0=1e5, direction=True):
    """1-D duct on the Sod tube mesh: total-pressure inlet (CBC_TOTAL_PT, BCs.py:164-184) on
    ``left``, characteristic outlet (CBC_UPT) on ``right``, empty sides; uniform initial flow;
    Sutherland viscosity, Roe inside and on the characteristic patches."""
    md = meshgen.sod_tube(n)
    bnd = md[4]

    def kind(patch, b, f):
        nf = b['nFaces']
        if patch == 'left':
            d = {'type': 'CBC_TOTAL_PT', 'Tt': np.full((nf, 1), Tt), 'pt': np.full((nf, 1), pt)}
            if direction:
                dd = np.zeros((nf, 3)); dd[:, 0] = 1.0
                d['direction'] = dd
            return d
        if patch == 'right':
            u = np.zeros((nf, 3)); u[:, 0] = U0
            return {'type': 'CBC_UPT', 'U0': u, 'T0': np.full((nf, 1), T0), 'p0': np.full((nf, 1), p0)}
        return {'type': 'empty'}
    case = Case('duct%d' % n, md, _uniform_bc(bnd, kind), None, None, None,
                config={'fixedTimeStep': True}, objective='sum_T')
    mesh = case.build_mesh()
    nc = mesh.nInternalCells
    case.U = np.zeros((nc, 3)); case.U[:, 0] = U0
    case.T = np.full((nc, 1), T0)
    case.p = np.full((nc, 1), p0)
    c = math.sqrt(GAMMA * R_GAS * T0)
    case.dt = float(0.5 * (1.0 / n) / (U0 + c))
    return case


def vane_channel(nx=64, ny=24, Tt=310.0, pt=1.08e5, U0=100.0, T0=300.0, p0=1e5, Tw=350.0, a=0.4, b=1e-5,
                 stretch=0.3, reference_constants=False):
    """Channel with the turbine-vane objective (adFVM/objectives/vane.py): the plane x = 0.052641
    and the ``pressure``/``suction`` walls of that file, a total-pressure inlet (CBC_TOTAL_PT, x
    direction) and a characteristic outlet (CBC_UPT); no-slip walls (fixedValue U = 0,
    zeroGradient T, p), empty front/back; Sutherland viscosity, Roe. The objective uses this
    inlet's total pressure for ptin, a wall temperature of 350 K and weights a = 0.4 (the
    reference's) and b = 1e-5 (the reference has 0; a non-zero b exercises the heat term).
    reference_constants=True keeps the constants of objectives/vane.py itself (ptin 175158,
    Tw 300, a 0.4, b 0), as its own objective function hard-codes them."""
    from . import vane
    md = meshgen.channel(nx, ny, stretch=stretch)
    bnd = md[4]

    def kind(patch, b_, f):
        nf = b_['nFaces']
        if patch == 'inlet':
            d = np.zeros((nf, 3)); d[:, 0] = 1.0
            return {'type': 'CBC_TOTAL_PT', 'Tt': np.full((nf, 1), Tt), 'pt': np.full((nf, 1), pt), 'direction': d}
        if patch == 'outlet':
            u = np.zeros((nf, 3)); u[:, 0] = U0
            return {'type': 'CBC_UPT', 'U0': u, 'T0': np.full((nf, 1), T0), 'p0': np.full((nf, 1), p0)}
        if patch in ('pressure', 'suction'):
            if f == 'U':
                return {'type': 'fixedValue', 'value': np.zeros((nf, 3))}
            return {'type': 'zeroGradient'}
        return {'type': 'empty'}
    case = Case('vane_channel%dx%d' % (nx, ny), md, _uniform_bc(bnd, kind), None, None, None,
                config={'fixedTimeStep': True})
    mesh = case.build_mesh()
    case.objective = vane.options(mesh) if reference_constants else vane.options(mesh, ptin=pt, Tw=Tw, a=a, b=b)
    nc = mesh.nInternalCells
    case.U = np.zeros((nc, 3)); case.U[:, 0] = U0
    case.T = np.full((nc, 1), T0)
    case.p = np.full((nc, 1), p0)
    c = math.sqrt(GAMMA * R_GAS * T0)
    dx = float(np.min(np.diff(np.unique(np.round(mesh.cellCentres[:nc, 0], 12)))))
    case.dt = float(0.5 * dx / (U0 + c))
    return case


def conservative(case, gamma=GAMMA, Cp=CP):
    """Initial conservative state of a case: RCF.conservative (adFVM/density.py:173-181)."""
    Cv = Cp / gamma
    e = Cv * case.T
    rho = case.p / (e * (gamma - 1))
    rhoE = rho * (e + 0.5 * np.sum(case.U * case.U, axis=1, keepdims=True))
    rhoU = case.U * rho
    return rho, rhoU, rhoE


def source_field(mesh, scale=1.0, seed=5):
    """A smooth seeded source term (S_rho, S_rhoU, S_rhoE) on the internal cells."""
    rng = np.random.default_rng(seed)
    cc = mesh.cellCentres[:mesh.nInternalCells]
    mid = cc.mean(axis=0) + 0.1 * rng.standard_normal(3) * (cc.max(0) - cc.min(0))
    width = 0.1 * (cc.max(0) - cc.min(0)).max()
    G = scale * np.exp(-np.sum((cc - mid) ** 2, axis=1, keepdims=True) / width ** 2)
    S_rhoU = np.zeros((len(cc), 3)); S_rhoU[:, 0] = 100 * G[:, 0]
    return (G.copy(), S_rhoU, 2e5 * G)


def gauge(case):
    """A gauge state for the FP32 records of the case's contexts (RCF(gauge=...)): the mean
    initial pressure, temperature and total enthalpy Cp T + |U|^2/2 - for a case whose boundary
    conditions fix no p or T (a periodic box), whose contexts would otherwise have none."""
    U = np.asarray(case.U, np.float64).reshape(-1, 3)
    T = np.asarray(case.T, np.float64).reshape(-1)
    p = np.asarray(case.p, np.float64).reshape(-1)
    return (float(p.mean()), float(T.mean()), float((CP * T + 0.5 * (U * U).sum(axis=1)).mean()))


def copies(case, K):
    """The case on K disjoint copies of its mesh (meshgen.copies): boundary values and the
    initial primitive fields repeated per copy, the same options, objective and dt."""
    md = meshgen.copies(case.meshData, K)
    rep = lambda a: np.concatenate([np.asarray(a)] * K) if isinstance(a, np.ndarray) else a
    bc = {f: {p: {k: rep(v) for k, v in e.items()} for p, e in case.bc[f].items()} for f in case.bc}
    c = Case('%sx%d' % (case.name, K), md, bc, rep(case.U), rep(case.T), rep(case.p), config=dict(case.config),
             objective=case.objective, dt=case.dt)
    c.build_mesh()
    return c
