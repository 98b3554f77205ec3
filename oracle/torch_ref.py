"""Oracle: CPU float64 restatement of the reference's residual, SSP-RK3 step and objectives.

TEST INFRASTRUCTURE ONLY. Imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline as the reference the GPU results are compared with; the product never calls it.

Written in torch (CPU, float64) so that ``torch.autograd`` of the same code gives the exact
discrete adjoint of a step (the reference obtains its adjoint by automatic differentiation
in adpy, apps/adjoint.py:101-126; adpy is absent, so AD of this restatement stands in).
Every operation follows the reference's expression order, left to right, and face
contributions are accumulated per cell in the reference's collate order (internal faces in
face order, then boundary patches in ``sortedPatches`` order, adFVM/density.py:390-402), so
results agree with the reference run (tests/golden) to rounding.

Pinned against trajectories of the reference's own solver code (tests/golden/*.npz, made
by tests/golden/make_golden.py).
"""
import numpy as np
import torch


SMALL = 1e-30                      # adFVM/config.py:171-178 (float64)
T64 = torch.float64


def _t(a, dtype=T64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype)


def dot3(a, b):
    """a . b over the last axis (3), products summed left to right."""
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


class Problem(object):
    """Mesh, boundary conditions and physics in the form the residual needs.

    mesh: an object with the reference Mesh attributes (adfvm_gb300.mesh.Mesh or the
    reference's own adFVM.mesh.Mesh). bc: the reference's boundary-dict form per field.
    config: RCF options (adFVM/density.py:22-39 names). objective: 'none',
    'kinetic_energy', 'sum_T' or 'drag:<patch>'.
    """

    def __init__(self, mesh, bc, config=None, objective='none'):
        cfg = {'Cp': 1004.5, 'gamma': 1.4, 'Pr': 0.7, 'riemannSolver': 'eulerRoe',
               'boundaryRiemannSolver': 'eulerRoe', 'mu': None}
        cfg.update(config or {})
        self.gamma = float(cfg['gamma'])
        self.Cp = float(cfg['Cp'])
        self.Pr = float(cfg['Pr'])
        self.Cv = self.Cp / self.gamma                    # density.py:44
        mu = cfg['mu']
        if mu is None:
            self.mu = lambda T: 1.4792e-06 * T ** 1.5 / (T + 116.)   # density.py:27
            self.mu_const = None
        else:
            v = float(mu)
            self.mu = lambda T, v=v: v
            self.mu_const = v
        self.riemann = cfg['riemannSolver']
        self.boundaryRiemann = cfg['boundaryRiemannSolver']
        self.objective = objective
        m = mesh
        self.mesh = mesh
        self.nIC = int(m.nInternalCells)
        self.nIF = int(m.nInternalFaces)
        self.nF = int(m.nFaces)
        self.nC = int(m.nCells)
        self.owner = _t(m.owner, torch.int64).reshape(-1)
        self.neighbour = _t(m.neighbour, torch.int64).reshape(-1)
        self.areas = _t(m.areas).reshape(-1, 1)
        self.normals = _t(m.normals).reshape(-1, 3)
        self.weights = _t(m.weights).reshape(-1, 1)
        self.deltas = _t(m.deltas).reshape(-1, 1)
        self.deltasUnit = _t(m.deltasUnit).reshape(-1, 3)
        self.lw = _t(m.linearWeights).reshape(-1, 2)
        self.qw = _t(m.quadraticWeights).reshape(-1, 2, 3)
        self.volumes = _t(m.volumes).reshape(-1, 1)
        self.volumesL = self.volumes[self.owner]
        self.volumesR = self.volumes[self.neighbour[:self.nIF]]
        self.cellFaces = _t(m.cellFaces, torch.int64).reshape(-1, 6)
        self.cellNeighbours = _t(m.cellNeighbours, torch.int64).reshape(-1, 6)
        self.cellOwner = _t(m.cellOwner, torch.int64).reshape(-1, 6)
        # op.div weights (op.py:12-29): wp = A/V_L, wn = A/V_R (sign applied per side)
        self.wp = self.areas / self.volumesL
        self.wnAbs = self.areas[:self.nIF] / self.volumesR

        # patches in sortedPatches order (mesh.py:100-101)
        self.patches = []
        for name in m.sortedPatches:
            b = m.boundary[name]
            s, n = int(b['startFace']), int(b['nFaces'])
            ptype = b['type']
            cs = s - self.nIF + self.nIC
            fb = {f: bc[f][name] for f in ('U', 'T', 'p')}
            kinds = {f: fb[f]['type'] for f in fb}
            char = any(k in ('CBC_UPT', 'CBC_TOTAL_PT') for k in kinds.values())
            coupled = ptype in ('cyclic', 'slidingPeriodic1D')
            if coupled:
                nb = m.boundary[b['neighbourPatch']]
                src = self.owner[int(nb['startFace']):int(nb['startFace']) + n]
            else:
                src = self.owner[s:s + n]
            entry = dict(name=name, start=s, n=n, cellStart=cs, type=ptype, kinds=kinds,
                         coupled=coupled, characteristic=char, src=src, bc=fb)
            if char and kinds['p'] == 'CBC_UPT':
                cb = bc['p'][name]      # characteristicBoundary uses p's BC objects (density.py:333-337)
                entry['U0'] = _t(cb['U0']).reshape(-1, 3)
                entry['T0'] = _t(cb['T0']).reshape(-1, 1)
                entry['p0'] = _t(cb['p0']).reshape(-1, 1)
            if char and kinds['p'] == 'CBC_TOTAL_PT':
                cb = bc['p'][name]
                entry['Tt'] = _t(cb['Tt']).reshape(-1, 1)
                entry['pt'] = _t(cb['pt']).reshape(-1, 1)
                entry['direction'] = (_t(cb['direction']).reshape(-1, 3) if 'direction' in cb
                                      else self.normals[s:s + n])
            for f, dims in (('U', 3), ('T', 1), ('p', 1)):
                if kinds[f] == 'fixedValue':
                    entry[f + '_fixed'] = _t(fb[f]['value']).reshape(-1, dims)
            self.patches.append(entry)
        # gradient ghosts: default boundary (mesh.py:702-711) -> copy of a source cell
        self.gradSrc = torch.zeros(self.nC - self.nIC, dtype=torch.int64)
        for P in self.patches:
            self.gradSrc[P['cellStart'] - self.nIC:P['cellStart'] - self.nIC + P['n']] = P['src']

        # per-cell accumulation table in collate order: (face, side) sorted by rank
        rank = np.arange(self.nF, dtype=np.int64)
        pos = self.nIF
        for P in self.patches:
            rank[P['start']:P['start'] + P['n']] = pos + np.arange(P['n'])
            pos += P['n']
        cf = np.asarray(m.cellFaces).reshape(-1, 6).astype(np.int64)
        order = np.argsort(rank[cf], axis=1, kind='stable')
        self.accFaces = torch.as_tensor(np.take_along_axis(cf, order, axis=1))
        own = np.asarray(m.owner).reshape(-1)[self.accFaces.numpy()] == np.arange(self.nIC)[:, None]
        self.accOwnerSide = torch.as_tensor(own)

    # ------------------------------------------------------------ conversions
    def primitive(self, rho, rhoU, rhoE):
        """adFVM/density.py:162-171."""
        U = rhoU / rho
        E = rhoE / rho
        e = E - 0.5 * dot3(U, U).unsqueeze(-1)
        p = (self.gamma - 1) * rho * e
        T = e * (1. / self.Cv)
        return U, T, p

    def conservative(self, U, T, p):
        """adFVM/density.py:173-181."""
        e = self.Cv * T
        rho = p / (e * (self.gamma - 1))
        rhoE = rho * (e + 0.5 * dot3(U, U).unsqueeze(-1))
        rhoU = U * rho
        return rho, rhoU, rhoE

    # ------------------------------------------------------------ boundary ghosts
    def ghosts(self, U, T, p):
        """Ghost rows of U, T, p (adFVM/BCs.py:86-161 via Solver.boundary, solver.py:106-114,
        and RCF.characteristicBoundary, density.py:333-337). U, T, p: internal rows. Ghost
        rows are ordered by cellStartFace (file order of the patches)."""
        pieces = []
        for P in self.patches:
            s, n, src = P['start'], P['n'], P['src']
            k = P['kinds']
            nrm = self.normals[s:s + n]
            if P['characteristic'] and 'Tt' in P:
                # CBC_TOTAL_PT (BCs.py:178-184)
                Uo, To = U[src], T[src]
                d = P['direction']
                Un = dot3(Uo, d).unsqueeze(-1)
                Ub = Un * d
                Tb = P['Tt'] - 0.5 * Un * Un / self.Cp
                pb = P['pt'] * (To / P['Tt']) ** (self.gamma / (self.gamma - 1))
                pieces.append((P['cellStart'], Ub, Tb, pb))
                continue
            if P['characteristic']:
                pieces.append((P['cellStart'], P['U0'] * 1, P['T0'] * 1, P['p0'] * 1))
                continue
            vals = []
            for f, val in (('U', U), ('T', T), ('p', p)):
                kind = k[f]
                if kind == 'fixedValue':
                    vals.append(P[f + '_fixed'] * 1)
                elif kind in ('zeroGradient', 'empty', 'inletOutlet', 'cyclic', 'calculated'):
                    vals.append(val[src])
                elif kind in ('symmetryPlane', 'slip'):
                    phiF = val[src]
                    if f == 'U':
                        phiF = phiF - dot3(phiF, nrm).unsqueeze(-1) * nrm
                    vals.append(phiF)
                else:
                    raise NotImplementedError(kind)
            pieces.append((P['cellStart'], vals[0], vals[1], vals[2]))
        pieces.sort(key=lambda x: x[0])
        return (torch.cat([U] + [x[1] for x in pieces]), torch.cat([T] + [x[2] for x in pieces]),
                torch.cat([p] + [x[3] for x in pieces]))

    # ------------------------------------------------------------ gradients
    def grad_cell(self, phi):
        """Green-Gauss cell gradient by gather over the 6 cellFaces (adFVM/op.py:45-63).
        phi: (nCells, k) -> (nIC, k, 3)."""
        scalar = phi.shape[1] == 1
        g = None
        phic = phi[:self.nIC]
        for i in range(6):
            P = self.cellFaces[:, i]
            S = self.areas[P]
            N = self.normals[P]
            w = self.weights[P]
            O = self.cellOwner[:, i:i + 1].to(T64)
            N = 2 * N * O - N
            w = w + O - 2 * w * O
            phiP = phi[self.cellNeighbours[:, i]]
            phiF = phic * (-w + 1) + phiP * w
            if scalar:
                term = (phiF * S * N).unsqueeze(1)                      # (n,1,3)
            else:
                term = phiF.unsqueeze(-1) * (S * N).unsqueeze(1)         # outer -> (n,k,3)
            g = term if g is None else g + term
        return g / self.volumes.unsqueeze(-1)

    def grad_full(self, g):
        """Append ghost gradient rows: copies of the source cells (default boundary)."""
        return torch.cat([g, g[self.gradSrc]])

    # ------------------------------------------------------------ face physics
    @staticmethod
    def _recon(phiC, phiD, gradC, lw, qw):
        """interp.secondOrder (adFVM/interp.py:20-28). phi (n,k), grad (n,k,3)."""
        phiF = phiC + (phiD - phiC) * lw
        return phiF + (qw[:, None, 0] * gradC[..., 0] + qw[:, None, 1] * gradC[..., 1] + qw[:, None, 2] * gradC[..., 2])

    def _roe(self, pL, pR, TL, TR, UL, UR, rhoL, rhoR, rhoUL, rhoUR, rhoEL, rhoER, N):
        """riemann.eulerRoe (adFVM/riemann.py:21-70)."""
        g = self.gamma
        rhoUnL, rhoUnR = rhoL * dot3(UL, N).unsqueeze(-1), rhoR * dot3(UR, N).unsqueeze(-1)
        hL = g * pL / ((g - 1) * rhoL) + 0.5 * dot3(UL, UL).unsqueeze(-1)
        hR = g * pR / ((g - 1) * rhoR) + 0.5 * dot3(UR, UR).unsqueeze(-1)
        rhoFlux = 0.5 * (rhoUnL + rhoUnR)
        rhoUFlux = 0.5 * (rhoUnL * UL + rhoUnR * UR + (pL + pR) * N)
        rhoEFlux = 0.5 * (rhoUnL * hL + rhoUnR * hR)
        sL, sR = rhoL.sqrt(), rhoR.sqrt()
        divRho = sL + sR
        UF = (UL * sL + UR * sR) / divRho
        hF = (hL * sL + hR * sR) / divRho
        qF = 0.5 * dot3(UF, UF).unsqueeze(-1)
        a2F = (g - 1) * (hF - qF)
        aF = a2F.sqrt()
        UnF = dot3(UF, N).unsqueeze(-1)
        drho = rhoR - rhoL
        drhoU = rhoR * UR - rhoL * UL
        drhoE = (hR * rhoR - pR) - (hL * rhoL - pL)
        lam1, lam2, lam3 = UnF.abs(), (UnF + aF).abs(), (UnF - aF).abs()
        eps = 0.5 * (rhoUnL / rhoL - rhoUnR / rhoR).abs()
        eps = eps + 0.5 * ((g * pL / rhoL).sqrt() - (g * pR / rhoR).sqrt()).abs()
        eps = torch.where(eps < 0, eps - SMALL, eps + SMALL)          # stabilise
        lam1 = torch.where(lam1 < 2. * eps, .25 * lam1 * lam1 / eps + eps, lam1)
        lam2 = torch.where(lam2 < 2. * eps, .25 * lam2 * lam2 / eps + eps, lam2)
        lam3 = torch.where(lam3 < 2. * eps, .25 * lam3 * lam3 / eps + eps, lam3)
        abv1 = 0.5 * (lam2 + lam3)
        abv2 = 0.5 * (lam2 - lam3)
        abv3 = abv1 - lam1
        abv4 = (g - 1) * (qF * drho - dot3(UF, drhoU).unsqueeze(-1) + drhoE)
        abv5 = UnF * drho - dot3(drhoU, N).unsqueeze(-1)
        abv6 = abv3 * abv4 / a2F - abv2 * abv5 / aF
        abv7 = abv3 * abv5 - abv2 * abv4 / aF
        rhoFlux = rhoFlux - 0.5 * (lam1 * drho + abv6)
        rhoUFlux = rhoUFlux - 0.5 * (lam1 * drhoU + UF * abv6 - abv7 * N)
        rhoEFlux = rhoEFlux - 0.5 * (lam1 * drhoE + hF * abv6 - UnF * abv7)
        return rhoFlux, rhoUFlux, rhoEFlux

    def _lf(self, pL, pR, TL, TR, UL, UR, rhoL, rhoR, rhoUL, rhoUR, rhoEL, rhoER, N):
        """riemann.eulerLaxFriedrichs (adFVM/riemann.py:6-18)."""
        g = self.gamma
        UnL, UnR = dot3(UL, N).unsqueeze(-1), dot3(UR, N).unsqueeze(-1)
        cL = (g * pL / rhoL).sqrt()
        cR = (g * pR / rhoR).sqrt()
        aF = torch.maximum(UnL.abs() + cL, UnR.abs() + cR)
        rhoFlux = 0.5 * (rhoL * UnL + rhoR * UnR) - 0.5 * aF * (rhoR - rhoL)
        rhoUFlux = 0.5 * (rhoUL * UnL + rhoUR * UnR + (pL + pR) * N) - 0.5 * aF * (rhoUR - rhoUL)
        rhoEFlux = 0.5 * ((rhoEL + pL) * UnL + (rhoER + pR) * UnR) - 0.5 * aF * (rhoER - rhoEL)
        return rhoFlux, rhoUFlux, rhoEFlux

    def _riemann(self, name, *args):
        return self._roe(*args) if name == 'eulerRoe' else self._lf(*args)

    def _viscous(self, TL, TR, UL, UR, TF, UF, gradTF, gradUF, sl):
        """RCF.viscousFlux (adFVM/density.py:192-222) with op.snGrad (op.py:66-67).
        gradTF (n,3), gradUF (n,3,3)."""
        mu = self.mu(TF)
        kappa = mu * (self.Cp / self.Pr)
        D = self.deltasUnit[sl]
        N = self.normals[sl]
        d = self.deltas[sl]
        snT = (TR - TL) / d
        gT = gradTF + snT * D - dot3(gradTF, D).unsqueeze(-1) * D
        snU = (UR - UL) / d
        gUD = gradUF[..., 0] * D[:, None, 0] + gradUF[..., 1] * D[:, None, 1] + gradUF[..., 2] * D[:, None, 2]
        gU = gradUF + snU.unsqueeze(-1) * D.unsqueeze(1) - gUD.unsqueeze(-1) * D.unsqueeze(1)
        qF = kappa * dot3(gT, N).unsqueeze(-1)
        sym = gU + gU.transpose(1, 2)
        tmp2 = sym[..., 0] * N[:, None, 0] + sym[..., 1] * N[:, None, 1] + sym[..., 2] * N[:, None, 2]
        tmp3 = (gU[:, 0, 0] + gU[:, 1, 1] + gU[:, 2, 2]).unsqueeze(-1)
        sigma = mu * (tmp2 - 2. / 3 * tmp3 * N)
        return -sigma, -(qF + dot3(sigma, UF).unsqueeze(-1))

    def face_fluxes(self, U, T, p, gU, gT, gp):
        """Per-face flux (rho, rhoU, rhoE) and the CFL term maxaF for every face.

        U, T, p: (nCells, .) with ghosts; gU (nCells,3,3), gT/gp (nCells,1,3) with ghosts.
        Internal faces: RCF.flux (density.py:253-305); coupled patches the same, owner side
        only; characteristic patches flux(characteristic=True); other patches
        RCF.boundaryFlux (density.py:307-331)."""
        out_f = [None] * 4
        pieces = []
        # internal
        pieces.append((0, self.nIF, 'internal', None))
        for P in self.patches:
            kind = 'coupled' if P['coupled'] else ('characteristic' if P['characteristic'] else 'boundary')
            pieces.append((P['start'], P['start'] + P['n'], kind, P))
        res = {}
        for s, e, kind, P in pieces:
            if e == s:
                continue
            sl = slice(s, e)
            own, nb = self.owner[sl], self.neighbour[sl]
            N = self.normals[sl]
            TL, TR = T[own], T[nb]
            UL, UR = U[own], U[nb]
            if kind == 'boundary':
                pR = p[nb]
                rho, rhoU, rhoE = self.conservative(UR, TR, pR)
                Un = dot3(UR, N).unsqueeze(-1)
                rhoFlux = rho * Un
                rhoUFlux = rhoU * Un + pR * N
                rhoEFlux = (rhoE + pR) * Un
                vU, vE = self._viscous(TL, TR, UL, UR, TR, UR, gT[nb][:, 0], gU[nb], sl)
                TF, UF = TR, UR
            else:
                lw, qw = self.lw[sl], self.qw[sl]
                ULF = self._recon(UL, UR, gU[own], lw[:, 0:1], qw[:, 0])
                TLF = self._recon(TL, TR, gT[own], lw[:, 0:1], qw[:, 0])
                pLF = self._recon(p[own], p[nb], gp[own], lw[:, 0:1], qw[:, 0])
                rhoLF, rhoULF, rhoELF = self.conservative(ULF, TLF, pLF)
                if kind == 'characteristic':
                    URF, TRF, pRF = UR, TR, p[nb]
                    rhoRF, rhoURF, rhoERF = self.conservative(URF, TRF, pRF)
                    rhoFlux, rhoUFlux, rhoEFlux = self._riemann(
                        self.boundaryRiemann, pLF, pRF, TLF, TRF, ULF, URF, rhoLF, rhoRF, rhoULF, rhoURF, rhoELF, rhoERF, N)
                    TF, UF = TR, UR
                    gTF, gUF = gT[nb][:, 0], gU[nb]
                else:
                    URF = self._recon(UR, UL, gU[nb], lw[:, 1:2], qw[:, 1])
                    TRF = self._recon(TR, TL, gT[nb], lw[:, 1:2], qw[:, 1])
                    pRF = self._recon(p[nb], p[own], gp[nb], lw[:, 1:2], qw[:, 1])
                    rhoRF, rhoURF, rhoERF = self.conservative(URF, TRF, pRF)
                    rhoFlux, rhoUFlux, rhoEFlux = self._riemann(
                        self.riemann, pLF, pRF, TLF, TRF, ULF, URF, rhoLF, rhoRF, rhoULF, rhoURF, rhoELF, rhoERF, N)
                    UF = 0.5 * (ULF + URF)
                    TF = 0.5 * (TLF + TRF)
                    gTF = 0.5 * (gT[own] + gT[nb])[:, 0]
                    gUF = 0.5 * (gU[own] + gU[nb])
                vU, vE = self._viscous(TL, TR, UL, UR, TF, UF, gTF, gUF, sl)
            rhoUFlux = rhoUFlux + vU
            rhoEFlux = rhoEFlux + vE
            aF = (self.Cp * TF * (self.gamma - 1)).sqrt()
            maxaF = dot3(UF, N).unsqueeze(-1).abs() + aF
            res[s] = torch.cat([rhoFlux, rhoUFlux, rhoEFlux, maxaF], dim=1)   # (n, 6)
        order = sorted(res)
        return torch.cat([res[k] for k in order])                            # face order

    def accumulate(self, F):
        """op.div / op.absDiv collated into cells in the reference order. F (nF, 6) ->
        R (nIC, 5), dtc (nIC, 1)."""
        R = None
        dtc = None
        for k in range(6):
            f = self.accFaces[:, k]
            sideOwn = self.accOwnerSide[:, k:k + 1]
            Ff = F[f]
            wpf = self.wp[f]
            if self.nIF > 0:
                wnf = self.wnAbs[torch.where(f < self.nIF, f, torch.zeros_like(f))]
            else:                                         # no internal faces: owner sides only
                wnf = torch.zeros_like(wpf)
            w = torch.where(sideOwn, wpf, wnf)
            c5 = Ff[:, :5] * w
            c5 = torch.where(sideOwn, c5, -c5)            # phi*(-A/V_R) == -(phi*(A/V_R))
            cd = Ff[:, 5:6] * w
            R = c5 if R is None else R + c5
            dtc = cd if dtc is None else dtc + cd
        return R, dtc

    # ------------------------------------------------------------ objective
    _MESH_ATTR = {'linearWeights': 'lw', 'quadraticWeights': 'qw'}

    def meshTensor(self, name):
        """A mesh array as a torch tensor for objectives written as functions: the residual's
        own tensors (so that parameter leaves reach the objective too), else the mesh's."""
        a = getattr(self, self._MESH_ATTR.get(name, name), None)
        if isinstance(a, torch.Tensor):
            return a
        v = np.asarray(getattr(self.mesh, name))
        return torch.as_tensor(np.ascontiguousarray(v), dtype=torch.int64 if v.dtype.kind in 'iu' else T64)

    def objective_value(self, U, T, p):
        """Objective on the (ghost-completed) primitives of RK stage 1: a built-in kind, or a
        function objective([U, T, p], solver) as a case file gives it (density.py:354-357)."""
        o = self.objective
        nIC = self.nIC
        if callable(o):
            return o([U, T, p], self)
        if isinstance(o, dict):
            return self._vane(o, U, T, p)
        if o == 'none':
            return torch.zeros((), dtype=T64)
        if o == 'kinetic_energy':
            Uc, Tc, pc = U[:nIC], T[:nIC], p[:nIC]
            rho = pc / ((self.Cv * Tc) * (self.gamma - 1))
            v = 0.5 * rho * dot3(Uc, Uc).unsqueeze(-1) * self.volumes
            return torch.cumsum(v.reshape(-1), 0)[-1]
        if o == 'sum_T':
            return torch.cumsum((T[:nIC] * 1).reshape(-1), 0)[-1]
        if o.startswith('drag:'):
            name = o.split(':', 1)[1]
            P = next(P for P in self.patches if P['name'] == name)
            sl = slice(P['start'], P['start'] + P['n'])
            own, nb = self.owner[sl], self.neighbour[sl]
            U0 = U[nb][:, 0:1]
            U0i = U[own][:, 0:1]
            p0 = p[nb]
            T0 = T[nb]
            nx = self.normals[sl][:, 0:1]
            mungUx = self.mu(T0) * (U0 - U0i) / self.deltas[sl]
            drag = (p0 * nx - mungUx) * self.areas[sl]
            return torch.cumsum(drag.reshape(-1), 0)[-1]
        raise ValueError(o)

    def _vane(self, v, U, T, p):
        """adFVM/objectives/vane.py:7-60, 118-131: a * pressure loss over the plane cells
        (objectivePressureLoss / objectivePressureLossWeighting) + b * weighted wall heat
        transfer (objectiveHeatTransfer / objectiveHeatTransferWeighting)."""
        g = self.gamma
        cells = _t(v['planeCells'], torch.int64).reshape(-1)
        areas = _t(v['planeAreas']).reshape(-1, 1)
        n = [float(x) for x in v['normal']]
        pi, Ti, Ui = p[cells], T[cells], U[cells]
        rhoi = pi / (self.Cv * Ti * (g - 1))
        ci = (g * pi / rhoi).sqrt()
        rhoUni = sum([rhoi * Ui[:, i:i + 1] * n[i] for i in range(3)])
        w = torch.cumsum((rhoUni * areas).reshape(-1), 0)[-1]
        Umagi = dot3(Ui, Ui).unsqueeze(-1)
        Mi = Umagi.sqrt() / ci
        pti = pi * (1 + 0.5 * (g - 1) * Mi * Mi) ** (g / (g - 1))
        pl = (v['ptin'] - pti) * rhoUni * areas / v['ptin']
        pl = torch.cumsum((pl / w).reshape(-1), 0)[-1]
        ht = torch.zeros((), dtype=T64)
        w2 = 0.0
        k = self.Cp * self.mu(torch.tensor(float(v['Tw']), dtype=T64)) / self.Pr
        for P in self.patches:
            if P['name'] not in v['heat']:
                continue
            sl = slice(P['start'], P['start'] + P['n'])
            wt = _t(v['heat'][P['name']]).reshape(-1, 1)
            w2 = w2 + float((self.areas[sl] * wt).sum())
        for P in self.patches:
            if P['name'] not in v['heat']:
                continue
            sl = slice(P['start'], P['start'] + P['n'])
            wt = _t(v['heat'][P['name']]).reshape(-1, 1)
            Tin = T[self.owner[sl]]
            dtdn = (v['Tw'] - Tin) / self.deltas[sl]
            ht = ht + torch.cumsum((k * dtdn * self.areas[sl] * wt / w2).reshape(-1), 0)[-1]
        return v['a'] * pl + v['b'] * ht

    # ------------------------------------------------------------ residual and step
    def equation(self, rho, rhoU, rhoE, want_objective=False):
        """RCF.equation (adFVM/density.py:339-414): returns (R(5 cols), dtc field, obj)."""
        U, T, p = self.primitive(rho, rhoU, rhoE)
        U, T, p = self.ghosts(U, T, p)
        obj = self.objective_value(U, T, p) if want_objective else None
        gU = self.grad_full(self.grad_cell(U))
        gT = self.grad_full(self.grad_cell(T))
        gp = self.grad_full(self.grad_cell(p))
        F = self.face_fluxes(U, T, p, gU, gT, gp)
        R, dtc = self.accumulate(F)
        return R, dtc, obj

    def step(self, rho, rhoU, rhoE, dt, S=None):
        """One SSP-RK3 step (adFVM/timestep.py:17-55). Returns (rhoN, rhoUN, rhoEN, dtc, obj)
        with dtc = max over cells of the stage-1 CFL sum and obj the stage-1 objective
        (density.py:405-413)."""
        alpha = np.array([[1, 0, 0], [3. / 4, 1. / 4, 0], [1. / 3, 0, 2. / 3]])
        beta = np.array([[1, 0, 0], [0, 1. / 4, 0], [0, 0, 2. / 3]])
        u0 = torch.cat([rho, rhoU, rhoE], dim=1)
        if S is None:
            S = torch.zeros_like(u0)
        elif isinstance(S, (list, tuple)):
            S = torch.cat([torch.as_tensor(s, dtype=T64).reshape(len(u0), -1) for s in S], dim=1)
        fields = [u0]
        dtc = obj = None
        for i in range(3):
            u = fields[i]
            R, dtcf, o = self.equation(u[:, 0:1], u[:, 1:4], u[:, 4:5], want_objective=(i == 1))
            if i == 1:
                dtc = dtcf.max()
                obj = o
            cur = None
            for j in range(i + 1):
                term = float(alpha[i, j]) * fields[j]
                cur = term if cur is None else cur + term
            cur = cur + (float(-beta[i, i]) * (R - S)) * dt
            fields.append(cur)
        u = fields[-1]
        return u[:, 0:1], u[:, 1:4], u[:, 4:5], dtc, obj


def run(problem, rho, rhoU, rhoE, nSteps, dt, CFL=None, stepFactor=1.0, fixed=True, endTime=np.inf, S=None):
    """Solver.run time loop (adFVM/solver.py:296-373) without IO: returns the list of states
    and the per-step (dt, dtc, obj) record."""
    states = [(rho, rhoU, rhoE)]
    record = []
    t = 0.0
    for n in range(nSteps):
        rho, rhoU, rhoE, dtc, obj = problem.step(rho, rhoU, rhoE, dt, S)
        record.append((dt, float(dtc), float(obj)))
        states.append((rho, rhoU, rhoE))
        t = round(t + dt, 12)
        if not fixed:
            dt = min(2 * CFL / float(dtc), dt * stepFactor, endTime - t)
    return states, record


def vjp_step(problem, rho, rhoU, rhoE, dt, S, seeds, obja=1.0):
    """Adjoint of one step with dt held fixed: d(sum(seeds*outputs) + obja*obj)/d(inputs).
    Returns (rhoa, rhoUa, rhoEa, S_a) where S_a stacks the source gradients (nIC, 5)."""
    x = [t.detach().clone().requires_grad_(True) for t in (rho, rhoU, rhoE)]
    if S is None:
        S = torch.zeros((len(rho), 5), dtype=T64)
    elif isinstance(S, (list, tuple)):
        S = torch.cat([torch.as_tensor(s, dtype=T64).reshape(len(rho), -1) for s in S], dim=1)
    S = S.detach().clone().requires_grad_(True)
    out = problem.step(x[0], x[1], x[2], dt, S)
    J = (out[0] * seeds[0]).sum() + (out[1] * seeds[1]).sum() + (out[2] * seeds[2]).sum()
    if obja != 0:
        J = J + obja * out[4]
    g = torch.autograd.grad(J, x + [S], allow_unused=True)
    g = [torch.zeros_like(v) if gi is None else gi for gi, v in zip(g, x + [S])]
    return g[0], g[1], g[2], g[3]


MESH_GRAD_FIELDS = ('areas', 'volumesL', 'volumesR', 'weights', 'deltas', 'normals', 'deltasUnit',
                    'linearWeights', 'quadraticWeights', 'volumes')
_ATTR = {'linearWeights': 'lw', 'quadraticWeights': 'qw'}


def with_parameter_leaves(problem, parameters, values=None):
    """A copy of ``problem`` whose parameters are autograd leaves read directly by the residual:
    'mesh' - the ten Mesh.gradFields tensors (adFVM/mesh.py:28-31; volumesL and volumesR are
    inputs of their own, as in the reference's map, apps/adjoint.py:108-110); ('BCs', field,
    patch, key) - one boundary input (apps/adjoint.py:111-118: fixedValue 'value', CBC_UPT
    U0/T0/p0 and CBC_TOTAL_PT direction/Tt/pt of the p field, density.py:333-337). values:
    the parameters' values (default: the problem's own). Returns (copy, leaves)."""
    import copy
    P = copy.copy(problem)
    P.patches = [dict(e) for e in problem.patches]
    if parameters == 'mesh':
        leaves = []
        for i, k in enumerate(MESH_GRAD_FIELDS):
            base = getattr(problem, _ATTR.get(k, k)) if values is None else \
                torch.as_tensor(values[i], dtype=T64).reshape(getattr(problem, _ATTR.get(k, k)).shape)
            t = base.detach().clone().requires_grad_(True)
            setattr(P, _ATTR.get(k, k), t)
            leaves.append(t)
        P.wp = P.areas / P.volumesL
        P.wnAbs = P.areas[:P.nIF] / P.volumesR
        for e in P.patches:
            if 'Tt' in e and 'direction' not in e['bc']['p']:
                e['direction'] = P.normals[e['start']:e['start'] + e['n']]
        return P, leaves
    _, phi, patch, key = parameters
    e = next(e for e in P.patches if e['name'] == patch)
    kind = e['kinds'][phi]
    if kind == 'fixedValue' and key == 'value':
        attr = phi + '_fixed'
    elif kind in ('CBC_UPT', 'CBC_TOTAL_PT') and phi == 'p':
        attr = key
    elif kind in ('CBC_UPT', 'CBC_TOTAL_PT'):
        # the U and T fields' copies of a characteristic input are never read by the step
        n = e['n']
        return P, [torch.zeros((n, 3 if key in ('U0', 'direction') else 1), dtype=T64, requires_grad=True)]
    else:
        raise ValueError(parameters)
    base = e[attr] if values is None else torch.as_tensor(values[0], dtype=T64).reshape(e[attr].shape)
    t = base.detach().clone().requires_grad_(True)
    e[attr] = t
    return P, [t]


def vjp_step_params(problem, rho, rhoU, rhoE, dt, S, seeds, obja=1.0, parameters='mesh'):
    """vjp_step that also returns the gradients with respect to ``parameters`` (see
    with_parameter_leaves): (rhoa, rhoUa, rhoEa, S_a, [parameter gradients])."""
    P, leaves = with_parameter_leaves(problem, parameters)
    x = [t.detach().clone().requires_grad_(True) for t in (rho, rhoU, rhoE)]
    if S is None:
        S = torch.zeros((len(rho), 5), dtype=T64)
    elif isinstance(S, (list, tuple)):
        S = torch.cat([torch.as_tensor(s, dtype=T64).reshape(len(rho), -1) for s in S], dim=1)
    S = S.detach().clone().requires_grad_(True)
    out = P.step(x[0], x[1], x[2], dt, S)
    J = (out[0] * seeds[0]).sum() + (out[1] * seeds[1]).sum() + (out[2] * seeds[2]).sum()
    if obja != 0:
        J = J + obja * out[4]
    ins = x + [S] + list(leaves)
    g = torch.autograd.grad(J, ins, allow_unused=True)
    g = [torch.zeros_like(v) if gi is None else gi for gi, v in zip(g, ins)]
    return g[0], g[1], g[2], g[3], g[4:]


def adjoint_energy(volumes, gamma, rhoa, rhoUa, rhoEa, rho, rhoU, rhoE):
    """cmesh.computeEnergy (adFVM/cpp/cmesh.cpp:342-425) restated in numpy."""
    g = gamma
    v = np.asarray(volumes).reshape(-1)
    rho = np.asarray(rho).reshape(-1)
    rhoE = np.asarray(rhoE).reshape(-1)
    rhoU = np.asarray(rhoU).reshape(-1, 3)
    u1, u2, u3 = rhoU[:, 0] / rho, rhoU[:, 1] / rho, rhoU[:, 2] / rho
    q2 = u1 * u1 + u2 * u2 + u3 * u3
    p = (rhoE - rho * q2 / 2) * (g - 1)
    H = g * p / (rho * (g - 1)) + q2 / 2
    a = np.asarray(rhoUa).reshape(-1, 3)
    w1, w2, w3, w4, w5 = (np.asarray(rhoa).reshape(-1) / v, a[:, 0] / v, a[:, 1] / v, a[:, 2] / v,
                          np.asarray(rhoEa).reshape(-1) / v)
    A11, A12, A13, A14, A15 = rho, rho * u1, rho * u2, rho * u3, rhoE
    A22, A23, A24, A25 = rho * u1 * u1 + p, rho * u1 * u2, rho * u1 * u3, rho * H * u1
    A33, A34, A35 = rho * u2 * u2 + p, rho * u2 * u3, rho * H * u2
    A44, A45 = rho * u3 * u3 + p, rho * H * u3
    A55 = rho * H * H - g * p * p / (rho * (g - 1))
    e = (A11 * w1 * w1 + A22 * w2 * w2 + A33 * w3 * w3 + A44 * w4 * w4 + A55 * w5 * w5 +
         2 * (A12 * w1 * w2 + A13 * w1 * w3 + A14 * w1 * w4 + A15 * w1 * w5 + A23 * w2 * w3 + A24 * w2 * w4 +
              A25 * w2 * w5 + A34 * w3 * w4 + A35 * w3 * w5 + A45 * w4 * w5)) * v
    return float(np.sum(e))


# ---------------------------------------------------------------- adjoint stabilisation

def _max_eig_sym(MS):
    """Largest eigenvalue of each symmetric 5x5 (LAPACK's ascending w[4], scaling.cpp:84-104)."""
    return np.linalg.eigvalsh(MS)[:, -1]


def viscosity_matrix(kind, g, U, T, p, Cv, gradU, divU, gradp, gradc, Uref=33., pref=1e5):
    """The symmetric part MS = (M + M^T)/2 of getMaxEigenvalue (adFVM/postpro.py:549-634) per
    cell, numpy float64: U (n,3), T, p (n,), gradU (n,3,3), divU (n,), gradp, gradc (n,3)."""
    n = len(T)
    rho = p / ((Cv * T) * (g - 1))
    c = np.sqrt(g * p / rho)
    gradrho = g * (gradp - (c * p)[:, None]) / (c * c)[:, None]
    Z = np.zeros(n)
    M = np.zeros((n, 5, 5))
    g1 = g - 1
    if kind == 'turkel':
        M1 = np.zeros((n, 5, 5))
        for k in range(5):
            M1[:, k, k] = divU
        for k in range(3):
            M1[:, 0, 1 + k] = gradc[:, k]
            M1[:, 1 + k, 0] = gradc[:, k]
        tmp1 = gradp / (rho * c)[:, None]
        tmp2 = g1 * gradp / (2 * rho * c)[:, None]
        tmp3 = gradp * pref / (2 * g * p * rho * Uref)[:, None]
        tmp4 = (gradp - (c * c)[:, None] * gradrho) * Uref / pref
        M2 = np.zeros((n, 5, 5))
        M2[:, 0, 0] = g1 * divU / 2
        M2[:, 0, 1:4] = tmp1
        M2[:, 0, 4] = divU * pref / (2 * rho * c * Uref)
        M2[:, 1:4, 0] = tmp2
        M2[:, 1:4, 1:4] = gradU
        M2[:, 1:4, 4] = tmp3
        M2[:, 4, 1:4] = tmp4
        M2[:, 4, 4] = g1 * divU / 2
        M = M1 / 2 - M2
    elif kind == 'abarbanel':
        sg, sg1 = np.sqrt(g), np.sqrt(g1)
        b = c / sg
        a = sg1 * c / sg
        gradb = gradc / sg
        grada = gradc * sg1 / sg
        M1 = np.zeros((n, 5, 5))
        for k in range(5):
            M1[:, k, k] = divU
        for k in range(3):
            M1[:, 0, 1 + k] = gradb[:, k]
            M1[:, 1 + k, 0] = gradb[:, k]
            M1[:, 1 + k, 4] = grada[:, k]
            M1[:, 4, 1 + k] = grada[:, k]
        tmp1 = b[:, None] * gradrho / rho[:, None]
        tmp2 = a[:, None] * gradp / (2 * p)[:, None]
        tmp3 = 2 * grada / g1
        M2 = np.zeros((n, 5, 5))
        M2[:, 0, 1:4] = tmp1
        M2[:, 0, 4] = sg1 * divU / 2
        M2[:, 1:4, 1:4] = gradU
        M2[:, 1:4, 4] = tmp2
        M2[:, 4, 1:4] = tmp3
        M2[:, 4, 4] = g1 * divU / 2
        M = M1 / 2 - M2
    else:
        raise ValueError(kind)
    del Z
    return (M + np.swapaxes(M, 1, 2)) / 2


def adjoint_viscosity(problem, rho, rhoU, rhoE, kind, scaling, Uref=33., pref=1e5):
    """postpro.computeAdjointViscosity (adFVM/postpro.py:491-697): the per-cell viscosity
    M_2norm (max eigenvalue of the symmetrised 5x5 of each cell, normalised to
    scaling * M / sqrt(sum M^2 V / sum V)) and its central interpolation DT on every face.
    Returns (M_2norm (nCells,) with ghost values, DT (nFaces,)), numpy float64."""
    P = problem
    g = P.gamma
    Rg = P.Cp - P.Cv
    with torch.no_grad():
        U, T, p = P.ghosts(*P.primitive(torch.as_tensor(rho), torch.as_tensor(rhoU), torch.as_tensor(rhoE)))
    U, T, p = U.numpy(), T.numpy().reshape(-1), p.numpy().reshape(-1)
    own, nbr = P.owner.numpy(), P.neighbour.numpy()
    w = P.weights.numpy().reshape(-1)
    A = P.areas.numpy().reshape(-1)
    N = P.normals.numpy()
    V = P.volumes.numpy().reshape(-1)
    nIC, nIF, nF = P.nIC, P.nIF, P.nF
    # face values (postpro.py:500-516): central on internal and coupled faces, ghost values on
    # the other boundary faces
    UF = np.zeros((nF, 3)); pF = np.zeros(nF); cF = np.zeros(nF)
    central = np.zeros(nF, bool)
    central[:nIF] = True
    for Pt in P.patches:
        if Pt['coupled']:
            central[Pt['start']:Pt['start'] + Pt['n']] = True
    cc = np.sqrt(g * T * Rg)
    wc = w[:, None]
    UF[central] = (U[own] * wc + U[nbr] * (1 - wc))[central]
    pF[central] = (p[own] * w + p[nbr] * (1 - w))[central]
    cF[central] = (cc[nbr] * (1 - w) + cc[own] * w)[central]
    UF[~central] = U[nbr][~central]
    pF[~central] = p[nbr][~central]
    cF[~central] = np.sqrt(g * T[nbr][~central] * Rg)
    # op.grad / op.div (op.py:12-43): + A/V_L to the owner, - A/V_R to the internal neighbour,
    # accumulated in collate order (internal faces, then the patches in sortedPatches order)
    gradU = np.zeros((nIC, 3, 3)); divU = np.zeros(nIC); gradp = np.zeros((nIC, 3)); gradc = np.zeros((nIC, 3))
    acc = P.accFaces.numpy()
    side = P.accOwnerSide.numpy()
    for s in range(6):
        f = acc[:, s]
        sgn = np.where(side[:, s], 1.0, -1.0)
        wgt = sgn * A[f] / V
        gradU += UF[f][:, :, None] * N[f][:, None, :] * wgt[:, None, None]
        divU += (UF[f] * N[f]).sum(axis=1) * wgt
        gradp += (pF[f][:, None] * N[f]) * wgt[:, None]
        gradc += (cF[f][:, None] * N[f]) * wgt[:, None]
    if kind == 'uniform':
        M = np.ones(nIC)
    else:
        MS = viscosity_matrix(kind, g, U[:nIC], T[:nIC], p[:nIC], P.Cv, gradU, divU, gradp, gradc, Uref, pref)
        M = _max_eig_sym(MS)
    Vt = V.sum()
    Nrm = (M * M * V / Vt).sum()
    M = M * scaling / np.sqrt(Nrm)
    # ghost values by the default boundary (cyclic: partner's owner, others: owner) and the
    # central interpolation to every face (postpro.py:680-697)
    Mc = np.concatenate([M, M[P.gradSrc.numpy()]])
    DT = Mc[own] * w + Mc[nbr] * (1 - w)
    return Mc, DT


def viscosity_solve(problem, DT, dt, rhoa, rhoUa, rhoEa):
    """postpro.viscositySolver (adFVM/postpro.py:699-718) with the implicit heat equation of
    apply_adjoint_viscosity (scaling.cpp:135-159, matop_petsc.cpp:230-372) solved exactly: per
    component x of the adjoint per unit volume,
        (1 + sum_k DTF_k dt/V) x_c - sum_k DTF_k dt/V x_nbr(k) = x0_c,  DTF = A DT / delta,
    over the faces k of cell c that have an internal neighbour (cellNeighboursMatOp >= 0).
    Returns the smoothed (rhoa, rhoUa, rhoEa) times the volumes again."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    P = problem
    nIC = P.nIC
    V = P.volumes.numpy().reshape(-1)
    A = P.areas.numpy().reshape(-1)
    dl = P.deltas.numpy().reshape(-1)
    DTF = A * np.asarray(DT).reshape(-1) / dl
    cf = P.cellFaces.numpy()
    cn = P.cellNeighbours.numpy()
    rows, cols, vals = [], [], []
    diag = np.ones(nIC)
    for k in range(6):
        f = cf[:, k]
        nb = cn[:, k]
        ok = nb < nIC
        coef = DTF[f] * dt / V
        diag += np.where(ok, coef, 0.0)
        rows.append(np.arange(nIC)[ok]); cols.append(nb[ok]); vals.append(-coef[ok])
    Amat = sp.csr_matrix((np.concatenate(vals + [diag]), (np.concatenate(rows + [np.arange(nIC)]),
                                                         np.concatenate(cols + [np.arange(nIC)]))), shape=(nIC, nIC))
    X = np.concatenate([np.asarray(rhoa).reshape(nIC, 1), np.asarray(rhoUa).reshape(nIC, 3),
                        np.asarray(rhoEa).reshape(nIC, 1)], axis=1) / V[:, None]
    lu = spla.splu(Amat.tocsc())
    Y = np.stack([lu.solve(X[:, k]) for k in range(5)], axis=1) * V[:, None]
    return Y[:, 0:1], Y[:, 1:4], Y[:, 4:5]
