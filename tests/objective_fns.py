"""Objectives written as functions objective([U, T, p], solver), the form of a reference case
file's objective (adFVM/density.py:354-357; e.g. templates/cylinder_test.py:9-37), in torch:
the same code runs on the oracle's CPU tensors and on the GPU solver's CUDA tensors."""


def kinetic_energy(fields, solver):
    """sum_c 0.5 rho |U|^2 V over the internal cells (templates/box.py:10-16 pattern)."""
    U, T, p = fields
    n = solver.mesh.nInternalCells
    rho = p[:n] / ((solver.Cv * T[:n]) * (solver.gamma - 1))
    V = solver.meshTensor('volumes').reshape(-1, 1)
    return (0.5 * rho * (U[:n] * U[:n]).sum(dim=1, keepdim=True) * V).sum()


def drag(patch):
    """The wall drag of templates/cylinder_test.py:9-19 on ``patch``."""
    def objective(fields, solver):
        U, T, p = fields
        b = solver.mesh.boundary[patch]
        s, n = int(b['startFace']), int(b['nFaces'])
        own = solver.meshTensor('owner').reshape(-1)[s:s + n]
        nb = solver.meshTensor('neighbour').reshape(-1)[s:s + n]
        U0, U0i, p0, T0 = U[nb][:, 0:1], U[own][:, 0:1], p[nb], T[nb]
        nx = solver.meshTensor('normals').reshape(-1, 3)[s:s + n, 0:1]
        dl = solver.meshTensor('deltas').reshape(-1, 1)[s:s + n]
        A = solver.meshTensor('areas').reshape(-1, 1)[s:s + n]
        return ((p0 * nx - solver.mu(T0) * (U0 - U0i) / dl) * A).sum()
    return objective


def pressure_mix(patch):
    """A made-up objective that reads ghost cells and several mesh tensors: the volume-weighted
    mean square pressure of the internal cells plus the area-weighted mean ghost pressure and
    temperature of ``patch``."""
    def objective(fields, solver):
        U, T, p = fields
        m = solver.mesh
        n = m.nInternalCells
        V = solver.meshTensor('volumes').reshape(-1, 1)
        b = m.boundary[patch]
        s, k = int(b['startFace']), int(b['nFaces'])
        g0 = n + s - m.nInternalFaces
        A = solver.meshTensor('areas').reshape(-1, 1)[s:s + k]
        inner = (p[:n] * p[:n] * V).sum() / V.sum()
        ghost = ((p[g0:g0 + k] + 300.0 * T[g0:g0 + k]) * A).sum() / A.sum()
        return 1e-10 * inner + 1e-5 * ghost
    return objective
