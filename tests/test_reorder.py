"""The cell renumbering's oracle (oracle/c/reorder_oracle.c): pinned to SciPy's
reverse_cuthill_mckee (the same order where SciPy starts from the same cell - meshes whose
least-degree cell is unique in SciPy's start rule - and the same bandwidth on the periodic
boxes, whose cells all have six neighbours), and checked to be a pure renumbering: the
reordered mesh has the same geometry cell for cell and the same residual, cell for cell."""
import numpy as np
import pytest
import torch
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import reverse_cuthill_mckee

from adfvm_gb300 import cases, meshgen
from adfvm_gb300.mesh import Mesh
from oracle import c_ref, torch_ref


def _graph(md):
    P, F, O, N, B = md
    O, N = np.asarray(O), np.asarray(N)
    nIC, nIF = int(O.max()) + 1, len(N)
    r, c = [O[:nIF]], [N]
    for b in B.values():
        if b['type'] == 'cyclic':
            q = B[b['neighbourPatch']]
            s, n = b['startFace'], b['nFaces']
            r.append(O[s:s + n])
            c.append(O[q['startFace']:q['startFace'] + n])
    r, c = np.concatenate(r), np.concatenate(c)
    rows, cols = np.concatenate([r, c]), np.concatenate([c, r])
    return csr_matrix((np.ones(len(rows), np.int8), (rows, cols)), shape=(nIC, nIC))


def _scipy_ids(md):
    g = _graph(md)
    perm = reverse_cuthill_mckee(g, symmetric_mode=True)
    ids = np.empty(g.shape[0], np.int64)
    ids[perm] = np.arange(g.shape[0])
    coo = g.tocoo()
    return ids, int(np.abs(ids[coo.row] - ids[coo.col]).max())


@pytest.mark.parametrize('make', [lambda: meshgen.cylinder_ogrid(32, 16), lambda: meshgen.sod_tube(50),
                                  lambda: meshgen.channel(16, 8), lambda: meshgen.channel(24, 10, stretch=0.3)])
def test_same_order_as_scipy_rcm(make):
    md = make()
    ids, bw = _scipy_ids(md)
    _, cn, _, (b0, b1) = c_ref.mesh_reorder(md)
    assert np.array_equal(cn, ids)
    assert b1 == bw


@pytest.mark.parametrize('n', [8, 16, 32])
def test_same_bandwidth_as_scipy_rcm_on_shuffled_boxes(n):
    md = meshgen.periodic_box(n, reorder=False)
    _, bw = _scipy_ids(md)
    _, cn, _, (b0, b1) = c_ref.mesh_reorder(md)
    assert b1 == bw and b0 > 5 * b1


def test_reordered_mesh_is_a_renumbering():
    md = meshgen.periodic_box(10, reorder=False)
    md2, cn, fold, _ = c_ref.mesh_reorder(md)
    P, F, O, N, B = md
    P2, F2, O2, N2, B2 = md2
    nIC, nIF = len(cn), len(N)
    assert np.array_equal(np.sort(cn), np.arange(nIC))
    # upper-triangular internal faces in (owner, neighbour) order
    assert np.all(O2[:nIF] < N2)
    key = O2[:nIF].astype(np.int64) * nIC + N2
    assert np.all(np.diff(key) > 0)
    # the face map: the same face between the same cells, flipped faces with p2 p1 p0 p3
    old = np.where(fold < 0, ~fold, fold)
    flip = fold < 0
    assert np.array_equal(np.sort(old), np.arange(len(O)))
    a, b = cn[O[old[:nIF]]], cn[N[old[:nIF]]]
    assert np.array_equal(np.where(flip[:nIF], b, a), O2[:nIF])
    assert np.array_equal(np.where(flip[:nIF], a, b), N2)
    assert np.array_equal(F2[flip], F[old[flip]][:, [0, 3, 2, 1, 4]])
    assert np.array_equal(F2[~flip], F[old[~flip]])
    # the reader's cell count: the last cell owns a boundary face
    assert int(O2.max()) == nIC - 1
    # geometry cell for cell (faces flipped exactly negate their normal; only the order of the
    # sums over a face's points changes)
    m0, m1 = Mesh.create(md), Mesh.create(md2)
    assert np.abs(m1.volumes[cn] - m0.volumes).max() <= 1e-13 * m0.volumes.max()
    assert np.abs(m1.cellCentres[cn] - m0.cellCentres[:nIC]).max() <= 1e-13
    n0 = m0.normals[old]
    assert np.abs(np.where(flip[:, None], -n0, n0) - m1.normals).max() == 0.0


def test_residual_is_renumbered():
    """One FP64 step of the torch oracle on the shuffled box and on its renumbering: the same
    state cell for cell (to the rounding of the reordered sums)."""
    case = cases.box(6, seed=0)
    md = meshgen.periodic_box(6, reorder=False)
    md2, cn, _, _ = c_ref.mesh_reorder(md)
    m0, m1 = Mesh.create(md), Mesh.create(md2)
    p0 = torch_ref.Problem(m0, case.bc, case.config, case.objective)
    p1 = torch_ref.Problem(m1, case.bc, case.config, case.objective)
    rng = np.random.default_rng(5)
    nIC = len(cn)
    rho = 1.2 * (1 + 0.01 * rng.standard_normal((nIC, 1)))
    rhoU = rng.standard_normal((nIC, 3))
    rhoE = 2.6e5 * (1 + 0.01 * rng.standard_normal((nIC, 1)))
    x0 = [torch.as_tensor(a) for a in (rho, rhoU, rhoE)]
    x1 = [torch.zeros_like(t) for t in x0]
    for a, b in zip(x1, x0):
        a[torch.as_tensor(cn, dtype=torch.long)] = b
    dt = 1e-6
    r0 = p0.step(x0[0], x0[1], x0[2], dt)
    r1 = p1.step(x1[0], x1[1], x1[2], dt)
    for i in range(3):
        back = r1[i][torch.as_tensor(cn, dtype=torch.long)]
        assert float((back - r0[i]).abs().max()) <= 1e-12 * float(r0[i].abs().max())
