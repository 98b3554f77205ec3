"""Hex mesh generators in OpenFOAM polyMesh layout.

Each generator returns ``(points, faces, owner, neighbour, boundary)`` exactly as the
reference's mesh reader hands them to ``Mesh.build`` (adFVM/mesh.py:177-204, 84-127):

* ``points``  float64 (nPoints, 3)
* ``faces``   int32 (nFaces, 5): point count (always 4) followed by 4 point ids; the
  right-hand rule over the first three points gives a normal pointing out of the owner
  cell (the normal formula of adFVM/cpp/cmesh.cpp:72-87).
* ``owner``   int32 (nFaces,), ``neighbour`` int32 (nInternalFaces,); internal faces come
  first, in upper-triangular order (sorted by owner, then neighbour, owner < neighbour),
  then the boundary faces grouped by patch.
* ``boundary`` dict patchID -> {'type', 'startFace', 'nFaces'[, 'neighbourPatch']}.

The meshes are the workloads named for this path: the 1-D Sod tube, the jittered periodic
box (cells shuffled, then reverse-Cuthill-McKee reordered) and the 2-D cylinder O-grid
extruded one cell.
"""
import numpy as np
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import reverse_cuthill_mckee


def _quad_x(pid, i, j, k):
    # normal +x: (j..j+1) then (k..k+1)
    return [pid(i, j, k), pid(i, j + 1, k), pid(i, j + 1, k + 1), pid(i, j, k + 1)]


def _quad_y(pid, i, j, k):
    # normal +y
    return [pid(i, j, k), pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j, k)]


def _quad_z(pid, i, j, k):
    # normal +z
    return [pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k)]


def _assemble(cellsA, cellsB, quads, bpatches):
    """Order internal faces upper-triangularly and orient them owner -> neighbour.

    cellsA/cellsB: cell ids on the minus/plus side of each internal face whose quad
    (point ids, normal pointing minus -> plus) is given in ``quads``.
    bpatches: list of (name, type, owner_cells, quads_outward, extra) in file order.
    """
    cellsA = np.asarray(cellsA, np.int64)
    cellsB = np.asarray(cellsB, np.int64)
    quads = np.asarray(quads, np.int64).reshape(-1, 4)
    flip = cellsA > cellsB
    own = np.where(flip, cellsB, cellsA)
    nbr = np.where(flip, cellsA, cellsB)
    q = quads.copy()
    # reversing the point order flips the normal
    q[flip] = q[flip][:, ::-1]
    order = np.lexsort((nbr, own))
    own, nbr, q = own[order], nbr[order], q[order]
    faces = [q]
    owners = [own]
    boundary = {}
    start = len(own)
    for name, ptype, bown, bq, extra in bpatches:
        bown = np.asarray(bown, np.int64)
        bq = np.asarray(bq, np.int64).reshape(-1, 4)
        faces.append(bq)
        owners.append(bown)
        patch = {'type': ptype, 'startFace': int(start), 'nFaces': int(len(bown))}
        patch.update(extra)
        boundary[name] = patch
        start += len(bown)
    q = np.concatenate(faces)
    faces = np.empty((len(q), 5), np.int32)
    faces[:, 0] = 4
    faces[:, 1:] = q
    owner = np.concatenate(owners).astype(np.int32)
    neighbour = nbr.astype(np.int32)
    return faces, owner, neighbour, boundary


def sod_tube(n=1000, length=1.0, side_type='empty'):
    """1-D shock tube: n x 1 x 1 hex cells on x in [0, length], y, z in [0, length/n].

    Patches (file order): ``left`` and ``right`` ends (type ``patch``), ``sides``
    (``empty`` or ``symmetryPlane``) holding the 4n lateral faces.
    """
    h = length / n
    xs = np.arange(n + 1, dtype=np.float64) * h
    xs[-1] = length
    # points (i, j, k) with j, k in {0, 1}
    pid = lambda i, j, k: i + (n + 1) * (j + 2 * k)
    P = np.zeros(((n + 1) * 4, 3))
    for k in range(2):
        for j in range(2):
            for i in range(n + 1):
                P[pid(i, j, k)] = (xs[i], j * h, k * h)
    cell = lambda i: i
    A, B, Q = [], [], []
    for i in range(1, n):
        A.append(cell(i - 1)); B.append(cell(i)); Q.append(_quad_x(pid, i, 0, 0))
    left = (cell(0), _quad_x(pid, 0, 0, 0)[::-1])
    right = (cell(n - 1), _quad_x(pid, n, 0, 0))
    sides_own, sides_q = [], []
    for i in range(n):
        sides_own += [cell(i)] * 4
        sides_q.append(_quad_y(pid, i, 0, 0)[::-1])   # y = 0, outward -y
        sides_q.append(_quad_y(pid, i, 1, 0))         # y = h, outward +y
        sides_q.append(_quad_z(pid, i, 0, 0)[::-1])   # z = 0, outward -z
        sides_q.append(_quad_z(pid, i, 0, 1))         # z = h, outward +z
    bp = [('left', 'patch', [left[0]], left[1], {}),
          ('right', 'patch', [right[0]], right[1], {}),
          ('sides', side_type, sides_own, sides_q, {})]
    faces, owner, neighbour, boundary = _assemble(A, B, Q, bp)
    return P, faces, owner, neighbour, boundary


def _rcm_permutation(nc, own, nbr):
    """new_id[old] from reverse Cuthill-McKee on the cell adjacency graph."""
    rows = np.concatenate([own, nbr])
    cols = np.concatenate([nbr, own])
    g = csr_matrix((np.ones(len(rows), np.int8), (rows, cols)), shape=(nc, nc))
    perm = reverse_cuthill_mckee(g, symmetric_mode=True)
    new_id = np.empty(nc, np.int64)
    new_id[perm] = np.arange(nc)
    return new_id


def periodic_box(n, length=1.0, jitter=0.1, seed_jitter=0, seed_shuffle=1, reorder=True):
    """Fully periodic n^3 hex box of side ``length``.

    Node coordinates are jittered by U(-jitter*h, jitter*h) per component; the jitter is
    drawn on the periodic lattice so that images on opposite faces move identically.
    Cells are shuffled (``seed_shuffle``) and then reverse-Cuthill-McKee reordered.
    Patches x0/x1, y0/y1, z0/z1 are cyclic pairs (face m of one pairs with face m of the
    other).
    """
    h = length / n
    n1 = n + 1
    rng = np.random.default_rng(seed_jitter)
    J = rng.uniform(-jitter * h, jitter * h, size=(n, n, n, 3))   # indexed [k, j, i]
    i = np.arange(n1)
    K, Jj, I = np.meshgrid(i, i, i, indexing='ij')
    base = np.stack([I * h, Jj * h, K * h], axis=-1).astype(np.float64)
    P = base + J[K % n, Jj % n, I % n]
    P = P.reshape(-1, 3)
    pid_arr = lambda i, j, k: i + n1 * (j + n1 * k)

    # natural cell id i + n*(j + n*k) -> shuffled -> RCM
    nat = lambda i, j, k: i + n * (j + n * k)
    nc = n ** 3
    perm = np.random.default_rng(seed_shuffle).permutation(nc)   # natural -> shuffled id
    r = np.arange(n)

    def quads(axis, idx_a, j, k):
        a = np.asarray(idx_a); j = np.asarray(j); k = np.asarray(k)
        if axis == 0:
            return np.stack([pid_arr(a, j, k), pid_arr(a, j + 1, k), pid_arr(a, j + 1, k + 1), pid_arr(a, j, k + 1)], -1)
        if axis == 1:
            # here a = j-lattice index, j = i index, k = k index
            ii, jj, kk = j, a, k
            return np.stack([pid_arr(ii, jj, kk), pid_arr(ii, jj, kk + 1), pid_arr(ii + 1, jj, kk + 1), pid_arr(ii + 1, jj, kk)], -1)
        ii, jj, kk = j, k, a
        return np.stack([pid_arr(ii, jj, kk), pid_arr(ii + 1, jj, kk), pid_arr(ii + 1, jj + 1, kk), pid_arr(ii, jj + 1, kk)], -1)

    A, B, Q = [], [], []
    # x faces at lattice i = 1..n-1
    L, Jg, Kg = np.meshgrid(np.arange(1, n), r, r, indexing='ij')
    A.append(nat(L - 1, Jg, Kg)); B.append(nat(L, Jg, Kg)); Q.append(quads(0, L, Jg, Kg))
    # y faces at lattice j = 1..n-1 (i, k free)
    L, Ig, Kg = np.meshgrid(np.arange(1, n), r, r, indexing='ij')
    A.append(nat(Ig, L - 1, Kg)); B.append(nat(Ig, L, Kg)); Q.append(quads(1, L, Ig, Kg))
    # z faces at lattice k = 1..n-1 (i, j free)
    L, Ig, Jg = np.meshgrid(np.arange(1, n), r, r, indexing='ij')
    A.append(nat(Ig, Jg, L - 1)); B.append(nat(Ig, Jg, L)); Q.append(quads(2, L, Ig, Jg))
    A = np.concatenate([a.ravel() for a in A])
    B = np.concatenate([b.ravel() for b in B])
    Q = np.concatenate([q.reshape(-1, 4) for q in Q])

    # boundary faces, enumerated (second index, third index) identically on paired patches
    G2, G3 = np.meshgrid(r, r, indexing='ij')
    G2 = G2.ravel(); G3 = G3.ravel()
    zero = np.zeros_like(G2)
    last = np.full_like(G2, n)
    bdefs = []
    # x: cells (0, j, k) / (n-1, j, k)
    bdefs.append(('x0', nat(zero, G2, G3), quads(0, zero, G2, G3)[:, ::-1]))
    bdefs.append(('x1', nat(last - 1, G2, G3), quads(0, last, G2, G3)))
    bdefs.append(('y0', nat(G2, zero, G3), quads(1, zero, G2, G3)[:, ::-1]))
    bdefs.append(('y1', nat(G2, last - 1, G3), quads(1, last, G2, G3)))
    bdefs.append(('z0', nat(G2, G3, zero), quads(2, zero, G2, G3)[:, ::-1]))
    bdefs.append(('z1', nat(G2, G3, last - 1), quads(2, last, G2, G3)))

    # shuffle, then RCM over the periodic adjacency
    A = perm[A]; B = perm[B]
    bdefs = [(nm, perm[c], q) for nm, c, q in bdefs]
    if reorder:
        e_own = np.concatenate([A] + [bdefs[0][1], bdefs[2][1], bdefs[4][1]])
        e_nbr = np.concatenate([B] + [bdefs[1][1], bdefs[3][1], bdefs[5][1]])
        new_id = _rcm_permutation(nc, e_own, e_nbr)
        A = new_id[A]; B = new_id[B]
        bdefs = [(nm, new_id[c], q) for nm, c, q in bdefs]
    # The reader counts cells as max(owner)+1 (adFVM/mesh.py:521), so the last cell must own a
    # face: a cell owns its boundary faces, so give the last id to a cell on a patch.
    last = nc - 1
    bcells = np.unique(np.concatenate([c for _, c, _ in bdefs]))
    if last not in set(bcells.tolist()):
        other = int(bcells.max())
        swap = np.arange(nc)
        swap[last], swap[other] = other, last
        A = swap[A]; B = swap[B]
        bdefs = [(nm, swap[c], q) for nm, c, q in bdefs]
    pair = {'x0': 'x1', 'x1': 'x0', 'y0': 'y1', 'y1': 'y0', 'z0': 'z1', 'z1': 'z0'}
    bp = [(nm, 'cyclic', c, q, {'neighbourPatch': pair[nm]}) for nm, c, q in bdefs]
    faces, owner, neighbour, boundary = _assemble(A, B, Q, bp)
    return P, faces, owner, neighbour, boundary


def cylinder_ogrid(n_theta=256, n_r=128, diameter=1.0, far=20.0, span=None, growth=None):
    """2-D cylinder O-grid, n_theta x n_r hex cells extruded one cell in z.

    The wall (patch ``cylinder``, type ``wall``) is at r = diameter/2, the far field
    (patch ``farfield``, type ``patch``) at r = far * diameter; radial spacing is
    geometric. Front/back (``front``, ``back``) are ``empty``. The theta direction wraps,
    so the seam faces are internal faces.
    """
    r0 = 0.5 * diameter
    r1 = far * diameter
    if growth is None:
        growth = (r1 / r0) ** (1.0 / n_r)
    rs = r0 * growth ** np.arange(n_r + 1)
    rs[-1] = r1
    dz = 2 * np.pi * r0 / n_theta if span is None else span
    th = 2 * np.pi * np.arange(n_theta) / n_theta
    # points (t, j, k): t in [0, n_theta) wraps, j in [0, n_r], k in {0, 1}
    pid = lambda t, j, k: (t % n_theta) + n_theta * (j + (n_r + 1) * k)
    T, Jr = np.meshgrid(np.arange(n_theta), np.arange(n_r + 1), indexing='ij')
    P = np.zeros((n_theta * (n_r + 1) * 2, 3))
    for k in range(2):
        ids = pid(T, Jr, k).ravel()
        P[ids, 0] = (rs[Jr] * np.cos(th[T])).ravel()
        P[ids, 1] = (rs[Jr] * np.sin(th[T])).ravel()
        P[ids, 2] = k * dz
    cell = lambda t, j: (t % n_theta) + n_theta * j
    # local frame: "i" = radial (outward), "j" = theta (counter-clockwise), "k" = z.
    # radial x theta = +z, so (i, j, k) is right-handed like (x, y, z).
    def q_r(t, j):   # face at radius index j spanning theta t..t+1, normal +r
        return np.stack([pid(t, j, 0), pid(t + 1, j, 0), pid(t + 1, j, 1), pid(t, j, 1)], -1)

    def q_t(t, j):   # face at theta index t spanning r j..j+1, normal +theta
        return np.stack([pid(t, j, 0), pid(t, j, 1), pid(t, j + 1, 1), pid(t, j + 1, 0)], -1)

    def q_z(t, j, k):  # normal +z
        return np.stack([pid(t, j, k), pid(t, j + 1, k), pid(t + 1, j + 1, k), pid(t + 1, j, k)], -1)

    Tt, Jj = np.meshgrid(np.arange(n_theta), np.arange(1, n_r), indexing='ij')
    A = [cell(Tt, Jj - 1).ravel()]; B = [cell(Tt, Jj).ravel()]; Q = [q_r(Tt, Jj).reshape(-1, 4)]
    Tt, Jj = np.meshgrid(np.arange(n_theta), np.arange(n_r), indexing='ij')
    A.append(cell(Tt - 1, Jj).ravel()); B.append(cell(Tt, Jj).ravel()); Q.append(q_t(Tt, Jj).reshape(-1, 4))
    A = np.concatenate(A); B = np.concatenate(B); Q = np.concatenate(Q)
    t = np.arange(n_theta)
    wall_own = cell(t, 0); wall_q = q_r(t, 0)[:, ::-1]
    far_own = cell(t, n_r - 1); far_q = q_r(t, n_r)
    Tt, Jj = np.meshgrid(np.arange(n_theta), np.arange(n_r), indexing='ij')
    fb_own = cell(Tt, Jj).ravel()
    back_q = q_z(Tt, Jj, 0).reshape(-1, 4)[:, ::-1]
    front_q = q_z(Tt, Jj, 1).reshape(-1, 4)
    bp = [('cylinder', 'wall', wall_own, wall_q, {}),
          ('farfield', 'patch', far_own, far_q, {}),
          ('front', 'empty', fb_own, front_q, {}),
          ('back', 'empty', fb_own, back_q, {})]
    faces, owner, neighbour, boundary = _assemble(A, B, Q, bp)
    return P, faces, owner, neighbour, boundary


def channel(nx=64, ny=32, x0=0.0, x1=0.1, y0=0.0, y1=0.044, dz=None, stretch=0.0):
    """2-D channel of nx x ny hex cells extruded one cell in z, for the pressure-loss and
    heat-transfer objective of adFVM/objectives/vane.py (whose plane and wall patches it names).

    x in [x0, x1] (optionally stretched towards both ends by ``stretch``), y in [y0, y1].
    Patches (file order): ``inlet`` (x = x0) and ``outlet`` (x = x1) of type ``patch``,
    ``pressure`` (y = y0) and ``suction`` (y = y1) of type ``wall``, ``front``/``back`` ``empty``.
    """
    s = np.linspace(0.0, 1.0, nx + 1)
    if stretch:
        s = s + stretch * np.sin(2 * np.pi * s) / (2 * np.pi)
    xs = x0 + (x1 - x0) * s
    xs[0], xs[-1] = x0, x1
    ys = np.linspace(y0, y1, ny + 1)
    if dz is None:
        dz = (y1 - y0) / ny
    pid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    I, J = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing='ij')
    P = np.zeros(((nx + 1) * (ny + 1) * 2, 3))
    for k in range(2):
        ids = pid(I, J, k).ravel()
        P[ids, 0] = xs[I].ravel()
        P[ids, 1] = ys[J].ravel()
        P[ids, 2] = k * dz
    cell = lambda i, j: i + nx * j

    def qx(i, j):    # normal +x
        return np.stack([pid(i, j, 0), pid(i, j + 1, 0), pid(i, j + 1, 1), pid(i, j, 1)], -1)

    def qy(i, j):    # normal +y
        return np.stack([pid(i, j, 0), pid(i, j, 1), pid(i + 1, j, 1), pid(i + 1, j, 0)], -1)

    def qz(i, j, k):  # normal +z
        return np.stack([pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k)], -1)

    Ii, Jj = np.meshgrid(np.arange(1, nx), np.arange(ny), indexing='ij')
    A = [cell(Ii - 1, Jj).ravel()]; B = [cell(Ii, Jj).ravel()]; Q = [qx(Ii, Jj).reshape(-1, 4)]
    Ii, Jj = np.meshgrid(np.arange(nx), np.arange(1, ny), indexing='ij')
    A.append(cell(Ii, Jj - 1).ravel()); B.append(cell(Ii, Jj).ravel()); Q.append(qy(Ii, Jj).reshape(-1, 4))
    A = np.concatenate(A); B = np.concatenate(B); Q = np.concatenate(Q)
    j = np.arange(ny)
    i = np.arange(nx)
    Ii, Jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing='ij')
    bp = [('inlet', 'patch', cell(0, j), qx(0, j)[:, ::-1], {}),
          ('outlet', 'patch', cell(nx - 1, j), qx(nx, j), {}),
          ('pressure', 'wall', cell(i, 0), qy(i, 0)[:, ::-1], {}),
          ('suction', 'wall', cell(i, ny - 1), qy(i, ny), {}),
          ('front', 'empty', cell(Ii, Jj).ravel(), qz(Ii, Jj, 1).reshape(-1, 4), {}),
          ('back', 'empty', cell(Ii, Jj).ravel(), qz(Ii, Jj, 0).reshape(-1, 4)[:, ::-1], {})]
    faces, owner, neighbour, boundary = _assemble(A, B, Q, bp)
    return P, faces, owner, neighbour, boundary


def copies(meshData, K):
    """K disjoint copies of a mesh as one mesh: points, cells and faces of copy j offset by j
    times the originals' counts; the internal faces copy after copy (still sorted by owner);
    each boundary patch keeps its name and holds its faces of every copy, copy after copy
    (a cyclic pair's faces still pair up face for face). Every cell sees the same neighbours,
    faces and patch order as in the original, so the residual of each copy is computed with
    exactly the arithmetic of the single mesh."""
    points, faces, owner, neighbour, boundary = meshData
    points = np.asarray(points)
    faces = np.asarray(faces)
    owner = np.asarray(owner).reshape(-1)
    neighbour = np.asarray(neighbour).reshape(-1)
    nP, nIF, nIC = len(points), len(neighbour), int(owner.max()) + 1
    pts = np.concatenate([points] * K)
    shift = lambda f, j: np.concatenate([f[:, :1], f[:, 1:] + j * nP], axis=1)
    fl = [shift(faces[:nIF], j) for j in range(K)]
    ol = [owner[:nIF] + j * nIC for j in range(K)]
    nl = [neighbour + j * nIC for j in range(K)]
    out = {}
    start = K * nIF
    for name, b in sorted(boundary.items(), key=lambda kv: int(kv[1]['startFace'])):
        s, n = int(b['startFace']), int(b['nFaces'])
        for j in range(K):
            fl.append(shift(faces[s:s + n], j))
            ol.append(owner[s:s + n] + j * nIC)
        e = dict(b)
        e['startFace'], e['nFaces'] = start, K * n
        out[name] = e
        start += K * n
    return (pts, np.concatenate(fl).astype(np.int32), np.concatenate(ol).astype(np.int32),
            np.concatenate(nl).astype(np.int32), out)
