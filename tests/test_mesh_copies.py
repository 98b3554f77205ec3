"""K disjoint copies of a mesh as one mesh (meshgen.copies / cases.copies, the meshes of the
server's batched slots): each copy's step is bitwise the single mesh's, in the oracle."""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from oracle import torch_ref


@pytest.mark.parametrize('make', [lambda: cases.box(6, objective='kinetic_energy'), lambda: cases.cylinder(16, 8)])
def test_each_copy_steps_like_the_single_mesh(make):
    base = make()
    m1 = base.build_mesh()
    c3 = cases.copies(base, 3)
    m3 = c3.mesh
    n = m1.nInternalCells
    assert m3.nInternalCells == 3 * n and m3.nFaces == 3 * m1.nFaces and m3.sortedPatches == m1.sortedPatches
    assert np.array_equal(np.asarray(m3.volumes).reshape(3, -1), np.tile(np.asarray(m1.volumes).reshape(1, -1), (3, 1)))
    x1 = [torch.as_tensor(a) for a in cases.conservative(base)]
    x3 = [torch.as_tensor(a) for a in cases.conservative(c3)]
    r1 = torch_ref.Problem(m1, base.bc, base.config, base.objective).step(*x1, base.dt)
    r3 = torch_ref.Problem(m3, c3.bc, c3.config, c3.objective).step(*x3, base.dt)
    for i in range(3):
        for j in range(3):
            assert torch.equal(r3[i][j * n:(j + 1) * n], r1[i]), (i, j)
    assert abs(float(r3[4]) - 3 * float(r1[4])) <= 1e-13 * abs(3 * float(r1[4]))
