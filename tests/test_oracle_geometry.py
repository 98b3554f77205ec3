"""The oracle's NumPy mesh builder (oracle/geometry.py, the CPU baseline's meshes) against the
reference's own compiled cmesh (tests/golden/geometry.npz): every array bit for bit."""
import os

import numpy as np
import pytest

from adfvm_gb300 import meshgen
from oracle import geometry

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
MESHES = {'sod50': lambda: meshgen.sod_tube(50), 'box6': lambda: meshgen.periodic_box(6),
          'cyl16x8': lambda: meshgen.cylinder_ogrid(16, 8)}
FIELDS = ['normals', 'faceCentres', 'areas', 'cellCentres', 'volumes', 'neighbour', 'deltas', 'deltasUnit',
          'weights', 'linearWeights', 'quadraticWeights', 'cellFaces', 'cellOwner', 'cellNeighbours', 'volumesL',
          'volumesR']


@pytest.mark.parametrize('name', sorted(MESHES))
def test_numpy_geometry_is_the_reference_bit_for_bit(name):
    g = np.load(os.path.join(HERE, 'geometry.npz'))
    m = geometry.build_mesh(MESHES[name]())
    assert list(g[name + '/sortedPatches']) == m.sortedPatches
    for f in FIELDS:
        ref = g['%s/%s' % (name, f)]
        got = np.asarray(getattr(m, f))
        assert got.size == ref.size, f
        assert np.array_equal(got.reshape(ref.shape), ref), (f, float(np.max(np.abs(got.reshape(ref.shape) - ref))))
    for f in ('nCells', 'nGhostCells'):
        assert int(g['%s/%s' % (name, f)]) == getattr(m, f)
