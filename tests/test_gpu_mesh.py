"""The device mesh builder (afvm_mesh_build_device) against the host builder, which is pinned
bit for bit to the reference's compiled cmesh (tests/test_capi.py): every geometry and
connectivity array must be bitwise identical, and malformed meshes must be refused with the
host builder's status codes. The device cell renumbering (afvm_mesh_reorder_device) against
its oracle (oracle/c/reorder_oracle.c, pinned to SciPy's reverse Cuthill-McKee in
tests/test_reorder.py): every output array bitwise."""
import numpy as np
import pytest

from adfvm_gb300 import _lib as L
from adfvm_gb300 import meshgen
from adfvm_gb300.mesh import Mesh, reorder
from oracle import c_ref

pytestmark = pytest.mark.gpu

ARRAYS = ['normals', 'faceCentres', 'areas', 'cellCentres', 'volumes', 'neighbour', 'deltas', 'deltasUnit',
          'weights', 'linearWeights', 'quadraticWeights', 'cellFaces', 'cellOwner', 'cellNeighbours',
          'cellNeighboursMatOp', 'volumesL', 'volumesR']


@pytest.mark.parametrize('make', [lambda: meshgen.sod_tube(100), lambda: meshgen.sod_tube(50, side_type='symmetryPlane'),
                                  lambda: meshgen.periodic_box(12), lambda: meshgen.periodic_box(7, reorder=False),
                                  lambda: meshgen.cylinder_ogrid(64, 32)])
def test_device_build_is_bitwise_the_host_build(make):
    md = make()
    a = Mesh.create(md)
    b = Mesh.create(md, device=0)
    assert a.nLocalCells == b.nLocalCells and list(a.sortedPatches) == list(b.sortedPatches)
    for k in ARRAYS:
        x, y = np.asarray(getattr(a, k)), np.asarray(getattr(b, k))
        assert x.shape == y.shape and x.dtype == y.dtype, k
        assert x.tobytes() == y.tobytes(), k


def test_device_build_refuses_malformed_meshes():
    P, F, O, N, B = meshgen.sod_tube(10)
    F2 = F.copy()
    F2[3, 0] = 3                       # a triangle
    with pytest.raises(L.AfvmError) as e:
        Mesh.create((P, F2, O, N, B), device=0)
    assert e.value.status == L.AFVM_ERR_UNSUPPORTED
    N2 = N.copy()
    N2[2] = O[2]                       # neighbour not above its owner
    with pytest.raises(L.AfvmError) as e:
        Mesh.create((P, F, O, N2, B), device=0)
    assert e.value.status == L.AFVM_ERR_BAD_ARG
    F3 = F.copy()
    F3[5, 2] = len(P) + 7              # a point id past the end
    with pytest.raises(L.AfvmError) as e:
        Mesh.create((P, F3, O, N, B), device=0)
    assert e.value.status == L.AFVM_ERR_BAD_ARG


@pytest.mark.parametrize('make', [lambda: meshgen.periodic_box(16, reorder=False), lambda: meshgen.periodic_box(5, reorder=False),
                                  lambda: meshgen.periodic_box(2, reorder=False), lambda: meshgen.cylinder_ogrid(64, 32),
                                  lambda: meshgen.sod_tube(200), lambda: meshgen.channel(32, 12, stretch=0.3),
                                  lambda: meshgen.periodic_box(48, reorder=False)])
def test_device_reorder_is_bitwise_the_oracle(make):
    md = make()
    ref, cn0, fo0, bw0 = c_ref.mesh_reorder(md)
    out, cn1, fo1, bw1 = reorder(md, device=0)
    assert np.array_equal(cn0, cn1)
    assert np.array_equal(fo0, fo1)
    assert bw0 == bw1
    for k in (1, 2, 3):
        assert np.array_equal(np.asarray(ref[k]), np.asarray(out[k])), k
    # the reordered mesh builds on the device bitwise as on the host
    a, b = Mesh.create(out), Mesh.create(out, device=0)
    for k in ARRAYS:
        assert np.asarray(getattr(a, k)).tobytes() == np.asarray(getattr(b, k)).tobytes(), k


def test_device_reorder_refuses_bad_indices():
    P, F, O, N, B = meshgen.sod_tube(10)
    O2 = O.copy()
    O2[4] = -1
    with pytest.raises(L.AfvmError) as e:
        reorder((P, F, O2, N, B), device=0)
    assert e.value.status == L.AFVM_ERR_BAD_ARG
    O3 = O.copy()
    O3[-1] = 12                       # cells 10 and 11 without faces
    with pytest.raises(L.AfvmError) as e:
        reorder((P, F, O3, N, B), device=0)
    assert e.value.status == L.AFVM_ERR_BAD_ARG
    N2 = N.copy()
    N2[2] = O[2]                      # a face between a cell and itself
    with pytest.raises(L.AfvmError) as e:
        reorder((P, F, O, N2, B), device=0)
    assert e.value.status == L.AFVM_ERR_BAD_ARG
