"""C ABI: the library loads and exports every declared symbol; the host mesh build is
bit-identical to the reference's own mesh builder; calls fail with status codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from adfvm_gb300 import _lib as L
from adfvm_gb300 import meshgen
from adfvm_gb300.mesh import Mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden', 'geometry.npz')


def declared_functions():
    src = open(os.path.join(ROOT, 'include', 'afvm.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(afvm_[a-z0-9_]+)\s*\(', src)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(L.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(L.SIGNATURES), set(names) - set(L.SIGNATURES)


@pytest.mark.parametrize('name,fn', [('sod50', lambda: meshgen.sod_tube(50)),
                                     ('box6', lambda: meshgen.periodic_box(6)),
                                     ('cyl16x8', lambda: meshgen.cylinder_ogrid(16, 8))])
def test_mesh_build_bit_identical_to_reference(name, fn):
    g = np.load(GOLDEN)
    md = fn()
    m = Mesh.create(md)
    assert list(m.sortedPatches) == list(g[name + '/sortedPatches'])
    for a in ['normals', 'faceCentres', 'areas', 'cellCentres', 'volumes', 'neighbour', 'deltas', 'deltasUnit',
              'weights', 'linearWeights', 'quadraticWeights', 'cellFaces', 'cellOwner', 'cellNeighbours',
              'volumesL', 'volumesR']:
        ref = g[name + '/' + a]
        x = np.asarray(getattr(m, a))
        assert ref.size == x.size, a
        assert np.array_equal(ref.reshape(-1), x.reshape(-1)), a       # bit-exact
    for a in ['nLocalCells', 'nCells', 'nGhostCells', 'nLocalFaces', 'nRemoteCells']:
        assert int(g[name + '/' + a]) == getattr(m, a), a


def test_mesh_build_rejects_bad_input():
    P, F, O, N, B = meshgen.sod_tube(10)
    F = F.copy()
    F[3, 0] = 3          # a triangle
    with pytest.raises(L.AfvmError) as e:
        Mesh.create((P, F, O, N, B))
    assert e.value.status == L.AFVM_ERR_UNSUPPORTED
    P, F, O, N, B = meshgen.sod_tube(10)
    N = N.copy()
    N[0] = O[0]          # neighbour must exceed owner
    with pytest.raises(L.AfvmError) as e:
        Mesh.create((P, F, O, N, B))
    assert e.value.status == L.AFVM_ERR_BAD_ARG


def test_null_arguments_return_status():
    lib = L.lib()
    assert lib.afvm_mesh_build(None, None) == L.AFVM_ERR_BAD_ARG
    assert lib.afvm_ctx_destroy(None) == L.AFVM_OK
    assert lib.afvm_primal_step(None, None, None, None, 0.0, None, None, None, None, None, None, None, None,
                                None) == L.AFVM_ERR_BAD_ARG
    assert lib.afvm_boundary_values(None, None, None, None, None, None) == L.AFVM_ERR_BAD_ARG
    out = C.c_void_p()
    assert lib.afvm_ctx_create(None, None, None, 0, 0, C.byref(out)) == L.AFVM_ERR_BAD_ARG


def test_host_copy_argument_checks():
    """afvm_copy_to_device / afvm_copy_to_host reject bad element sizes, negative counts, null
    pointers and negative devices before any CUDA call; an empty copy is a no-op."""
    lib = L.lib()
    a = np.zeros(4)
    hp = C.c_void_p(a.ctypes.data)
    for fn in (lib.afvm_copy_to_device, lib.afvm_copy_to_host):
        assert fn(0, None, 8, None, 8, 0, None) == L.AFVM_OK
        assert fn(0, None, 8, hp, 8, 4, None) == L.AFVM_ERR_BAD_ARG
        assert fn(0, hp, 8, None, 8, 4, None) == L.AFVM_ERR_BAD_ARG
        assert fn(0, hp, 2, hp, 8, 4, None) == L.AFVM_ERR_BAD_ARG
        assert fn(0, hp, 8, hp, 16, 4, None) == L.AFVM_ERR_BAD_ARG
        assert fn(0, hp, 8, hp, 8, -1, None) == L.AFVM_ERR_BAD_ARG
        assert fn(-1, hp, 8, hp, 8, 4, None) == L.AFVM_ERR_BAD_ARG
