"""OpenFOAM case files and status.pkl (adfvm_gb300.foam), on the host.

* our writer -> our reader is lossless (bitwise) for meshes and fields of every boundary kind;
* a mesh read back builds the same geometry, bit for bit;
* the reference's own readers (mesh.py readFoam/readFoamBoundary, field.py IOField.readFoam)
  read our files to the same arrays, and our reader reads files the reference's writers
  (IOField.writeFoamField, Mesh.writeFoamBoundary) produce and the OpenFOAM-written fields of
  the reference's example cases - those run only where the reference checkout is present;
* ascii files read to the same arrays as binary; malformed files raise FoamFormatError.
"""
import os
import types

import numpy as np
import pytest

from adfvm_gb300 import cases, foam
from adfvm_gb300.mesh import Mesh

from oracle.build import REFERENCE as REF  # noqa: E402
needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, 'adFVM')), reason='reference checkout absent')


def _bc_with_arrays(case):
    return {f: {p: dict(e) for p, e in case.bc[f].items()} for f in ('U', 'T', 'p')}


def _assert_dict_equal(a, b):
    assert set(a) == set(b)
    for patch in a:
        assert set(a[patch]) == set(b[patch]), patch
        for k, v in a[patch].items():
            w = b[patch][k]
            if isinstance(v, np.ndarray):
                assert np.array_equal(np.asarray(v, np.float64).reshape(w.shape), w), (patch, k)
            else:
                assert str(v) == str(w), (patch, k)


@pytest.mark.parametrize('make', [lambda: cases.cylinder(24, 12), lambda: cases.duct(20),
                                  lambda: cases.box(6), lambda: cases.sod(50, side='symmetryPlane')])
def test_round_trip(tmp_path, make):
    case = make()
    md = case.meshData
    foam.write_mesh(str(tmp_path), md)
    bc = _bc_with_arrays(case)
    fields = {'U': case.U, 'T': case.T, 'p': case.p}
    td = str(tmp_path / '0')
    for name in ('U', 'T', 'p'):
        foam.write_field(td, name, fields[name], bc[name])
    points, faces, owner, neighbour, boundary = foam.read_mesh(str(tmp_path))
    assert np.array_equal(points, md[0]) and points.dtype == np.float64
    assert np.array_equal(faces, md[1]) and np.array_equal(owner, md[2]) and np.array_equal(neighbour, md[3])
    for patch, b in md[4].items():
        for k, v in b.items():
            assert str(boundary[patch][k]) == str(v), (patch, k)
    nIC = int(np.max(md[2])) + 1
    for name in ('U', 'T', 'p'):
        internal, b = foam.read_field(td, name, boundary, nIC)
        assert np.array_equal(internal, np.asarray(fields[name], np.float64).reshape(internal.shape))
        _assert_dict_equal(bc[name], b)


def test_read_mesh_builds_identical_geometry(tmp_path):
    case = cases.cylinder(32, 16)
    foam.write_mesh(str(tmp_path), case.meshData)
    a = Mesh.create(case.meshData)
    b = Mesh.create(foam.read_mesh(str(tmp_path)))
    for attr in ('normals', 'areas', 'volumes', 'deltas', 'weights', 'linearWeights', 'quadraticWeights',
                 'cellFaces', 'cellNeighbours', 'cellOwner', 'sortedPatches'):
        assert np.array_equal(np.asarray(getattr(a, attr)), np.asarray(getattr(b, attr))), attr


def test_time_names_and_status(tmp_path):
    assert foam.time_name(0.0) == '0' and foam.time_name(3.0) == '3'
    assert foam.time_name(1.5e-3) == '0.00150000000'
    path = str(tmp_path / 'status.pkl')
    assert foam.read_status(path) is None
    foam.write_status(path, [12, 0.0012, 1e-4, 3.25])
    assert foam.read_status(path) == [12, 0.0012, 1e-4, 3.25]
    for t in (0.0, 0.5, 2.0):
        os.makedirs(str(tmp_path / foam.time_name(t)))
    os.makedirs(str(tmp_path / 'constant'))
    assert foam.times(str(tmp_path)) == [0.0, 0.5, 2.0]


def test_ascii_reads_like_binary(tmp_path):
    case = cases.box(3)
    md = case.meshData
    d = tmp_path / 'constant' / 'polyMesh'
    os.makedirs(str(d))

    def header(cls, obj):
        return ('FoamFile\n{\n    version 2.0;\n    format ascii;\n    class %s;\n    object %s;\n}\n'
                '// comment (with brackets) 12\n' % (cls, obj))
    with open(str(d / 'points'), 'w') as f:
        f.write(header('vectorField', 'points') + '%d\n(\n' % len(md[0]))
        f.write(''.join('(%r %r %r)\n' % tuple(map(float, p)) for p in md[0]) + ')\n')
    with open(str(d / 'faces'), 'w') as f:
        f.write(header('faceList', 'faces') + '%d\n(\n' % len(md[1]))
        f.write(''.join('4(%d %d %d %d)\n' % tuple(r[1:]) for r in md[1]) + ')\n')
    for name, arr in (('owner', md[2]), ('neighbour', md[3])):
        with open(str(d / name), 'w') as f:
            f.write(header('labelList', name) + '%d\n(\n' % len(arr) + '\n'.join(str(int(x)) for x in arr) + '\n)\n')
    foam.write_boundary(str(d / 'boundary'), md[4])
    points, faces, owner, neighbour, boundary = foam.read_mesh(str(tmp_path))
    assert np.array_equal(points, md[0]) and np.array_equal(faces, md[1])
    assert np.array_equal(owner, md[2]) and np.array_equal(neighbour, md[3])
    nIC = int(np.max(md[2])) + 1
    patch = sorted(md[4])[0]
    nb = md[4][patch]['nFaces']
    U = np.random.default_rng(0).standard_normal((nIC, 3))
    with open(str(tmp_path / 'U'), 'w') as f:
        f.write(header('volVectorField', 'U') + 'dimensions [0 1 -1 0 0 0 0];\n')
        f.write('internalField nonuniform List<vector>\n%d\n(\n' % nIC)
        f.write(''.join('(%r %r %r)\n' % tuple(map(float, u)) for u in U) + ')\n;\n')
        f.write('boundaryField\n{\n')
        for p in md[4]:
            if p == patch:
                f.write('  %s\n  {\n    type fixedValue;\n    value nonuniform List<vector> %d(%s);\n  }\n' % (
                    p, nb, ' '.join('(%r %r %r)' % tuple(map(float, u)) for u in U[:nb])))
            else:
                f.write('  %s { type cyclic; }\n' % p)
        f.write('}\n')
    internal, b = foam.read_field(str(tmp_path), 'U', md[4], nIC)
    assert np.array_equal(internal, U)
    assert np.array_equal(b[patch]['value'], U[:nb]) and b[patch]['type'] == 'fixedValue'


def test_malformed_files_raise(tmp_path):
    case = cases.box(3)
    nIC = int(np.max(case.meshData[2])) + 1
    td = str(tmp_path)
    foam.write_field(td, 'T', case.T, _bc_with_arrays(case)['T'])
    raw = open(os.path.join(td, 'T'), 'rb').read()
    k = raw.index(b'internalField')
    with open(os.path.join(td, 'T1'), 'wb') as f:      # binary payload cut short
        f.write(raw[:k + 200])
    with pytest.raises(foam.FoamFormatError):
        foam.read_field(td, 'T1', case.meshData[4], nIC)
    with pytest.raises(foam.FoamFormatError):           # wrong number of cells
        foam.read_field(td, 'T', case.meshData[4], nIC + 1)
    extra = dict(case.meshData[4])
    extra['missing'] = {'type': 'patch', 'nFaces': 1, 'startFace': 0}
    with pytest.raises(foam.FoamFormatError):           # a mesh patch without an entry
        foam.read_field(td, 'T', extra, nIC)


# ------------------------------------------------------------ against the reference's own IO

@needs_ref
def test_reference_reads_our_files(tmp_path):
    from oracle import refrun
    ns = refrun.legacy_numpy()
    case = cases.cylinder(24, 12)
    md = case.meshData
    foam.write_mesh(str(tmp_path), md)
    bc = _bc_with_arrays(case)
    td = str(tmp_path / '0') + '/'
    for name, val in (('U', case.U), ('T', case.T), ('p', case.p)):
        foam.write_field(td, name, val, bc[name])
    points, faces, owner, neighbour, addressing, boundary = ns.mesh.Mesh().readFoam(str(tmp_path) + '/', 'constant')
    assert np.array_equal(points, md[0]) and np.array_equal(faces, md[1])
    assert np.array_equal(owner, md[2]) and np.array_equal(neighbour, md[3]) and addressing == []
    for patch, b in md[4].items():
        for k, v in b.items():
            assert str(boundary[patch][k]) == str(v), (patch, k)
    IO = ns.field.IOField
    nIC = int(np.max(md[2])) + 1
    IO.mesh = types.SimpleNamespace(nInternalCells=nIC, boundary=boundary)
    IO._handle, IO.time = td, 0.0
    for name, val in (('U', case.U), ('T', case.T), ('p', case.p)):
        phi = IO.readFoam(name)
        assert np.array_equal(phi.field, np.asarray(val, np.float64).reshape(phi.field.shape))
        for patch, entry in bc[name].items():
            for k, v in entry.items():
                got = phi.boundary[patch][k]
                if isinstance(v, np.ndarray):
                    # non-'value' lists stay text in the reference reader; both go through extractField
                    raw = got if isinstance(got, bytes) else got.encode()
                    arr = ns.mesh.extractField(raw, boundary[patch]['nFaces'], (v.reshape(len(v), -1).shape[1],))
                    assert np.array_equal(arr, v.reshape(arr.shape)), (name, patch, k)
                else:
                    assert got == v


@needs_ref
def test_we_read_reference_written_files(tmp_path):
    from oracle import refrun
    ns = refrun.legacy_numpy()
    case = cases.cylinder(24, 12)
    md = case.meshData
    m = Mesh.create(md)
    rng = np.random.default_rng(3)
    IO = ns.field.IOField
    IO.mesh = types.SimpleNamespace(nInternalCells=m.nInternalCells, boundary=md[4])
    td = str(tmp_path / '0.00100000000') + '/'
    for name, dims in (('U', 3), ('p', 1)):
        internal = rng.standard_normal((m.nInternalCells, dims)).view(refrun.LegacyArray)
        boundary = {}
        for patch, entry in case.bc[name].items():
            e = {k: v for k, v in entry.items() if not isinstance(v, np.ndarray)}
            if e['type'] in ('cyclic', 'empty', 'zeroGradient', 'symmetryPlane'):
                pass
            else:
                e['type'] = 'calculated'     # a value type: written as a binary list
                e['value'] = rng.standard_normal((md[4][patch]['nFaces'], dims)).view(refrun.LegacyArray)
            boundary[patch] = e
        IO(name, internal, (dims,), boundary).writeFoamField(internal, boundary, timeDir=td)
        got, gb = foam.read_field(td, name, md[4], m.nInternalCells)
        assert np.array_equal(got, np.asarray(internal))
        for patch, e in boundary.items():
            assert gb[patch]['type'] == e['type']
            if 'value' in e:
                assert np.array_equal(gb[patch]['value'], np.asarray(e['value']))
    bfile = str(tmp_path / 'boundary')
    ns.mesh.Mesh().writeFoamBoundary(bfile, {k: dict(v) for k, v in md[4].items()})
    rb = foam.read_boundary(bfile)
    for patch, b in md[4].items():
        for k, v in b.items():
            assert str(rb[patch][k]) == str(v), (patch, k)
    assert foam.time_name(0.001) == '0.00100000000' == ns.mesh.Mesh.getTimeString(0.001)


@needs_ref
@pytest.mark.parametrize('case_name,nIC', [('shockTube', 500), ('forwardStep', 7), ('sliding', 9)])
def test_reference_example_case_fields(case_name, nIC):
    """Fields OpenFOAM wrote for the reference's example cases (uniform and binary lists,
    4-space layout, quoted location) read the same as through the reference's IOField.readFoam."""
    from oracle import refrun
    ns = refrun.legacy_numpy()
    base = os.path.join(REF, 'cases', case_name)
    boundary = foam.read_boundary(os.path.join(base, 'constant', 'polyMesh', 'boundary'))
    assert boundary == ns.mesh.Mesh().readFoamBoundary(os.path.join(base, 'constant', 'polyMesh', 'boundary'))
    IO = ns.field.IOField
    IO.mesh = types.SimpleNamespace(nInternalCells=nIC, boundary=boundary)
    IO._handle, IO.time = os.path.join(base, '0') + '/', 0.0
    for name in ('U', 'T', 'p'):
        try:
            ref = IO.readFoam(name)
        except Exception:
            continue       # a uniform field given a different cell count than the file's list
        internal, b = foam.read_field(os.path.join(base, '0'), name, boundary, nIC)
        assert np.array_equal(internal, ref.field)
        for patch, entry in b.items():
            for k, v in entry.items():
                r = ref.boundary[patch][k]
                if isinstance(v, np.ndarray):
                    raw = r if isinstance(r, bytes) else r.encode()
                    assert np.array_equal(v, ns.mesh.extractField(raw, boundary[patch]['nFaces'], (v.shape[1],)))
                else:
                    assert v == r
